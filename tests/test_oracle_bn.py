"""Known answers of the Green-tensor kernel B_pq(k) of the elastic force
(elastic_calculate_BN, source_beta_to_omega/src/elastic.c:460-605), as the
oracle computes it (orc_compute_bn) and the device kernel reproduces it
(through the elastic force, pinned to the reference's felas): symmetric in
p and q, even in k, a function of the direction of k only, the k = 0 entry
taken at the direction (0, 1, 0) as the reference sets it, and, for an
isotropic medium with purely dilatational eigenstrains, the same value in
every direction (a dilatational misfit's elastic energy does not depend on
the inclusion's shape)."""
import ctypes

import numpy as np
import pytest

import cases


def bn(oracle_lib, big_n, voigt, eps):
    out = np.zeros(16 * big_n ** 3)
    lib = oracle_lib._lib()
    lib.orc_compute_bn(ctypes.c_int(big_n), oracle_lib._ptr(np.ascontiguousarray(voigt.reshape(-1), dtype=np.float64)),
                       oracle_lib._ptr(np.ascontiguousarray(np.stack(eps).reshape(-1), dtype=np.float64)),
                       oracle_lib._ptr(out))
    return out.reshape(4, 4, big_n, big_n, big_n)  # [p][q][z][y][x]


@pytest.fixture(scope="module")
def cubic(oracle_lib):
    N = 12
    return N, bn(oracle_lib, N, cases.cubic_voigt(1.0, 0.6, 0.4), cases.rhombohedral_eigenstrains())


def test_symmetric_in_p_and_q(cubic):
    _, B = cubic
    np.testing.assert_allclose(B, B.transpose(1, 0, 2, 3, 4), rtol=0, atol=1e-15)


def test_even_in_k(cubic):
    N, B = cubic
    neg = (-np.arange(N)) % N  # index of -k on the periodic grid
    flipped = B[:, :, neg][:, :, :, neg][:, :, :, :, neg]
    # away from the Nyquist planes (k_i = -N/2 has no +N/2 partner on the grid)
    keep = np.arange(N) != N // 2
    sel = np.ix_(keep, keep, keep)
    np.testing.assert_allclose(B[:, :][(slice(None), slice(None)) + sel], flipped[(slice(None), slice(None)) + sel],
                               rtol=0, atol=1e-15)


def test_depends_on_the_direction_only(cubic):
    N, B = cubic
    # k and 2k (both inside the grid's frequency range) share a direction
    for k in [(1, 0, 0), (0, 1, 1), (1, 2, -1), (-2, 1, 1), (1, -1, 2)]:
        a = tuple(v % N for v in k)
        b = tuple((2 * v) % N for v in k)
        np.testing.assert_allclose(B[:, :, a[2], a[1], a[0]], B[:, :, b[2], b[1], b[0]], rtol=1e-13, atol=1e-16)


def test_zero_frequency_uses_direction_y(cubic):
    N, B = cubic
    np.testing.assert_allclose(B[:, :, 0, 0, 0], B[:, :, 0, 1, 0], rtol=1e-13, atol=1e-16)
    assert not np.allclose(B[:, :, 0, 0, 0], B[:, :, 0, 0, 1])  # a cubic medium is not isotropic


def test_isotropic_dilatation_is_direction_independent(oracle_lib):
    N = 8
    lam, mu = 0.6, 0.5
    iso = cases.cubic_voigt(lam + 2 * mu, lam, mu)
    eps = [np.eye(3) * e for e in (0.01, -0.02, 0.005, 0.03)]
    B = bn(oracle_lib, N, iso, eps).reshape(4, 4, -1)
    np.testing.assert_allclose(B, B[:, :, :1].repeat(N ** 3, axis=2), rtol=1e-12, atol=1e-16)
    # and it is the closed form 4 mu (3 lam + 2 mu) / (lam + 2 mu) e_p e_q of a dilatational misfit
    e = np.array([0.01, -0.02, 0.005, 0.03])
    want = 4 * mu * (3 * lam + 2 * mu) / (lam + 2 * mu) * np.outer(e, e)
    np.testing.assert_allclose(B[:, :, 0], want, rtol=1e-12, atol=1e-16)
