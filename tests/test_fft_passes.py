"""The two-pass line FFT of the elastic force (fft2::lines_kernel in
energy-stability_gb300/csrc/k_fft.cu), restated in numpy with the kernel's
index maps: pass A transforms x[t + N2 n1] over n1 for each t (N1 points, in
registers), applies W_N^(t k1) and stores to the exchange table; pass B
transforms the table over t for each k1 (N2 points) and writes X[k1 + N1 k2].
The small DFTs are composite (A-point DFTs over stride-B subsequences, W_R^(b ka),
B-point DFTs) down to radices 2, 3, 4, 5.  Checked against numpy's FFT for
every supported N = 16 N1, both signs."""
import numpy as np
import pytest


def _first(r):
    if r % 4 == 0 and r > 4:
        return 4
    if r % 2 == 0 and r > 2:
        return 2
    if r % 3 == 0 and r > 3:
        return 3
    return r


def _w(r, m, sign):
    w = np.exp(-2j * np.pi * m / r)
    return np.conj(w) if sign > 0 else w


def _dft(v, sign):
    r = len(v)
    if r in (1, 2, 3, 4, 5):
        return np.array([sum(v[n] * _w(r, n * k % r, sign) for n in range(r)) for k in range(r)])
    a = _first(r)
    b = r // a
    y = np.zeros((b, a), complex)
    for bi in range(b):
        u = _dft(np.array([v[bi + b * ai] for ai in range(a)]), sign)
        for ka in range(a):
            y[bi, ka] = u[ka] * (_w(r, bi * ka, sign) if bi * ka else 1)
    out = np.zeros(r, complex)
    for ka in range(a):
        w = _dft(y[:, ka].copy(), sign)
        for kb in range(b):
            out[ka + a * kb] = w[kb]
    return out


def _line(x, n1, n2, sign):
    n = n1 * n2
    tab = np.zeros((n1, n2), complex)
    for t in range(n2):
        v = _dft(np.array([x[t + n2 * k] for k in range(n1)]), sign)
        for k1 in range(n1):
            tab[k1, t] = v[k1] * (_w(n, t * k1, sign) if t * k1 else 1)
    out = np.zeros(n, complex)
    for k1 in range(n1):
        v = _dft(tab[k1].copy(), sign)
        for k2 in range(n2):
            out[k1 + n1 * k2] = v[k2]
    return out


@pytest.mark.parametrize("n1", [2, 3, 4, 5, 6, 8, 10, 12, 16, 32])
def test_two_pass_line_transform(n1):
    rng = np.random.default_rng(n1)
    x = rng.standard_normal(16 * n1) + 1j * rng.standard_normal(16 * n1)
    np.testing.assert_allclose(_line(x, n1, 16, -1), np.fft.fft(x), rtol=0, atol=1e-9)
    np.testing.assert_allclose(_line(x, n1, 16, +1), np.fft.ifft(x) * x.size, rtol=0, atol=1e-9)
