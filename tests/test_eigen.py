"""Eigen-data generator (oracle/cases.py) against the reference's shipped
n = 260 files (summarised in tests/golden/eigen260.npz by make_golden.py) and
the defining identities."""
import os

import numpy as np
import pytest

import cases

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "eigen260.npz")


@pytest.mark.parametrize("variant", [0, 1, 2, 3])
@pytest.mark.parametrize("n", [12, 36, 68])
def test_decomposition_identities(n, variant):
    d, v, vi = cases.eigen_variant(n, variant)
    t = cases.second_difference(n, variant)
    assert np.abs(v @ np.diag(d) @ vi - t).max() < 1e-12
    assert np.abs(v @ vi - np.eye(n)).max() < 1e-12
    assert np.all(np.diff(d) >= -1e-12)


@pytest.mark.parametrize("variant", [0, 1, 2, 3])
def test_matches_shipped_260_files(variant):
    g = np.load(GOLD)
    d, v, vi = cases.eigen_variant(260, variant)
    # same spectrum (the shipped files are not sorted for variants 0-2)
    np.testing.assert_allclose(np.sort(d), np.sort(g[f"d{variant}"]), rtol=0, atol=1e-12)
    # same second-difference operator: stencil rows the files reproduce
    np.testing.assert_allclose(cases.second_difference(260, variant)[[0, 1, -2, -1]], g[f"T{variant}"], atol=1e-12)
    # same eigenvectors up to sign: compare |V| column sums per eigenvalue
    order = np.argsort(g[f"d{variant}"])
    np.testing.assert_allclose(np.abs(v).sum(axis=0), g[f"colabs{variant}"][order], rtol=1e-9)
