"""C-ABI library: loads without a GPU, exports every entry point declared in
include/sclet_gb300.h, and its host-side input handling matches the
reference's formats and the oracle's case writer."""
import ctypes
import os
import re

import numpy as np

import case_defs
import cases

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    with open(os.path.join(ROOT, "include", "sclet_gb300.h")) as fp:
        text = fp.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sclet_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(sclet_lib):
    L = sclet_lib.lib()
    syms = declared_symbols()
    assert len(syms) >= 30
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing
    # and the Python bindings cover the whole header
    assert set(syms) == set(sclet_lib.SIGNATURES), set(syms) ^ set(sclet_lib.SIGNATURES)


def test_read_case_matches_writer(sclet_lib, tmp_path):
    c = case_defs.write("full", str(tmp_path))
    p = sclet_lib.read_case(str(tmp_path), "full")
    assert (p.nx, p.ny, p.nz) == (c.n,) * 3
    assert (p.px, p.py, p.pz, p.nghost, p.periodic) == (1, 1, 1, 2, 1)
    assert (p.nac, p.nch, p.etd2, p.elastic, p.anisotropic) == (c.nac, c.nch, c.etd2, c.elastic, c.anisotropic)
    assert p.dt == c.dt and p.epn2 == c.epn2
    assert abs(p.t_total - (c.steps - 0.5) * c.dt) < 1e-15
    assert (p.kkx, p.kky, p.kkz) == tuple(c.kk)
    assert p.xmax == c.domain and p.restart == 1 and p.restart_dir == b"./restart/"
    assert p.elastic_scale == c.elastic_scale
    np.testing.assert_array_equal(np.array(p.voigt).reshape(6, 6), c.voigt)
    np.testing.assert_array_equal(np.array(p.eigenstrain).reshape(4, 3, 3), np.array(c.eigenstrains))
    np.testing.assert_array_equal(np.array(p.lambda_file).reshape(4, 3, 3), np.array(c.lambdas))
    np.testing.assert_array_equal(np.array(p.landau), np.array(c.landau))


def test_missing_input_is_an_error_not_an_exit(sclet_lib, tmp_path):
    p = sclet_lib.Params()
    rc = sclet_lib.lib().sclet_read_case(str(tmp_path).encode(), b"nothing", ctypes.byref(p))
    assert rc == 2  # SCLET_ERR_IO


def test_seeded_values_match_case_writer(sclet_lib):
    L = sclet_lib.lib()
    ref = cases.seeded_field(1234, 2, 8, -0.01, 0.01).reshape(-1)
    got = np.array([L.sclet_seeded_value(1234, 2, i, -0.01, 0.01) for i in range(ref.size)])
    np.testing.assert_array_equal(got, ref)


def test_restart_text_roundtrip(sclet_lib, tmp_path):
    L = sclet_lib.lib()
    n = 12
    blk = np.random.default_rng(3).standard_normal((n, n, n))
    path = str(tmp_path / "f.txt").encode()
    assert L.sclet_write_restart(path, n, blk.ctypes.data_as(ctypes.POINTER(ctypes.c_double))) == 0
    out = np.zeros_like(blk)
    assert L.sclet_read_restart(path, n, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))) == 0
    np.testing.assert_array_equal(out[2:-2, 2:-2, 2:-2], blk[2:-2, 2:-2, 2:-2])
    assert not out[:2].any() and not out[-2:].any()


def test_closed_form_eigen_matches_case_files(sclet_lib, tmp_path):
    """The library's closed-form DST basis equals the eigen files the oracle
    writes for the reference (variant 3), to rounding."""
    L = sclet_lib.lib()
    n = 36
    cases.write_eigen_files(str(tmp_path), n, variants=(3,))
    d, v, vi = (np.zeros(n), np.zeros((n, n)), np.zeros((n, n)))
    dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    L.sclet_eigen_dirichlet(n, dp(d), dp(v), dp(vi))
    fd, fv, fvi = (np.zeros(n), np.zeros((n, n)), np.zeros((n, n)))
    assert L.sclet_read_eigen(str(tmp_path).encode(), n, 3, dp(fd), dp(fv), dp(fvi)) == 0
    np.testing.assert_allclose(d, fd, rtol=0, atol=1e-14)
    np.testing.assert_allclose(v, fv, rtol=0, atol=1e-14)
    np.testing.assert_allclose(vi, fvi, rtol=0, atol=1e-14)


def test_physics_plugin_selection(sclet_lib, tmp_path):
    """physics_input.txt names the plugin; a plugin that cannot run the case
    (the reference's formula.c has no concentration physics) or an unknown id
    is refused before any device work, with a message instead of an exit."""
    L = sclet_lib.lib()
    c = case_defs.write("formula234", str(tmp_path))
    p = sclet_lib.read_case(str(tmp_path), "formula234")
    assert p.physics == sclet_lib.PHYSICS_FORMULA234
    p.nch = 1
    h = ctypes.c_void_p()
    assert L.sclet_create(ctypes.byref(p), sclet_lib.FP64, 0, ctypes.byref(h)) == 4  # SCLET_ERR_UNSUPPORTED
    assert b"concentration" in L.sclet_last_error(None)
    p.nch = 0
    p.physics = 7
    assert L.sclet_create(ctypes.byref(p), sclet_lib.FP64, 0, ctypes.byref(h)) == 4
    assert b"physics plugin" in L.sclet_last_error(None)
    (tmp_path / "physics_input.txt").write_text("nosuchplugin\n")
    p2 = sclet_lib.Params()
    assert L.sclet_read_case(str(tmp_path).encode(), b"formula234", ctypes.byref(p2)) == 1  # SCLET_ERR_ARG
    assert c.physics == 1


def test_variable_mobility_needs_its_fields(sclet_lib, tmp_path):
    """VariableMobility = 1 takes the mobility of the one conserved field from
    the first order parameter (update_M_C, mobility.c:860-922): without a
    Cahn-Hilliard field or an order parameter the context is refused before
    any device work; a value other than 0 or 1 is an argument error."""
    L = sclet_lib.lib()
    case = cases.Case(big_n=8, nac=1, nch=1, steps=1, variable_mobility=1, suffix="vm")
    cases.write_case(case, str(tmp_path))
    p = sclet_lib.read_case(str(tmp_path), "vm")
    assert p.variable_mobility == 1
    h = ctypes.c_void_p()
    p.nch = 0
    assert L.sclet_create(ctypes.byref(p), sclet_lib.FP64, 0, ctypes.byref(h)) == 4  # SCLET_ERR_UNSUPPORTED
    assert b"Cahn-Hilliard" in L.sclet_last_error(None)
    p.nch, p.nac = 1, 0
    p.elastic = 0
    assert L.sclet_create(ctypes.byref(p), sclet_lib.FP64, 0, ctypes.byref(h)) == 4
    p.nac, p.variable_mobility = 1, 2
    assert L.sclet_create(ctypes.byref(p), sclet_lib.FP64, 0, ctypes.byref(h)) == 1  # SCLET_ERR_ARG
