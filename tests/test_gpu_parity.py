"""CUDA path (libsclet_gb300.so through the C ABI) against the reference's
golden fixtures and the oracle.  Plain FP64 form; tolerances: exact for the
halo gather, 1e-12 relative L2 for one right-hand-side evaluation, 1e-10
relative L2 per field for multi-step runs (the spec bar)."""
import os

import numpy as np
import pytest

import case_defs
import cases

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def solver_for(sclet_lib, case_dir, suffix, precision=0):
    p = sclet_lib.read_case(case_dir, suffix)
    s = sclet_lib.Solver(p, precision)
    n = p.nx
    d, v, vi = (np.loadtxt(os.path.join(case_dir, f"{k}3{n}.dat")) for k in ("d", "v", "vi"))
    s.set_eigen(d, v, vi)  # the same eigen files the reference read
    s.load_restart_dir(case_dir)
    return s


@pytest.mark.parametrize("name", list(case_defs.load_defs()))
def test_first_evaluation_matches_reference(name, tmp_path, sclet_lib):
    c = case_defs.write(name, str(tmp_path))
    g = np.load(os.path.join(case_defs.HERE, f"{name}.npz"))
    s = solver_for(sclet_lib, str(tmp_path), name)
    s.transfer()
    np.testing.assert_array_equal(s.get_fields(), g["filled0"])
    s.elastic()
    if c.elastic:
        felas = s.get_felas()
        for m in range(c.nac):
            assert rel(felas[m], g["felas0"][m]) <= 1e-12, m
    s.calc_rhs(1)
    rhs = s.get_rhs(1)
    for f in range(s.F):
        assert rel(rhs[f], g["rhs0"][f]) <= 1e-12, f
    s.close()


@pytest.mark.parametrize("name", list(case_defs.load_defs()))
def test_steps_match_reference(name, tmp_path, sclet_lib):
    c = case_defs.write(name, str(tmp_path))
    g = np.load(os.path.join(case_defs.HERE, f"{name}.npz"))
    s = solver_for(sclet_lib, str(tmp_path), name)
    s.set_energy_tensors(np.zeros((4, 3, 3)) if not c.anisotropic else
                         np.array([np.diag(c.kk) - l for l in c.lambdas]))
    cols = 4 if c.nac in (0, 4) else 3
    for k in range(c.steps):
        d = s.check_soln(form=0)[:, :cols]
        np.testing.assert_allclose(d, g["diag"][:, k, :cols], rtol=1e-10, atol=1e-13)
        s.step(1)
    u = s.get_fields()
    for f in range(s.F):
        assert rel(u[f], g["final"][f]) <= 1e-10, f
    s.close()


def test_mode_product_matches_einsum(tmp_path, sclet_lib):
    c = case_defs.write("radix5", str(tmp_path))
    s = solver_for(sclet_lib, str(tmp_path), "radix5")
    n = c.n
    a = np.random.default_rng(5).standard_normal((n, n, n))
    vi = np.loadtxt(os.path.join(str(tmp_path), f"vi3{n}.dat"))
    v = np.loadtxt(os.path.join(str(tmp_path), f"v3{n}.dat"))
    for inverse, m in ((False, vi), (True, v)):
        got = s.mode_product(a, inverse)
        # out[a', c, b] = sum_a M[a', a] in[c, b, a]
        want = np.einsum("pa,cba->pcb", m, a)
        assert rel(got, want) <= 1e-14
    s.close()


def _oracle_vs_gpu(tmp_path, sclet_lib, oracle_lib, case, steps):
    d = str(tmp_path)
    cases.write_case(case, d)
    s = solver_for(sclet_lib, d, case.suffix)
    o = oracle_lib.Oracle(oracle_lib.load_case(d, case.suffix))
    o.step(steps)
    s.step(steps)
    u = s.get_fields()
    errs = [rel(u[f], o.u[f]) for f in range(s.F)]
    eg = s.check_soln(form=1)
    eo = o.check_soln()
    s.close()
    return errs, eg, eo


def test_all_options_match_oracle(tmp_path, sclet_lib, oracle_lib):
    rng = np.random.default_rng(7)
    case = cases.Case(big_n=32, nac=4, nch=1, etd2=1, anisotropic=1, kk=(0.5, 0.5, 0.5),
                      lambdas=[np.diag([0.5, 0.5, 0.3]) + 0.05 * rng.standard_normal((3, 3)) for _ in range(4)],
                      dt=0.005, epn2=1.0, steps=20, seed=21, suffix="opts")
    errs, eg, eo = _oracle_vs_gpu(tmp_path, sclet_lib, oracle_lib, case, 20)
    assert max(errs) <= 1e-10, errs
    np.testing.assert_allclose(eg, eo, rtol=1e-10, atol=1e-13)


def test_variable_mobility_matches_oracle(tmp_path, sclet_lib, oracle_lib):
    """Variable-mobility Cahn-Hilliard (VariableMobility = 1, the mobility of
    the first concentration following the first order parameter, which
    ranges over [0, 0.9] here) with anisotropy, elasticity and ETD2, 32^3 for
    20 steps against the oracle (itself pinned to the reference's own
    update_M_C / ch_calc_FU_VariableMobility by the golden case varmob)."""
    rng = np.random.default_rng(8)
    case = cases.Case(big_n=32, nac=4, nch=1, etd2=1, anisotropic=1, kk=(0.5, 0.5, 0.5),
                      lambdas=[np.diag([0.5, 0.5, 0.3]) + 0.05 * rng.standard_normal((3, 3)) for _ in range(4)],
                      dt=0.005, epn2=1.0, steps=20, seed=22, eta_range=(0.0, 0.9), variable_mobility=1,
                      suffix="vmob")
    errs, eg, eo = _oracle_vs_gpu(tmp_path, sclet_lib, oracle_lib, case, 20)
    assert max(errs) <= 1e-10, errs
    np.testing.assert_allclose(eg, eo, rtol=1e-10, atol=1e-13)


def test_beta_omega_64_cubed_1000_steps(tmp_path, sclet_lib):
    """The beta->omega plain-ETD workload (64^3, 4 order parameters, Landau
    2-4-6, cubic elasticity, dt = 0.01) for 1000 steps against the
    reference's own code (fixture tests/golden/beta_omega_64_1000.npz, made by
    tests/golden/make_long_golden.py from oracle/_ref): per-field relative L2
    <= 1e-10 after 1000 steps, the check_soln_new record of every pass within
    1e-10, and the free energy of the run (the plugin's, energy form 1 with
    the dynamics' gradient tensors diag(kk)) non-increasing from pass to
    pass.  The reference's own energy column is its hard-coded 2-3-4
    polynomial without gradient terms here, which this physics does not
    decrease, so it is compared but not tested for monotonicity."""
    import make_long_golden
    case = make_long_golden.long_case()
    g = np.load(os.path.join(case_defs.HERE, "beta_omega_64_1000.npz"))
    d = str(tmp_path)
    cases.write_case(case, d)
    s = solver_for(sclet_lib, d, case.suffix)
    zero, dyn = np.zeros((4, 3, 3)), np.array([np.diag(case.kk)] * 4)
    ours, free = [], []
    for k in range(case.steps):
        s.set_energy_tensors(zero)  # the reference's energy without ANISOTROPIC
        ours.append(s.check_soln(form=0))
        s.set_energy_tensors(dyn)
        free.append(s.check_soln(form=1)[0, 3])
        s.step(1)
    ours = np.stack(ours, axis=1)  # [field][pass][max, min, vol, energy]
    u = s.get_fields()
    s.close()
    own = (slice(2, -2),) * 3
    errs = [rel(u[f][own], g["final"][f]) for f in range(case.nac)]
    assert max(errs) <= 1e-10, errs
    np.testing.assert_allclose(ours, g["diag"], rtol=1e-10, atol=1e-13)
    free = np.array(free)
    assert np.all(np.diff(free) <= 1e-12 * np.abs(free[:-1])), "free energy increased"


@pytest.mark.parametrize("precision_name", ["FP64", "MIXED"])
def test_nan_in_the_state_is_reported(precision_name, tmp_path, sclet_lib):
    """A NaN planted in one owned cell on the host: the diagnostics report
    SCLET_ERR_NONFINITE (an error code, no exit and no device fault), before
    and after a step that spreads it, and the device stays usable: a new
    context on it steps and checks normally."""
    sg = sclet_lib
    case = cases.Case(big_n=24, nac=4, nch=1, steps=2, seed=3, suffix="nan")
    d = str(tmp_path)
    cases.write_case(case, d)
    p = sg.read_case(d, case.suffix)
    s = sg.Solver(p, getattr(sg, precision_name))
    u0 = np.zeros((s.F, case.n, case.n, case.n))
    u0[:, 2:-2, 2:-2, 2:-2] = 0.01
    u0[s.nac:] += 0.5
    bad = u0.copy()
    bad[1, 7, 8, 9] = np.nan
    s.set_fields(bad)
    for _ in range(2):
        with pytest.raises(sg.ScletError, match=r"\(7\)"):
            s.check_soln(1)
        s.step(1)
    s.close()
    s = sg.Solver(p, getattr(sg, precision_name))
    s.set_fields(u0)
    s.step(1)
    assert np.isfinite(s.check_soln(1)).all()
    s.close()
