"""Mixed-precision form (SCLET_MIXED): split-BF16 tcgen05 eigenbasis products
with FP32 accumulation, FP32 stencils and FFT, FP64 diagnostics.  Checked
against the plain FP64 form of the same library (itself checked against the
reference and the oracle): rel L2 <= 1e-5 per field, energy within 1e-6
relative."""
import dataclasses
import tempfile

import numpy as np
import pytest

import bench
import cases

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def params_for(sg, case):
    with tempfile.TemporaryDirectory() as td:
        cases.write_case(case, td, eigen=False, fields=False)
        return sg.read_case(td, case.suffix)


@pytest.mark.parametrize("big_n", [32, 64, 192, 252])
def test_tc_mode_product_accuracy(big_n, sclet_lib):
    """One tensor-core product against FP64 einsum of the FP32-rounded input.
    n = 36, 68 take one a'-tile of 128 rows, n = 196 two, n = 256 exactly two
    full ones."""
    sg = sclet_lib
    case = cases.Case(big_n=big_n, nac=1, nch=0, elastic=0, steps=1, suffix="mp")
    s = sg.Solver(params_for(sg, case), sg.MIXED)
    n = s.n
    a = np.random.default_rng(1).standard_normal((n, n, n))
    d, v, vi = cases.eigen_variant(n, 3)
    a32 = a.astype(np.float32).astype(np.float64)
    for inverse, m in ((False, vi), (True, v)):
        got = s.mode_product(a, inverse)
        want = np.einsum("pa,cba->pcb", m, a32)
        assert rel(got, want) <= 2e-7, (n, inverse, rel(got, want))
    s.sync()
    s.close()


def _mixed_vs_fp64(sg, case, steps, every=1):
    """Both forms from the same state for `steps` steps: per-field relative L2
    over the owned cells at the end, and the energy-curve error max |dE| /
    max |E| over the diagnostics taken every `every` steps."""
    p = params_for(sg, case)
    u0 = bench.block_fields(case)
    out = {}
    for prec in (sg.FP64, sg.MIXED):
        s = sg.Solver(p, prec)
        s.set_fields(u0)
        energies = []
        done = 0
        while done < steps:
            k = min(every, steps - done)
            s.step(k)
            done += k
            energies.append(s.check_soln()[0, 3])
        out[prec] = (s.get_fields(), np.array(energies))
        s.sync()
        s.close()
    (u64, e64), (u32, e32) = out[sg.FP64], out[sg.MIXED]
    own = (slice(2, -2),) * 3
    errs = [rel(u32[f][own], u64[f][own]) for f in range(u64.shape[0])]
    eerr = float(np.max(np.abs(e32 - e64)) / np.max(np.abs(e64)))
    return errs, eerr


def test_mixed_matches_fp64_beta_omega_64(sclet_lib):
    """64^3 beta->omega physics (4 order parameters, elasticity), 200 steps."""
    case = cases.Case(big_n=64, steps=200, seed=77, suffix="m64")
    errs, eerr = _mixed_vs_fp64(sclet_lib, case, 200)
    assert max(errs) <= 1e-5, errs
    assert eerr <= 1e-6, eerr


def test_mixed_matches_fp64_variable_mobility(sclet_lib):
    """Variable-mobility CH coupled to four order parameters (64^3, the
    mobility following the first order parameter over [0, 0.9], elastic,
    anisotropic), 200 steps: per field <= 1e-5, energy curve within 1e-6."""
    case = bench.workload(64, seed=5)
    case = dataclasses.replace(case, variable_mobility=1, eta_range=(0.0, 0.9), suffix="vm64")
    errs, eerr = _mixed_vs_fp64(sclet_lib, case, 200, every=50)
    assert max(errs) <= 1e-5, errs
    assert eerr <= 1e-6, eerr


def test_mixed_matches_fp64_beta_alpha_192_2000_steps(sclet_lib):
    """The 192^3 coupled CH + AC workload (one conserved concentration, four
    order parameters, c-eta coupling, anisotropic, elastic, dt 0.005) for its
    2000 steps: per field <= 1e-5, energy curve within 1e-6."""
    case = bench.workload(192, seed=9)
    errs, eerr = _mixed_vs_fp64(sclet_lib, case, 2000, every=100)
    assert max(errs) <= 1e-5, errs
    assert eerr <= 1e-6, eerr


def test_mixed_matches_fp64_beta_alpha_512(sclet_lib):
    """The 512^3 workload of the benchmark (block 516^3, 5 fields, about 30 GB
    for the FP64 form), 20 steps."""
    case = bench.workload(512, seed=9)
    errs, eerr = _mixed_vs_fp64(sclet_lib, case, 20, every=5)
    assert max(errs) <= 1e-5, errs
    assert eerr <= 1e-6, eerr


@pytest.mark.parametrize("precision_name", ["FP64", "MIXED"])
def test_step_diagnostics_match_check_soln(precision_name, sclet_lib):
    """Diagnostics queued inside sclet_step (as the reference's loop runs
    check_soln_new every pass) equal a separate sclet_check_soln."""
    sg = sclet_lib
    case = bench.workload(32, seed=11)
    s = sg.Solver(params_for(sg, case), getattr(sg, precision_name))
    s.set_fields(bench.block_fields(case))
    s.set_step_diagnostics(1)
    s.step(3)
    queued = s.last_diagnostics()
    s.set_step_diagnostics(-1)
    np.testing.assert_array_equal(queued, s.check_soln(1))
    s.close()


@pytest.mark.parametrize("big_n", [24, 32, 48, 80, 96, 160, 512])
def test_fp32_elastic_force_matches_fp64(big_n, sclet_lib):
    """FP32 elastic force (pack, three line-FFT passes each way, contraction)
    against the FP64 form on the same state.  N = 16 N1 takes the two-pass
    register transforms (N1 = 32 at 512, eight lines per CTA); 24 the generic
    Stockham stages."""
    sg = sclet_lib
    case = bench.workload(big_n, seed=13)
    p = params_for(sg, case)
    u0 = bench.block_fields(case)
    u0[:case.nac] *= 50.0  # order parameters of order 0.5
    out = {}
    for prec in (sg.FP64, sg.MIXED):
        s = sg.Solver(p, prec)
        s.set_fields(u0)
        s.transfer()
        s.elastic()
        out[prec] = s.get_felas()
        s.close()
    for m in range(case.nac):
        err = rel(out[sg.MIXED][m], out[sg.FP64][m])
        assert err <= 2e-6, (big_n, m, err)


@pytest.mark.parametrize("precision_name", ["FP64", "MIXED"])
def test_pipelined_field_transfers(precision_name, sclet_lib):
    """set/get_fields(_async) of all fields against the per-field accessors,
    and a pipelined loop (inputs of step k+1 queued while step k runs)
    against the same calls made synchronously on a second context with the
    same history (the elastic ghost shell carries state between calls)."""
    sg = sclet_lib
    prec = getattr(sg, precision_name)
    case = bench.workload(24, seed=21)
    p = params_for(sg, case)
    u0 = bench.block_fields(case)
    s = sg.Solver(p, prec)
    s.set_fields(u0)
    per_field = np.zeros_like(u0)
    for f in range(s.F):
        k, m = s._kind(f)
        assert s.L.sclet_get_field(s.h, k, m, sg._dp(per_field[f])) == 0
    np.testing.assert_array_equal(s.get_fields(), per_field)
    want = []
    for k in range(3):
        s.set_fields(u0)
        s.step(k + 1)
        want.append(s.get_fields())
    s.close()
    s = sg.Solver(p, prec)
    s.set_fields(u0)
    pin_in = sg.PinnedArray(u0.shape)
    pin_in.array[...] = u0
    outs = [sg.PinnedArray(u0.shape) for _ in range(3)]
    s.set_fields_async(pin_in.array)
    for k in range(3):
        s.step(k + 1)
        s.get_fields_async(outs[k].array)
        if k < 2:
            s.set_fields_async(pin_in.array)
    s.sync()
    for k in range(3):
        np.testing.assert_array_equal(outs[k].array, want[k])
    for a in outs + [pin_in]:
        a.free()
    s.close()


def test_mixed_conserves_ch_mass_like_fp64(sclet_lib):
    """The conserved field's mass (volume integral of check_soln_new) of the
    mixed form tracks the FP64 form's through the FP64 mass correction.  What
    remains is the FP32 rounding of the stored state (c - c0 of about 0.02:
    ulp 2e-9 per cell, a random sum over 32^3 cells of about 2e-11 of the
    mass), so the bar is 1e-10."""
    sg = sclet_lib
    case = bench.workload(32, seed=17)
    p = params_for(sg, case)
    u0 = bench.block_fields(case)
    vols = {}
    for prec in (sg.FP64, sg.MIXED):
        s = sg.Solver(p, prec)
        s.set_fields(u0)
        s.step(40)
        vols[prec] = s.check_soln(1)[case.nac, 2]
        s.close()
    assert abs(vols[sg.MIXED] - vols[sg.FP64]) <= 1e-10 * abs(vols[sg.FP64]), vols


def test_mixed_matches_fp64_reference_formula(sclet_lib):
    """The reference's own physics plugin (formula.c: LE = 1, KE = 42, the
    2-3-4 polynomial) through both forms: 32^3, 4 order parameters,
    elasticity, 100 steps."""
    case = cases.Case(big_n=32, steps=100, seed=78, dt=0.002, physics=1, suffix="f234")
    errs, eerr = _mixed_vs_fp64(sclet_lib, case, 100)
    assert max(errs) <= 1e-5, errs
    assert eerr <= 1e-6, eerr


def test_bounded_wait_gives_up_and_is_reported(sclet_lib):
    """A tensor-core launch whose barriers receive nothing (no copy is issued)
    gives up after its poll limit instead of hanging: the status is
    SCLET_ERR_TIMEOUT, reported once, and the context steps on unchanged."""
    sg = sclet_lib
    case = bench.workload(32, seed=23)
    p = params_for(sg, case)
    u0 = bench.block_fields(case)
    s = sg.Solver(p, sg.MIXED)
    s.set_fields(u0)
    s.step(1)
    rc = s.L.sclet_selftest_wait_timeout(s.h)
    assert rc == 6, (rc, s.L.sclet_last_error(s.h))  # SCLET_ERR_TIMEOUT
    assert b"bounded" in s.L.sclet_last_error(s.h)
    assert s.L.sclet_sync(s.h) == 0
    s.step(3)
    ref = sg.Solver(p, sg.MIXED)
    ref.set_fields(u0)
    ref.step(4)
    np.testing.assert_array_equal(s.get_fields(), ref.get_fields())
    s.close()
    ref.close()
