"""The batched ensemble on the GPU: runs side by side in one context
(sclet_create_runs) against the same runs each in a context of its own
(bit for bit: every stage computes each run exactly as the single-run path),
CUDA-graph steps against ordinary steps, the autotuner's choice against the
default launch shapes, and an ensemble of several block sizes against each
context stepped alone."""
import numpy as np
import pytest

import bench

pytestmark = pytest.mark.gpu


def _runs(sg, edge, seeds, a2s):
    case = bench.ensemble_case(edge, seeds[0], a2s[0])
    p = bench.case_params(sg, case)
    u0 = np.concatenate([bench.block_fields(bench.ensemble_case(edge, s, a)) for s, a in zip(seeds, a2s)])
    return p, u0


def test_runs_side_by_side_match_single_runs(sclet_lib):
    sg = sclet_lib
    seeds, a2s = [3, 4, 5], [-1.1, -0.9, -1.0]
    for edge in (32, 48):
        p, u0 = _runs(sg, edge, seeds, a2s)
        s = sg.Solver(p, sg.MIXED, runs=3, krun=np.array(a2s))
        s.set_fields(u0)
        s.step(5)
        got, diag = s.get_fields(), s.check_soln(1)
        s.close()
        F = 4
        for r, (seed, a2) in enumerate(zip(seeds, a2s)):
            q = bench.case_params(sg, bench.ensemble_case(edge, seed, a2))
            one = sg.Solver(q, sg.MIXED)
            one.set_fields(u0[r * F:(r + 1) * F])
            one.step(5)
            np.testing.assert_array_equal(got[r * F:(r + 1) * F], one.get_fields(), err_msg=f"edge {edge} run {r}")
            np.testing.assert_array_equal(diag[r * F:(r + 1) * F], one.check_soln(1))
            one.close()


def test_graph_steps_match_ordinary_steps(sclet_lib):
    sg = sclet_lib
    p, u0 = _runs(sg, 32, [7, 8], [-1.0, -1.2])
    out = []
    for graph in (False, True):
        s = sg.Solver(p, sg.MIXED, runs=2, krun=np.array([-1.0, -1.2]))
        s.set_fields(u0)
        if graph:
            s.graph_step(6)
        else:
            s.step(6)
        out.append(s.get_fields())
        s.close()
    np.testing.assert_array_equal(out[0], out[1])


def test_tuned_shapes_give_the_same_results(sclet_lib):
    sg = sclet_lib
    p, u0 = _runs(sg, 48, [9, 10], [-0.8, -1.0])
    out = []
    for tune in (False, True):
        s = sg.Solver(p, sg.MIXED, runs=2, krun=np.array([-0.8, -1.0]))
        s.set_fields(u0)
        s.step(1)
        if tune:
            zc, ctas = s.tune(2)
            assert zc in (8, 16, 32, 64) and 0 <= ctas <= 1000
        s.step(4)
        out.append(s.get_fields())
        s.close()
    np.testing.assert_array_equal(out[0], out[1])


def test_ensemble_of_sizes_matches_each_context(sclet_lib):
    sg = sclet_lib
    groups = [(32, [1, 2], [-1.0, -0.9]), (48, [3], [-1.1]), (64, [4, 5], [-1.2, -0.8])]
    made = []
    for edge, seeds, a2s in groups:
        p, u0 = _runs(sg, edge, seeds, a2s)
        made.append((p, u0, a2s))
    solvers = []
    for p, u0, a2s in made:
        s = sg.Solver(p, sg.MIXED, runs=len(a2s), krun=np.array(a2s))
        s.set_fields(u0)
        solvers.append(s)
    ens = sg.Ensemble(solvers)
    ens.step(5)
    ens.sync()
    got = [s.get_fields() for s in solvers]
    ens.close()
    for s in solvers:
        s.close()
    for (p, u0, a2s), g in zip(made, got):
        s = sg.Solver(p, sg.MIXED, runs=len(a2s), krun=np.array(a2s))
        s.set_fields(u0)
        s.step(5)
        np.testing.assert_array_equal(g, s.get_fields())
        s.close()
