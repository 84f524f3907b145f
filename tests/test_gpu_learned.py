"""Learned coarse-step corrector on the GPU: the tcgen05 convolution network
(sclet_net_*) against the CPU FP64 oracle (oracle/cnn_oracle.py) -- forward
pass and every parameter's gradient --, training on solver-generated pairs
with the gain over the coarse step without the corrector on held-out runs,
and the plain-ETD judge of sclet_learned_step (energy, deviation, fallback)."""
import numpy as np
import pytest

import cases
import cnn_oracle as co

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.ravel(a - b)) / max(np.linalg.norm(np.ravel(b)), 1e-300))


@pytest.fixture(scope="module")
def learned(sclet_lib):
    import learned
    return learned


def _torch():
    return pytest.importorskip("torch")


@pytest.mark.parametrize("N,B", [(16, 2), (12, 1), (40, 1)])
def test_forward_matches_oracle(N, B, learned):
    torch = _torch()
    rng = np.random.default_rng(N)
    p = co.random_params(7 + N)
    scale = 0.5
    inp = (rng.random((B, co.NIN, N, N, N)) - 0.5).astype(np.float32)
    net = learned.Net(seed=1, out_scale=scale)
    net.set_params(p.astype(np.float32))
    x = torch.from_numpy(inp).cuda()
    y = torch.empty((B, co.NOUT, N, N, N), dtype=torch.float32, device="cuda")
    net.forward(x, y)
    want, _ = co.forward(p.astype(np.float32).astype(np.float64), inp.astype(np.float64), scale, bf16_round=True)
    got = y.cpu().numpy()
    assert rel(got, want) <= 1e-2, rel(got, want)
    net.close()


def test_conv_tilings_agree(learned, sclet_lib):
    """The convolution kernel's two tilings (one input run per stencil plane
    and channel chunk, as small grids use; one per stencil row, as grids of
    N >= 146 use) give the same forward pass bit for bit, at 24^3 and at a
    grid where the planes' slot counts are not multiples of 8."""
    torch = _torch()
    L = sclet_lib.lib()
    p = co.random_params(9).astype(np.float32)
    for N, B in ((24, 2), (13, 1)):
        rng = np.random.default_rng(N)
        inp = torch.from_numpy((rng.random((B, co.NIN, N, N, N)) - 0.5).astype(np.float32)).cuda()
        outs = []
        try:
            for runs in (1, 3):
                assert L.sclet_net_set_conv_runs(runs) in (0, 1, 3)
                net = learned.Net(seed=1, out_scale=0.5)
                net.set_params(p)
                y = torch.empty((B, co.NOUT, N, N, N), dtype=torch.float32, device="cuda")
                net.forward(inp, y)
                outs.append(y.cpu().numpy())
                net.close()
        finally:
            L.sclet_net_set_conv_runs(0)
        np.testing.assert_array_equal(outs[0], outs[1], err_msg=f"N={N}")
        assert np.isfinite(outs[0]).all() and np.abs(outs[0]).max() > 0
    assert L.sclet_net_set_conv_runs(2) == -1


def test_gradients_match_oracle(learned):
    torch = _torch()
    rng = np.random.default_rng(3)
    N, B = 8, 2
    p = co.random_params(11).astype(np.float32)
    scale = 0.5
    inp = co.bf16(rng.random((B, co.NIN, N, N, N)) - 0.5).astype(np.float32)
    tgt = (0.2 * rng.standard_normal((B, co.NOUT, N, N, N))).astype(np.float32)
    net = learned.Net(seed=1, out_scale=scale)
    net.set_params(p)
    loss, g = net.gradient(torch.from_numpy(inp).cuda(), torch.from_numpy(tgt).cuda())
    # the oracle with the GPU's BF16 storage emulated (weights, activations,
    # activation gradients), exact sums.  What remains is where FP32 and FP64
    # sums round to neighbouring BF16 values: the oracle itself moves as much
    # when its sums are perturbed by 1e-6 relative before rounding (about
    # 0.3% on every layer, 2.5% on the first layer's weights, whose gradient
    # sums products with the random-signed input).
    want_loss, want = co.loss_and_grad(p.astype(np.float64), inp.astype(np.float64), tgt.astype(np.float64), scale,
                                       bf16_round=True)
    assert loss == pytest.approx(want_loss, rel=1e-3)
    gW, gb = co.unpack(g.astype(np.float64))
    wW, wb = co.unpack(want)
    for layer in range(co.LAYERS):
        assert rel(gW[layer], wW[layer]) <= (5e-2 if layer == 0 else 1e-2), (layer, rel(gW[layer], wW[layer]))
        assert rel(gb[layer], wb[layer]) <= 1e-2, (layer, rel(gb[layer], wb[layer]))
    net.close()


def _omega(seed, N=32):
    return cases.Case(big_n=N, nac=4, nch=0, dt=0.01, steps=1000, epn2=0.5, elastic=1, seed=seed, suffix="lc")


def test_training_gains_over_coarse_step(learned):
    """Pairs from the solver (32^3 beta->omega, the coarse step 8 fine steps of
    dt 0.01); after training, the corrected coarse step is closer to the fine
    steps than the coarse step alone on runs it has not seen."""
    torch = _torch()
    samples = [0, 40, 120, 240, 400]
    X, Y = learned.make_pairs(_omega, range(12), samples, 8)
    Xh, Yh = learned.make_pairs(_omega, range(100, 103), samples, 8)
    net = learned.Net(seed=5, out_scale=1.0)
    losses = learned.train(net, X, Y, iters=600, batch=4, lr=1e-3)
    assert np.mean(losses[-40:]) < 0.5 * np.mean(losses[:10]), (losses[:10], losses[-40:])
    err = learned.relative_errors(net, Xh, Yh)
    # 1.0 is the coarse step without the corrector
    assert np.mean(err) <= 0.7, err
    net.close()


def _solvers(learned, sg, seed, N=24):
    case = _omega(seed, N)
    fine = sg.Solver(learned.case_params(case), sg.MIXED)
    coarse = sg.Solver(learned.case_params(case, dt=case.dt * 8), sg.MIXED)
    u0 = learned.block_fields(case)
    return case, fine, coarse, u0


def test_failed_steps_fall_back_to_fine_steps(learned, sclet_lib):
    """A corrector that raises the energy fails the energy check on every
    step; each step is replaced by eight fine steps, so the run equals the
    fine run itself."""
    sg = sclet_lib
    torch = _torch()
    case, fine, coarse, u0 = _solvers(learned, sg, 5)
    net = learned.Net(seed=2, out_scale=5.0)
    net.set_params(co.random_params(4, scale=3.0).astype(np.float32))
    coarse.set_fields(u0)
    fine.set_fields(u0)
    st = learned.learned_steps(coarse, fine, net, 8, 6, check_every=0)
    assert st["steps"] == 6 and st["fallbacks"] == 6 and st["energy_fail"] == 6, st
    ref = sg.Solver(learned.case_params(case), sg.MIXED)
    ref.set_fields(u0)
    ref.step(48)
    own = (slice(None),) + (slice(2, -2),) * 3
    np.testing.assert_array_equal(coarse.get_fields()[own], ref.get_fields()[own])
    for s in (ref, fine, coarse):
        s.close()
    net.close()
    del torch


def test_deviation_bound_is_checked(learned, sclet_lib):
    """With a bound below the coarse step's own error, every checked step
    fails the deviation check and falls back; with no corrector and no bound
    the coarse steps are the plain coarse ETD run."""
    sg = sclet_lib
    case, fine, coarse, u0 = _solvers(learned, sg, 6)
    coarse.set_fields(u0)
    st = learned.learned_steps(coarse, fine, None, 8, 4, check_every=2, deviation_bound=1e-12)
    assert st["deviation_checks"] == 2 and st["deviation_fail"] == 2 and st["fallbacks"] == 2, st
    assert st["max_deviation"] > 1e-6
    for s in (fine, coarse):
        s.close()
    # fresh contexts: the elastic scratch carries state between steps
    case, fine, coarse, u0 = _solvers(learned, sg, 6)
    plain = sg.Solver(learned.case_params(case, dt=0.08), sg.MIXED)
    plain.set_fields(u0)
    plain.step(3)
    coarse.set_fields(u0)
    st = learned.learned_steps(coarse, fine, None, 8, 3, check_every=0, energy_tol=1.0)
    assert st["fallbacks"] == 0, st
    own = (slice(None),) + (slice(2, -2),) * 3
    np.testing.assert_array_equal(coarse.get_fields()[own], plain.get_fields()[own])
    for s in (plain, fine, coarse):
        s.close()
