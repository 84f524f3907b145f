"""The CPU FP64 oracle of the corrector network (oracle/cnn_oracle.py): its
analytic gradient against central finite differences of its own loss, its
periodic convolution against a direct loop, and BF16 rounding against torch's."""
import numpy as np
import pytest

import cnn_oracle as co


def test_convolution_matches_direct_sum():
    rng = np.random.default_rng(0)
    N = 4
    x = rng.standard_normal((1, co.CH, N, N, N))
    W = rng.standard_normal((co.TAPS, co.CH, co.CH))
    b = rng.standard_normal(co.CH)
    y = co.conv(x, W, b)
    z0, y0, x0 = 3, 0, 2
    want = b.copy()
    for t, (dz, dy, dx) in enumerate(co.OFFS):
        want += W[t] @ x[0, :, (z0 + dz) % N, (y0 + dy) % N, (x0 + dx) % N]
    np.testing.assert_allclose(y[0, :, z0, y0, x0], want, rtol=1e-12)


def test_adjoint_is_the_transpose():
    rng = np.random.default_rng(1)
    N = 4
    x = rng.standard_normal((2, co.CH, N, N, N))
    g = rng.standard_normal((2, co.CH, N, N, N))
    W = rng.standard_normal((co.TAPS, co.CH, co.CH))
    lhs = np.sum(co.conv(x, W, None) * g)
    rhs = np.sum(x * co.conv_adjoint(g, W))
    assert abs(lhs - rhs) <= 1e-10 * abs(lhs)


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(2)
    N, B = 4, 1
    p = co.random_params(3)
    inp = rng.standard_normal((B, co.NIN, N, N, N)) * 0.5
    tgt = rng.standard_normal((B, co.NOUT, N, N, N)) * 0.1
    scale = 0.3
    loss, g = co.loss_and_grad(p, inp, tgt, scale)
    assert loss == pytest.approx(co.loss_only(p, inp, tgt, scale), rel=1e-14)
    W, b = co.unpack(p)
    # a sample of parameters from every layer (weights of used channels and biases)
    idx = []
    for layer in range(co.LAYERS):
        cin = co.NIN if layer == 0 else co.CH
        cout = co.NOUT if layer == co.LAYERS - 1 else co.CH
        for _ in range(3):
            t, o, c = rng.integers(co.TAPS), rng.integers(cout), rng.integers(cin)
            idx.append(layer * co.WPER + (t * co.CH + o) * co.CH + c)
        idx.append(co.LAYERS * co.WPER + layer * co.CH + rng.integers(cout))
    eps = 1e-6
    for i in idx:
        q = p.copy()
        q[i] += eps
        lp = co.loss_only(q, inp, tgt, scale)
        q[i] -= 2 * eps
        lm = co.loss_only(q, inp, tgt, scale)
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-6 * max(abs(g[i]), 1e-3 * np.abs(g).max()), (i, fd, g[i])
    # unused channels carry no gradient
    gW, gb = co.unpack(g)
    assert not gW[0, :, :, co.NIN:].any()
    assert not gW[-1, :, co.NOUT:, :].any() and not gb[-1, co.NOUT:].any()


def test_bf16_rounding_matches_torch():
    torch = pytest.importorskip("torch")
    a = np.random.default_rng(4).standard_normal(10000) * 10.0 ** np.random.default_rng(5).integers(-8, 8, 10000)
    want = torch.from_numpy(a.astype(np.float32)).to(torch.bfloat16).to(torch.float64).numpy()
    np.testing.assert_array_equal(co.bf16(a), want)
