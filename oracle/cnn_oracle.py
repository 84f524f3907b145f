"""CPU FP64 oracle of the learned corrector network (TEST INFRASTRUCTURE ONLY:
the product never imports it).  The reference has no such network; this is
the definition the CUDA kernels of energy-stability_gb300/csrc/k_conv*.cu and
sclet_net.cu are checked against:

  x (8 channels, zero padded to 32), periodic 3x3x3 convolutions of 32
  channels, out[co](c) = sum_t sum_ci W[t][co][ci] x[ci](c + off(t)) + b[co]
  with off(t) = (dz, dy, dx), t = 9 (dz + 1) + 3 (dy + 1) + (dx + 1);
  h0 = relu(conv0 x); r_k = relu(conv_{2k+1} h_k); h_{k+1} = h_k + conv_{2k+2} r_k
  (k < 4); y = conv_9(h_4)[:4] * out_scale.
  loss = mean over every value of (y - target)^2.

Arrays are [batch][channel][z][y][x].  `bf16=True` rounds what the GPU stores
in BF16 (inputs, weights, every activation; biases and the output stay FP32)
to the nearest BF16 value, so that a forward pass can be compared with the
GPU's closely; gradients are those of the unrounded FP64 function.
"""
import numpy as np

CH, TAPS, BLOCKS, NIN, NOUT = 32, 27, 4, 8, 4
LAYERS = 2 + 2 * BLOCKS
WPER = TAPS * CH * CH
NPARAM = LAYERS * (WPER + CH)
OFFS = [(t // 9 - 1, (t // 3) % 3 - 1, t % 3 - 1) for t in range(TAPS)]


def bf16(a):
    """Round to the nearest BF16 value (ties to even), as float64."""
    b = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params):
    p = np.asarray(params, dtype=np.float64)
    W = p[: LAYERS * WPER].reshape(LAYERS, TAPS, CH, CH)
    b = p[LAYERS * WPER:].reshape(LAYERS, CH)
    return W, b


def pack(W, b):
    return np.concatenate([W.reshape(-1), b.reshape(-1)])


def shift(x, off):
    """x(c + off) on the periodic grid (axes -3, -2, -1 = z, y, x)."""
    dz, dy, dx = off
    return np.roll(x, shift=(-dz, -dy, -dx), axis=(-3, -2, -1))


def conv(x, W, b):
    """x [B][CH][N][N][N], W [TAPS][co][ci], b [co] (or None)."""
    out = np.zeros_like(x)
    for t, off in enumerate(OFFS):
        out += np.einsum("oc,bc...->bo...", W[t], shift(x, off))
    if b is not None:
        out += b[None, :, None, None, None]
    return out


def conv_adjoint(g, W):
    """The adjoint of conv (without bias) applied to g."""
    out = np.zeros_like(g)
    for t, off in enumerate(OFFS):
        out += shift(np.einsum("oc,bo...->bc...", W[t], g), tuple(-o for o in off))
    return out


def wgrad(x, g):
    """dW[t][co][ci] = sum over cells and batch of g[co](c) x[ci](c + off(t))."""
    return np.stack([np.einsum("bozyx,bczyx->oc", g, shift(x, off)) for off in OFFS])


def forward(params, inp, out_scale, bf16_round=False):
    W, b = unpack(params)
    rnd = bf16 if bf16_round else (lambda a: a)
    if bf16_round:
        W = bf16(W)
    B, cin = inp.shape[:2]
    x = np.zeros((B, CH) + inp.shape[2:])
    x[:, :cin] = inp
    x = rnd(x)
    cache = {"x": x, "W": W, "b": b}
    h = rnd(np.maximum(conv(x, W[0], b[0]), 0.0))
    cache["h0"] = h
    for k in range(BLOCKS):
        r = rnd(np.maximum(conv(h, W[2 * k + 1], b[2 * k + 1]), 0.0))
        h = rnd(h + conv(r, W[2 * k + 2], b[2 * k + 2]))
        cache[f"r{k}"] = r
        cache[f"h{k + 1}"] = h
    y = conv(h, W[LAYERS - 1], b[LAYERS - 1])[:, :NOUT] * out_scale
    return y, cache


def loss_and_grad(params, inp, target, out_scale, bf16_round=False):
    """FP64 loss and the analytic gradient of every parameter (layout of
    sclet_net_get_params).  bf16_round=True also rounds, as the GPU stores
    them, the activations of the forward pass and the activation gradients
    of the backward pass (the output gradient, and each adjoint
    convolution's result) to BF16; the sums stay exact."""
    rnd = bf16 if bf16_round else (lambda a: a)
    y, c = forward(params, inp, out_scale, bf16_round=bf16_round)
    W = c["W"]
    count = y.size
    r = y.astype(np.float32).astype(np.float64) - target if bf16_round else y - target
    loss = float(np.sum(r * r) / count)
    gW = np.zeros_like(W)
    gb = np.zeros((LAYERS, CH))
    gy = np.zeros((y.shape[0], CH) + y.shape[2:])
    gy[:, :NOUT] = rnd(r * np.float32(2.0 / count * out_scale))
    L = LAYERS - 1
    h = c[f"h{BLOCKS}"]
    gW[L] = wgrad(h, gy)
    gb[L] = gy.sum(axis=(0, 2, 3, 4))
    gh = rnd(conv_adjoint(gy, W[L]))
    for k in range(BLOCKS - 1, -1, -1):
        l1, l2 = 2 * k + 1, 2 * k + 2
        rk, hk = c[f"r{k}"], c[f"h{k}"]
        gW[l2] = wgrad(rk, gh)
        gb[l2] = gh.sum(axis=(0, 2, 3, 4))
        ga = rnd(conv_adjoint(gh, W[l2]) * (rk > 0))
        gW[l1] = wgrad(hk, ga)
        gb[l1] = ga.sum(axis=(0, 2, 3, 4))
        gh = rnd(gh + conv_adjoint(ga, W[l1]))
    ga = gh * (c["h0"] > 0)
    gW[0] = wgrad(c["x"], ga)
    gb[0] = ga.sum(axis=(0, 2, 3, 4))
    return loss, pack(gW, gb)


def loss_only(params, inp, target, out_scale):
    y, _ = forward(params, inp, out_scale)
    return float(np.sum((y - target) ** 2) / y.size)


def random_params(seed, scale=1.0):
    """Random parameters of the network's shape (unused channels zero), the
    output layer included, for tests."""
    rng = np.random.default_rng(seed)
    W = np.zeros((LAYERS, TAPS, CH, CH))
    for l in range(LAYERS):
        cin = NIN if l == 0 else CH
        cout = NOUT if l == LAYERS - 1 else CH
        W[l, :, :cout, :cin] = rng.standard_normal((TAPS, cout, cin)) * scale * np.sqrt(2.0 / (TAPS * cin))
    b = np.zeros((LAYERS, CH))
    b[:, :] = 0.05 * rng.standard_normal((LAYERS, CH)) * scale
    b[LAYERS - 1, NOUT:] = 0.0
    return pack(W, b)
