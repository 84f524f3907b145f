"""The fixed-point BF16 slice format of the mixed-precision products,
restated in numpy (float32 arithmetic, round to nearest even):

* a line x with power-of-two scale S >= max|x| splits into four slices
  d_p = rint(r_p 2^b), r_{p+1} = r_p 2^b - d_p, each an integer that BF16
  holds exactly; their sum rebuilds x to within S 2^(-4b - 1);
* rint of |y| < 2^22 equals the 1.5 * 2^23 shift (the converter warps'
  rounding), and the BF16 bits of an integer-valued float of magnitude
  <= 256 are its upper 16 bits (their packing);
* weight classes 0 and 1 stay exact integers: K * 2^(2b) <= 2^24 for the
  contraction lengths the slice width is chosen for."""
import numpy as np

B = 7


def slices(x):
    s = np.float32(2.0 ** np.ceil(np.log2(np.max(np.abs(x))))) if np.any(x) else np.float32(1.0)
    step = np.float32(2.0 ** B)
    r = (x / s).astype(np.float32)
    out = []
    for _ in range(4):
        y = (r * step).astype(np.float32)
        d = np.rint(y).astype(np.float32)
        out.append(d)
        r = (y - d).astype(np.float32)
    return s, out


def test_slices_are_exact_small_integers_and_rebuild_the_line():
    rng = np.random.default_rng(3)
    x = (rng.standard_normal(200) * 10.0 ** rng.uniform(-3, 3)).astype(np.float32)
    s, d = slices(x)
    assert np.abs(d[0]).max() <= 2 ** B and all(np.abs(p).max() <= 2 ** (B - 1) for p in d[1:])
    for p in d:
        assert np.array_equal(p, np.round(p))
    rebuilt = sum(p.astype(np.float64) * 2.0 ** (-B * (k + 1)) for k, p in enumerate(d)) * float(s)
    assert np.max(np.abs(rebuilt - x.astype(np.float64))) <= float(s) * 2.0 ** (-4 * B - 1)


def test_shift_rounding_and_bf16_packing():
    rng = np.random.default_rng(5)
    y = rng.uniform(-129.0, 129.0, 100000).astype(np.float32)
    y = np.concatenate([y, np.float32([0.5, 1.5, 2.5, -0.5, -2.5, 127.5, -128.5])])
    m = np.float32(12582912.0)
    shifted = ((y + m).astype(np.float32) - m).astype(np.float32)
    assert np.array_equal(shifted, np.rint(y))
    d = np.rint(y).astype(np.float32)
    upper = (d.view(np.uint32) >> 16).astype(np.uint16)
    back = (upper.astype(np.uint32) << 16).view(np.float32)
    assert np.array_equal(back, d)


def test_exact_classes_bound():
    for n in (28, 36, 68, 196, 516, 1028):
        k = 32 * ((n + 31) // 32)
        bits = 7 if k <= 1024 else 6
        assert k * 2 ** (2 * bits) <= 2 ** 24, (n, k, bits)
