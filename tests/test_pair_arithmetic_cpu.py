"""The FP32-pair arithmetic of the block kernels (csrc/pairs.cuh), restated with numpy float32
operations, against exact (FP64 / rational) results: the split is exact in its high word and
within 2^-48 overall, one multiply-add is within 2^-45 of the product, and renormalised sums
of a few hundred products stay within ~1e-14 of the sum of magnitudes.  This pins the numerical
method on the CPU; the GPU tests compare the kernels themselves with FP64."""

import numpy as np

f32 = np.float32


def split(a: float):
    """hi = the top 24 significant bits of a (truncated), lo = the rest rounded to float32."""
    a = float(a)
    if a == 0.0:
        return f32(0.0), f32(0.0)
    m, e = np.frexp(a)                       # a = m 2^e, 0.5 <= |m| < 1
    hi = np.ldexp(np.trunc(np.ldexp(m, 24)), e - 24)
    return f32(hi), f32(a - hi)


def fma32(a, b, c):
    # float32 inputs: a*b is exact in float64, so one rounding of the exact sum to float32
    # (ties aside) is what the hardware FMA returns
    return f32(float(a) * float(b) + float(c))


def mac(acc, a, b):
    ah, al = a
    bh, bl = b
    p = f32(ah * bh)
    e = fma32(ah, bh, -p)
    e = fma32(ah, bl, e)
    e = fma32(al, bh, e)
    h, l = acc
    t = f32(h + p)
    bp = f32(t - h)
    err = f32(f32(h - f32(t - bp)) + f32(p - bp))
    return t, f32(l + f32(err + e))


def renorm(acc):
    h, l = acc
    s = f32(h + l)
    return s, f32(l - f32(s - h))


def join(acc):
    return float(acc[0]) + float(acc[1])


def test_split_is_exact_in_the_high_word():
    rng = np.random.default_rng(1)
    for a in np.concatenate([rng.normal(size=500), rng.normal(size=500) * 1e-20, rng.normal(size=500) * 1e20]):
        h, l = split(a)
        assert float(h) == float(np.float32(h))          # representable
        assert abs(float(h) + float(l) - a) <= 2.0 ** -48 * abs(a)
        assert abs(float(l)) <= 2.0 ** -23 * abs(float(h))


def test_one_product_within_2_pow_45():
    rng = np.random.default_rng(2)
    worst = 0.0
    for _ in range(3000):
        a, b = rng.normal(), rng.normal()
        got = join(mac((f32(0), f32(0)), split(a), split(b)))
        worst = max(worst, abs(got - a * b) / abs(a * b))
    # the dropped lo*lo term alone reaches 2^-46
    assert worst <= 2.0 ** -45


def test_renormalised_sums_track_fp64():
    """Sums of 300 products (a long matrix row) with a renormalisation after every product, as
    the kernels do: within 1e-14 of the sum of magnitudes (the FP64 sum itself carries ~1e-16)."""
    rng = np.random.default_rng(3)
    for trial in range(20):
        a = rng.normal(size=300) * (10.0 ** rng.uniform(-3, 3, size=300))
        b = rng.normal(size=300)
        acc = (f32(0), f32(0))
        for x, y in zip(a, b):
            acc = renorm(mac(acc, split(x), split(y)))
        exact = float(np.sum(np.array(a, dtype=np.longdouble) * np.array(b, dtype=np.longdouble)))
        scale = float(np.sum(np.abs(a * b)))
        assert abs(join(acc) - exact) <= 1e-14 * scale, trial
