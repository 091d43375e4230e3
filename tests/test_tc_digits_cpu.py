"""CPU restatement of the fixed-point digit arithmetic behind the tensor-core block products
(lattice-symmetries_gb300/csrc/blockops_tc.cu), in exact Python integers:

- fixed56 + digits8: v = sign(v) sum_i d_i 2^(E - 7 - 7i) exactly (up to the truncation of v below
  2^(E - 56)), every digit an exact bf16 value with |d_i| <= 128 (i = 0, 3, 6) or <= 64;
- the exactness bound of the FP32 group sums: K * max_t sum_{i+j=t} |d_i| |d_j| <= 2^22 for K = 64;
- the update's integer combination (Horner in base 2^7 over groups 0..6, group 7 truncated) and its
  error against the exact dot product, within (K + 2) 2^-54 2^(E_r + E_c);
- the integer-to-FP64 conversion with a power-of-two scale: round to nearest even.

The device code follows the same steps with 64-bit integers, fmaf/fadd rounding tricks and
tcgen05 MMAs; the GPU tests compare it with torch FP64."""

import math
import random
import struct

import numpy as np

DIGITS = 8


def exp_field(v: float) -> int:
    return (struct.unpack("<Q", struct.pack("<d", v))[0] >> 52) & 0x7FF


def fixed56(v: float, emax: int) -> int:
    u = struct.unpack("<Q", struct.pack("<d", v))[0]
    e = (u >> 52) & 0x7FF
    if e == 0:
        return 0
    m = ((u & ((1 << 52) - 1)) | (1 << 52)) << 3
    d = emax - e
    return m >> d if d < 56 else 0


def rint(x: float) -> int:
    """Round half to even, as fmaf(x, s, 1.5 * 2^23) - 1.5 * 2^23 does for |x| < 2^22."""
    return int(round(x))


def digits8(F: int, neg: bool):
    """Top-down signed digits of each chunk: 21 bits -> d0 2^14 + d1 2^7 + d2 (twice), 14 bits ->
    d6 2^7 + d7."""
    sg = -1 if neg else 1
    chunks = [F >> 35, (F >> 14) & ((1 << 21) - 1), F & ((1 << 14) - 1)]
    d = []
    for c, y in enumerate(chunks):
        y *= sg
        if c < 2:
            d0 = rint(y / 2 ** 14)
            r = y - d0 * 2 ** 14
            d1 = rint(r / 2 ** 7)
            d += [d0, d1, r - d1 * 2 ** 7]
        else:
            d6 = rint(y / 2 ** 7)
            d += [d6, y - d6 * 2 ** 7]
    return d


def bf16_exact(x: int) -> bool:
    if x == 0:
        return True
    a = abs(x)
    return a >> max(0, a.bit_length() - 8) << max(0, a.bit_length() - 8) == a


def frame_of(values):
    return max(exp_field(v) for v in values)


def test_digits_reconstruct_the_fixed_point_value():
    rng = random.Random(1)
    for _ in range(3000):
        v = rng.uniform(-1, 1) * 10.0 ** rng.uniform(-30, 30)
        emax = exp_field(v) + rng.randrange(0, 60)
        F = fixed56(v, emax)
        assert F < 2 ** 56
        d = digits8(F, v < 0)
        assert sum(di * 2 ** (49 - 7 * i) for i, di in enumerate(d)) == (-F if v < 0 else F)
        for i, di in enumerate(d):
            assert abs(di) <= (128 if i in (0, 3, 6) else 64)
            assert bf16_exact(di)
        # F is |v| 2^(56 - E) truncated, E = emax - 1022
        E = emax - 1022
        assert 0 <= abs(v) * 2.0 ** (56 - E) - F < 1.0 + 1e-9 * F


def test_group_sums_fit_fp32_exactly():
    b = [128, 64, 64, 128, 64, 64, 128, 64]
    worst = max(sum(b[i] * b[t - i] for i in range(max(0, t - 7), min(t, 7) + 1)) for t in range(8))
    assert worst == 2 ** 16
    assert 64 * worst <= 2 ** 22  # K = 4 kp reals with kp = 16: below 2^24, and within the 2^22 of the
    # magic-number integer extraction (1.5 * 2^23 offset)


def update_combination(x_row, m_col):
    """One output of the tensor-core update: row frame, column frame, digit-group sums, Horner with
    group 7 truncated, returned as an exact rational (integer H and scale exponent)."""
    er, ec = frame_of(x_row), frame_of(m_col)
    dx = [digits8(fixed56(v, er), v < 0) for v in x_row]
    dm = [digits8(fixed56(v, ec), v < 0) for v in m_col]
    acc = [0] * DIGITS
    for a, b in zip(dx, dm):
        for i in range(DIGITS):
            for j in range(DIGITS - i):
                acc[i + j] += a[i] * b[j]
    assert all(abs(s) <= 2 ** 22 for s in acc)
    H = acc[0]
    for t in range(1, DIGITS - 1):
        H = H * 128 + acc[t]
    H += acc[7] >> 7  # arithmetic shift: floor
    assert abs(H) < 2 ** 63
    return H, er + ec - 2100, er, ec


def test_update_combination_error_bound():
    rng = np.random.default_rng(2)
    K = 64
    for trial in range(200):
        spread = rng.uniform(0, 6)
        x = (rng.standard_normal(K) * 10.0 ** rng.uniform(-spread, spread, K)).tolist()
        m = (rng.standard_normal(K) * 10.0 ** rng.uniform(-3, 3)).tolist()
        H, scale, er, ec = update_combination(x, m)
        from fractions import Fraction
        exact = sum(Fraction(a) * Fraction(b) for a, b in zip(x, m))
        got = Fraction(H) * Fraction(2) ** scale
        Er, Ec = er - 1022, ec - 1022
        bound = Fraction(K + 2) * Fraction(2) ** (Er + Ec - 54)
        assert abs(got - exact) <= bound, trial


def int64_scaled_to_double(H: int, scale: int) -> float:
    """Restatement of the device conversion: normalise, keep 53 bits, round half to even."""
    if H == 0:
        return 0.0
    neg = H < 0
    a = -H if neg else H
    lz = 64 - a.bit_length()
    n = a << lz
    mant = n >> 11
    rem = n & 0x7FF
    if rem > 0x400 or (rem == 0x400 and (mant & 1)):
        mant += 1
    be = 63 - lz + scale + 1023
    assert 0 < be < 2047
    bits = ((be - 1) << 52) + mant
    out = struct.unpack("<d", struct.pack("<Q", bits))[0]
    return -out if neg else out


def test_integer_to_double_rounds_to_nearest_even():
    rng = random.Random(3)
    for _ in range(5000):
        H = rng.randrange(-(2 ** 62), 2 ** 62)
        s = rng.randrange(-200, 200)
        # Python's int -> float conversion rounds half to even; ldexp by a power of two is exact
        assert int64_scaled_to_double(H, s) == math.ldexp(float(H), s)
    for H in (2 ** 53 + 1, 2 ** 53 + 3, 2 ** 60 + 2 ** 7, -(2 ** 54 + 2), 1, -1):
        assert int64_scaled_to_double(H, 0) == float(H)
