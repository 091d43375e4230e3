"""CPU replay of the MMA schedules of the tensor-core block products
(lattice-symmetries_gb300/csrc/blockops_tc.cu), checking that every digit pair (i, j) of weight
t = i + j <= 7 is accumulated exactly once, into a cell that holds weight t only, and that the
FP32 cell sums stay exact.

Update: MMA (plane i of X, planes 0..7-i of M) writes accumulator columns [i NC, 8 NC): pair (i, j)
lands in the column block of group t = i + j.

Gram: MMA (X planes a .. a+Q-1 as lane blocks q, Y planes j, j+1 as column blocks b) for region
r, a = r Q - j, even j, skipped when every plane is negative; zero planes stand in for planes < 0.
Lane block q and column block b of region r hold weight t = r Q + q + b."""

import collections

import pytest

DIGITS = 8
B_MAX = [128, 64, 64, 128, 64, 64, 128, 64]  # |d_i| bounds of the base-2^7 digits


def update_schedule():
    cells = collections.defaultdict(list)  # group t -> pairs
    for i in range(DIGITS):
        for j in range(DIGITS - i):  # N = NC (8 - i): M planes 0 .. 7 - i
            cells[i + j].append((i, j))
    return cells


def test_update_schedule_covers_every_pair_once():
    cells = update_schedule()
    seen = collections.Counter(p for ps in cells.values() for p in ps)
    want = {(i, j) for i in range(DIGITS) for j in range(DIGITS) if i + j <= 7}
    assert set(seen) == want and all(v == 1 for v in seen.values())
    for t, ps in cells.items():
        assert all(i + j == t for i, j in ps)
        K = 64  # 4 kp reals, kp = 16
        assert K * sum(B_MAX[i] * B_MAX[j] for i, j in ps) <= 2 ** 22


@pytest.mark.parametrize("kp", [16, 8])
def test_gram_schedule_covers_every_pair_once(kp):
    NR = 2 * kp
    Q = 128 // NR
    REG = DIGITS // Q
    Z = 2 if Q == 4 else 6  # zero planes in front of X's planes
    cells = collections.defaultdict(list)  # (r, q, b) -> pairs
    mmas = 0
    for r in range(REG):
        for j in range(0, DIGITS, 2):
            a = r * Q - j
            if a + Q - 1 < 0:
                continue  # only zero planes
            assert a >= -Z, "plane below the zero planes"
            assert a + Q - 1 <= DIGITS - 1, "plane above X's planes"
            mmas += 1
            for q in range(Q):
                i = a + q
                if i < 0:
                    continue  # a zero plane: contributes nothing
                for b in range(2):
                    jj = j + b
                    assert jj < DIGITS
                    cells[(r, q, b)].append((i, jj))
    # every pair with i + j <= 7 exactly once, in a cell of its weight
    seen = collections.Counter(p for ps in cells.values() for p in ps)
    want = {(i, j) for i in range(DIGITS) for j in range(DIGITS) if i + j <= 7}
    assert want <= set(seen)
    assert all(v == 1 for v in seen.values())
    for (r, q, b), ps in cells.items():
        t = r * Q + q + b
        assert all(i + j == t for i, j in ps)
        # a cell sums <= 128 rows of these products: exact in FP32
        assert 128 * sum(B_MAX[i] * B_MAX[j] for i, j in ps) <= 2 ** 23
    # a lane block q's cells span weights q .. q + TOP: the 64-bit join stays below 2^63
    top = (REG - 1) * Q + 1
    assert 2 ** 23 * 2 ** (7 * top) < 2 ** 63
    assert mmas == (6 if kp == 16 else 4)  # MMAs per K step
