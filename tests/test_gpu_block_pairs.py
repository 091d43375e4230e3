"""Complex blocks of 8 and 16 right-hand sides in FP32-pair arithmetic (opt-in; FP64 is the
default block arithmetic): every column against the oracle (relative L2 <= 1e-12, the tolerance of the hot
path) and against the FP64 block kernels (relative L2 <= 1e-13), for the plain, adjoint,
fermionic and batched multi-sector kernels."""

import numpy as np
import pytest

from ls_helpers import LAT, chain_case, ls, square_case

pytestmark = pytest.mark.gpu

RTOL = 1e-12
PAIR_VS_FP64 = 1e-13


def rel_l2(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture
def arithmetic():
    """Restores the default ("fp64") after each test."""
    yield ls.Operator.block_arithmetic
    ls.Operator.block_arithmetic("fp64")


def both_modes(apply, arithmetic):
    """(pairs for every group, FP64)."""
    arithmetic("fp64")
    y64 = apply()
    arithmetic("pairs")
    yp = apply()
    return yp, y64


def random_block(D, k, seed):
    import torch
    rng = np.random.default_rng(seed)
    return torch.from_numpy(rng.normal(size=(D, k)) + 1j * rng.normal(size=(D, k))).cuda()


CASES = {
    "chain16_k8_p1_zm1": lambda: chain_case(16, k=8, p=1, inv=-1),  # real elements, spin inversion
    "chain14_k3_h7": lambda: chain_case(14, k=3, h=7),               # complex sector
    "square4_pipi_z1": lambda: square_case(4, 2, 2, inv=1, J2=0.5),  # 128-element group
}


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("k", [8, 16, 24])
def test_pair_blocks_match_oracle_and_fp64(arithmetic, name, k):
    c = CASES[name]()
    c.basis.build()
    D = c.basis.number_states
    X = random_block(D, k, seed=k)
    yp, y64 = both_modes(lambda: c.op.apply_device(X).cpu().numpy(), arithmetic)
    states = c.basis.states
    Xh = X.cpu().numpy()
    for j in range(0, k, 5):
        yo = c.oracle_matvec(states, Xh[:, j], complex_=True)
        assert rel_l2(yp[:, j], yo) <= RTOL, j
    for j in range(k):
        assert rel_l2(yp[:, j], y64[:, j]) <= PAIR_VS_FP64, j


def test_pair_adjoint_matches_fp64(arithmetic):
    c = chain_case(14, k=3, h=7)
    c.basis.build()
    X = random_block(c.basis.number_states, 16, seed=3)
    yp, y64 = both_modes(lambda: c.op.apply_device(X, adjoint=True).cpu().numpy(), arithmetic)
    for j in range(16):
        assert rel_l2(yp[:, j], y64[:, j]) <= PAIR_VS_FP64
    # H is Hermitian: H^dagger X = H X
    yf = c.op.apply_device(X).cpu().numpy()
    assert rel_l2(yp, yf) <= RTOL


def test_pair_fermionic_blocks_match_fp64(arithmetic):
    L = 3
    syms = ls.Symmetries(LAT.square_symmetries(L, 1, 0, False))
    basis = ls.SpinfulFermionBasis(L * L, (3, 3), symmetries=syms)
    basis.build()
    t, U = LAT.hubbard_parts(LAT.square_bonds(L), L * L)
    op = ls.Operator(basis, t + U.scale(4.0))
    X = random_block(basis.number_states, 8, seed=4)
    yp, y64 = both_modes(lambda: op.apply_device(X).cpu().numpy(), arithmetic)
    for j in range(8):
        assert rel_l2(yp[:, j], y64[:, j]) <= PAIR_VS_FP64
    # column by column (one right-hand side always runs in FP64)
    for j in range(8):
        yj = op.apply_device(X[:, j].contiguous()).cpu().numpy()
        assert rel_l2(yp[:, j], yj) <= PAIR_VS_FP64


def test_pair_batched_sectors_match_fp64(arithmetic):
    n = 16
    expr = LAT.xxz(LAT.chain_bonds(n), 1.0, 1.5)
    ops = []
    for k in range(n):
        for z in (1, -1):
            b = ls.SpinBasis(n, n // 2, z, ls.Symmetries(LAT.chain_symmetries(n, k)))
            b.build()
            if b.number_states:
                ops.append(ls.Operator(b, expr))
    batch = ls.SectorBatch(ops, k=16)
    assert batch.batched
    import torch
    g = torch.Generator(device="cpu").manual_seed(7)
    batch.X.zero_()
    for s in range(batch.number_sectors):
        d = batch.sizes[s]
        batch.X[s, :d].copy_(torch.randn((d, 16), generator=g, dtype=torch.float64)
                             + 1j * torch.randn((d, 16), generator=g, dtype=torch.float64))

    def run():
        batch.run(check=True)
        return batch.Y.clone().cpu().numpy()

    yp, y64 = both_modes(run, arithmetic)
    for s in range(batch.number_sectors):
        d = batch.sizes[s]
        assert rel_l2(yp[s, :d], y64[s, :d]) <= PAIR_VS_FP64, s
        # and the single-sector pair kernel
        ref = ops[s].apply_device(batch.x(s).contiguous()).cpu().numpy()
        assert rel_l2(yp[s, :d], ref) <= PAIR_VS_FP64, s


def test_block_arithmetic_setting(arithmetic):
    assert arithmetic() == "fp64"
    assert arithmetic("fp64") == "fp64"
    assert arithmetic() == "fp64"
    with pytest.raises(ValueError):
        arithmetic("fp32")
    from importlib import import_module
    N = import_module("lattice-symmetries_gb300._native")
    assert N.lib().ls_gpu_set_block_arithmetic(3) == -1
    assert arithmetic("pairs") == "pairs"
    assert arithmetic("auto") == "auto"


def test_auto_uses_pairs_for_small_groups_only(arithmetic):
    """auto = pairs for a 16-element group (same result as "pairs"), FP64 for a 128-element group
    (bit-identical to "fp64")."""
    import torch
    small = chain_case(16, k=8, p=1, inv=-1)
    large = square_case(4, 2, 2, inv=1, J2=0.5)
    for c, same_as in ((small, "pairs"), (large, "fp64")):
        c.basis.build()
        X = random_block(c.basis.number_states, 16, seed=9)
        arithmetic("auto")
        ya = c.op.apply_device(X)
        arithmetic(same_as)
        yb = c.op.apply_device(X)
        assert torch.equal(ya, yb), same_as
