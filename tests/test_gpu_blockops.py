"""Dense products of the block eigensolver (ls_gpu_block_gram / ls_gpu_block_update, FP32-pair
arithmetic) against torch FP64 on the same inputs, and block Lanczos with the FP32-pair products
against the same recurrence with torch FP64 GEMMs.

Tolerance: every entry within 1e-13 of the sum of the magnitudes of its terms (one product is
below 2^-45 relative; the Gram adds 32-row tiles in FP64)."""

import importlib

import numpy as np
import pytest

from ls_helpers import LAT, ls

pytestmark = pytest.mark.gpu
lanczos = importlib.import_module("lattice-symmetries_gb300.lanczos")
N = importlib.import_module("lattice-symmetries_gb300._native")

TOL = 1e-13


def rand_block(S, D, k, seed, scale=1.0, spread=0.0):
    import torch
    g = torch.Generator(device="cpu").manual_seed(seed)
    x = torch.randn((S, D, k), generator=g, dtype=torch.float64) + \
        1j * torch.randn((S, D, k), generator=g, dtype=torch.float64)
    if spread:
        # row magnitudes spread over 10^-spread .. 10^spread
        e = (torch.rand((S, D, 1), generator=g, dtype=torch.float64) * 2 - 1) * spread
        x = x * torch.pow(10.0, e)
    return (scale * x).to(torch.complex128).cuda()


def gram(X, Y):
    import torch
    S, D, k = X.shape
    G = torch.empty((S, k, k), dtype=torch.complex128, device="cuda")
    rc = N.lib().ls_gpu_block_gram(S, D, k, X.data_ptr(), Y.data_ptr(), G.data_ptr(),
                                   torch.cuda.current_stream().cuda_stream)
    N.check(rc, "block Gram")
    torch.cuda.synchronize()
    return G


def update(out, beta, W, X1, M1, X2=None, M2=None):
    import torch
    S, D, k = X1.shape
    rc = N.lib().ls_gpu_block_update(S, D, k, beta, W.data_ptr() if W is not None else None, X1.data_ptr(),
                                     M1.data_ptr(), X2.data_ptr() if X2 is not None else None,
                                     M2.data_ptr() if M2 is not None else None, out.data_ptr(),
                                     torch.cuda.current_stream().cuda_stream)
    N.check(rc, "block update")
    torch.cuda.synchronize()
    return out


@pytest.mark.parametrize("S,D,k,scale,spread", [
    (1, 1, 1, 1.0, 0.0), (1, 1000, 16, 1.0, 0.0), (3, 777, 8, 1e-6, 0.0), (2, 33, 3, 1e5, 0.0),
    (5, 4097, 16, 1.0, 3.0), (2, 70001, 16, 1e-3, 0.0), (1, 200000, 5, 1.0, 1.0), (4, 31, 12, 1.0, 0.0),
])
def test_gram_matches_fp64(S, D, k, scale, spread):
    X = rand_block(S, D, k, seed=D + k, scale=scale, spread=spread)
    Y = rand_block(S, D, k, seed=D + k + 1, scale=1.0 / scale, spread=spread)
    G = gram(X, Y)
    ref = X.mH @ Y
    bound = X.abs().mT @ Y.abs()
    assert float(((G - ref).abs() / bound).max()) <= TOL
    # X == Y: the Hermitian Gram of one block
    G2 = gram(X, X)
    ref2 = X.mH @ X
    bound2 = X.abs().mT @ X.abs()
    assert float(((G2 - ref2).abs() / bound2).max()) <= TOL


def test_gram_of_empty_blocks_is_zero():
    import torch
    X = torch.empty((3, 0, 4), dtype=torch.complex128, device="cuda")
    G = torch.full((3, 4, 4), 7.0 + 1j, dtype=torch.complex128, device="cuda")
    rc = N.lib().ls_gpu_block_gram(3, 0, 4, X.data_ptr(), X.data_ptr(), G.data_ptr(),
                                   torch.cuda.current_stream().cuda_stream)
    N.check(rc, "block Gram")
    torch.cuda.synchronize()
    assert float(G.abs().max()) == 0.0


def test_gram_deterministic():
    X = rand_block(4, 50000, 16, seed=5)
    Y = rand_block(4, 50000, 16, seed=6)
    import torch
    assert torch.equal(gram(X, Y), gram(X, Y))


@pytest.mark.parametrize("S,D,k", [(1, 1, 1), (2, 1000, 16), (3, 517, 8), (2, 70001, 16), (1, 333, 5)])
def test_update_matches_fp64(S, D, k):
    import torch
    W = rand_block(S, D, k, seed=1)
    X1 = rand_block(S, D, k, seed=2)
    X2 = rand_block(S, D, k, seed=3)
    g = torch.Generator(device="cpu").manual_seed(4)
    M1 = (torch.randn((S, k, k), generator=g, dtype=torch.float64) + 1j * torch.randn(
        (S, k, k), generator=g, dtype=torch.float64)).to(torch.complex128).cuda()
    M2 = (torch.randn((S, k, k), generator=g, dtype=torch.float64) * 1e3 + 0j).to(torch.complex128).cuda()
    for beta in (0.0, 1.0, -0.5):
        out = torch.empty_like(W)
        update(out, beta, W, X1, M1, X2, M2)
        ref = beta * W + X1 @ M1 + X2 @ M2
        bound = abs(beta) * W.abs() + X1.abs() @ M1.abs() + X2.abs() @ M2.abs()
        assert float(((out - ref).abs() / bound).max()) <= TOL, beta
    # one term, no W
    out = torch.empty_like(W)
    update(out, 0.0, None, X1, M1)
    ref = X1 @ M1
    assert float(((out - ref).abs() / (X1.abs() @ M1.abs())).max()) <= TOL


def test_update_in_place():
    import torch
    S, D, k = 3, 20000, 16
    W = rand_block(S, D, k, seed=7)
    X1 = rand_block(S, D, k, seed=8)
    M1 = rand_block(S, k, k, seed=9)
    M2 = rand_block(S, k, k, seed=10)
    # out = W (beta = 1): W <- W + X1 M1
    ref = W + X1 @ M1
    bound = W.abs() + X1.abs() @ M1.abs()
    update(W, 1.0, W, X1, M1)
    assert float(((W - ref).abs() / bound).max()) <= TOL
    # out = X1 (beta = 0): X1 <- X1 M2
    ref = X1 @ M2
    bound = X1.abs() @ M2.abs()
    update(X1, 0.0, None, X1, M2)
    assert float(((X1 - ref).abs() / bound).max()) <= TOL


def test_invalid_shapes_are_rejected():
    import torch
    X = rand_block(1, 10, 17, seed=0)
    G = torch.empty((1, 17, 17), dtype=torch.complex128, device="cuda")
    rc = N.lib().ls_gpu_block_gram(1, 10, 17, X.data_ptr(), X.data_ptr(), G.data_ptr(), None)
    assert rc == -1
    assert "k <= 16" in N.lib().ls_gpu_last_error().decode()
    # beta != 0 without W
    rc = N.lib().ls_gpu_block_update(1, 10, 4, 1.0, None, X.data_ptr(), G.data_ptr(), None, None, X.data_ptr(),
                                     None)
    assert rc == -1
    assert "NULL" in N.lib().ls_gpu_last_error().decode()


def test_cholqr_paired_orthonormal():
    import torch
    W = rand_block(3, 30000, 16, seed=11, spread=2.0)
    Q, R = lanczos._cholqr(W.clone(), dense="paired")
    eye = torch.eye(16, dtype=torch.complex128, device="cuda")
    assert float((Q.mH @ Q - eye).abs().max()) < 1e-12
    assert float((Q @ R - W).abs().max()) < 1e-12 * float(W.abs().max())


def test_sector_lanczos_paired_equals_fp64():
    """The same 60 block-Lanczos steps with FP32-pair and with FP64 dense products: every sector's
    lowest Ritz value agrees to 1e-12 relative, and both equal dense diagonalisation."""
    import torch
    n = 18
    expr = LAT.xxz(LAT.chain_bonds(n), 1.0, 1.5)
    ops = []
    for k in (0, 3, 9):
        b = ls.SpinBasis(n, n // 2, 1, ls.Symmetries(LAT.chain_symmetries(n, k)))
        b.build(exact_norms=True)
        ops.append(ls.Operator(b, expr))
    batch = ls.SectorBatch(ops, k=8)
    e_pair = lanczos.sector_ground_states(batch, steps=60, seed=2, graph=True, dense="paired")
    e_fp64 = lanczos.sector_ground_states(batch, steps=60, seed=2, graph=True, dense="fp64")
    assert np.abs(e_pair - e_fp64).max() <= 1e-12 * np.abs(e_fp64).max()
    for s, op in enumerate(ops):
        d = op.basis.number_states
        h = op.apply_device(torch.eye(d, dtype=torch.complex128, device="cuda")).cpu().numpy()
        ref = np.linalg.eigvalsh(h)[0]
        assert abs(e_pair[s] - ref) < 1e-10 * abs(ref), (s, e_pair[s], ref)


def test_gram_and_update_on_blocks_larger_than_l2():
    """4 sectors x 400,000 rows x 16 columns (410 MB per block): the Gram and a two-term update
    against torch FP64 (this shape is also the one profiled for the dense kernels)."""
    import torch
    S, D, k = 4, 400000, 16
    X = rand_block(S, D, k, seed=31)
    Y = rand_block(S, D, k, seed=32)
    G = gram(X, Y)
    ref = X.mH @ Y
    assert float(((G - ref).abs() / (X.abs().mT @ Y.abs())).max()) <= TOL
    del ref
    M1 = rand_block(S, k, k, seed=33)
    M2 = rand_block(S, k, k, seed=34)
    out = torch.empty_like(X)
    update(out, 1.0, Y, X, M1, X, M2)
    ref = Y + X @ (M1 + M2)
    bound = Y.abs() + X.abs() @ (M1.abs() + M2.abs())
    assert float(((out - ref).abs() / bound).max()) <= TOL


def test_gram_of_orthonormal_blocks_within_the_absolute_bound():
    """The Gram of an orthonormal block: off-diagonal entries cancel to ~1e-16, so the pair
    kernel's error is not small relative to them; it stays within 2^-45 per product times the sum
    of the products' magnitudes (with a factor 8 for the tile sums), the bound it documents."""
    import torch
    X = rand_block(2, 60000, 16, seed=21)
    Q = torch.stack([torch.linalg.qr(X[s])[0] for s in range(X.shape[0])]).contiguous()
    G = gram(Q, Q)
    G64 = torch.einsum("sdi,sdj->sij", Q.conj(), Q)
    mag = torch.einsum("sdi,sdj->sij", Q.abs(), Q.abs())
    err = (G - G64).abs()
    assert bool((err <= 8 * 2.0 ** -45 * mag).all())
    off = ~torch.eye(16, dtype=torch.bool, device="cuda")
    assert float(G64.abs()[:, off].max()) < 1e-14
