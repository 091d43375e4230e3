"""The block eigensolver's dense products on the tensor cores (ls_gpu_block_update_tc: fixed-point
digit slicing, tcgen05 MMAs) against torch FP64 on the same inputs.

Two kinds of checks:
- small-integer blocks and matrices, whose exact products fit FP64: the tensor-core result must
  equal torch's bit for bit (layouts, frames, digits, the integer combination and the FP64
  conversion are all exercised without rounding);
- random blocks with magnitudes spread over decades: every entry within the documented bound
  (4k + 2) 2^-54 2^(E_r + E_c) (frames: below twice the largest magnitude of the row of [X1 | X2]
  and of the real column of [M1; M2]) plus torch FP64's own dot-product error bound."""

import importlib

import numpy as np
import pytest

from ls_helpers import LAT, ls

pytestmark = pytest.mark.gpu
lanczos = importlib.import_module("lattice-symmetries_gb300.lanczos")
N = importlib.import_module("lattice-symmetries_gb300._native")


def rand_block(S, D, k, seed, scale=1.0, spread=0.0):
    import torch
    g = torch.Generator(device="cpu").manual_seed(seed)
    x = torch.randn((S, D, k), generator=g, dtype=torch.float64) + \
        1j * torch.randn((S, D, k), generator=g, dtype=torch.float64)
    if spread:
        e = (torch.rand((S, D, 1), generator=g, dtype=torch.float64) * 2 - 1) * spread
        x = x * torch.pow(10.0, e)
    return (scale * x).to(torch.complex128).cuda()


def int_block(shape, seed, hi):
    import torch
    g = torch.Generator(device="cpu").manual_seed(seed)
    re = torch.randint(-hi, hi + 1, shape, generator=g).to(torch.float64)
    im = torch.randint(-hi, hi + 1, shape, generator=g).to(torch.float64)
    return torch.complex(re, im).cuda()


def update_tc(out, beta, W, X1, M1, X2=None, M2=None):
    import torch
    S, D, k = X1.shape
    rc = N.lib().ls_gpu_block_update_tc(S, D, k, beta, W.data_ptr() if W is not None else None, X1.data_ptr(),
                                        M1.data_ptr(), X2.data_ptr() if X2 is not None else None,
                                        M2.data_ptr() if M2 is not None else None, out.data_ptr(),
                                        torch.cuda.current_stream().cuda_stream)
    N.check(rc, "block update (tensor cores)")
    torch.cuda.synchronize()
    return out


def real_block_colmax(M):
    """Largest magnitude in each real column of [[Re m, Im m], [-Im m, Re m]] per entry, [S, 2k]."""
    import torch
    a = torch.maximum(M.real.abs(), M.imag.abs()).amax(dim=1)  # [S, k]
    return torch.repeat_interleave(a, 2, dim=1)


def frame_bound(k, X_parts, M_parts):
    """(4k + 2) 2^-54 (2 rowmax) (2 colmax) per real output, as a complex tensor of (re, im) bounds."""
    import torch
    rows = torch.stack([torch.maximum(X.real.abs(), X.imag.abs()).amax(dim=2) for X in X_parts]).amax(0)
    cols = torch.stack([real_block_colmax(M) for M in M_parts]).amax(0)
    b = (4 * k + 2) * 2.0 ** -54 * 4 * rows[:, :, None] * cols[:, None, :]  # [S, D, 2k]
    return torch.complex(b[..., 0::2], b[..., 1::2])


def within(out, ref, bound):
    import torch
    err = torch.complex((out - ref).real.abs(), (out - ref).imag.abs())
    return bool((err.real <= bound.real).all()) and bool((err.imag <= bound.imag).all())


@pytest.mark.parametrize("S,D,k", [(1, 1, 1), (2, 129, 16), (3, 1000, 8), (1, 257, 5), (2, 300, 12),
                                   (1, 128, 16), (2, 70001, 16)])
def test_update_tc_exact_on_small_integers(S, D, k):
    import torch
    W = int_block((S, D, k), 1, 1000)
    X1 = int_block((S, D, k), 2, 1000)
    X2 = int_block((S, D, k), 3, 1000)
    M1 = int_block((S, k, k), 4, 1000)
    M2 = int_block((S, k, k), 5, 1000)
    for beta in (0.0, 1.0, -2.0):
        out = torch.empty_like(W)
        update_tc(out, beta, W, X1, M1, X2, M2)
        ref = beta * W + X1 @ M1 + X2 @ M2
        assert torch.equal(out, ref), (beta, float((out - ref).abs().max()))
    out = torch.empty_like(W)
    update_tc(out, 0.0, None, X1, M1)
    assert torch.equal(out, X1 @ M1)


@pytest.mark.parametrize("S,D,k,spread,mixed", [(1, 1000, 16, 0.0, False), (3, 777, 8, 2.0, False),
                                                (2, 4097, 16, 3.0, False), (1, 333, 5, 1.0, False),
                                                (4, 31, 12, 0.0, False), (2, 1000, 16, 0.0, True)])
def test_update_tc_within_the_frame_bound(S, D, k, spread, mixed):
    """mixed: X2 1e-3 and M2 1e3 times X1 and M1, so that the shared frames of a row of [X1 | X2]
    and of a column of [M1; M2] are far above some of the terms (the bound still holds; the
    error relative to the sum of magnitudes is then larger than FP64's)."""
    import torch
    W = rand_block(S, D, k, seed=11, spread=spread)
    X1 = rand_block(S, D, k, seed=12, spread=spread)
    X2 = rand_block(S, D, k, seed=13, scale=1e-3 if mixed else 1.0, spread=spread)
    M1 = rand_block(S, k, k, seed=14)
    M2 = rand_block(S, k, k, seed=15, scale=1e3 if mixed else 1.0)
    for beta in (0.0, 1.0, -0.5):
        out = torch.empty_like(W)
        update_tc(out, beta, W, X1, M1, X2, M2)
        ref = beta * W + X1 @ M1 + X2 @ M2
        # torch's own FP64 error: 4k 2^-53 sum |x| |m| per real output, plus the final roundings
        terms = X1.abs() @ M1.abs() + X2.abs() @ M2.abs()
        own = (4 * k * 2.0 ** -53) * terms + 2.0 ** -52 * (ref.abs() + abs(beta) * W.abs())
        bound = frame_bound(k, [X1, X2], [M1, M2]) + torch.complex(own, own)
        assert within(out, ref, bound), beta
        if not mixed:  # far inside the FP32-pair kernels' 1e-13 of the sum of magnitudes
            rel = (out - ref).abs() / (abs(beta) * W.abs() + terms)
            assert float(rel.max()) < 1e-14, beta


def test_update_tc_in_place_and_aliasing():
    import torch
    S, D, k = 3, 20000, 16
    W = rand_block(S, D, k, seed=7)
    X1 = rand_block(S, D, k, seed=8)
    M1 = rand_block(S, k, k, seed=9)
    M2 = rand_block(S, k, k, seed=10)
    ref = W + X1 @ M1
    bound = W.abs() + X1.abs() @ M1.abs()
    update_tc(W, 1.0, W, X1, M1)  # out = W
    assert float(((W - ref).abs() / bound).max()) < 1e-14
    ref = X1 @ M2
    bound = X1.abs() @ M2.abs()
    update_tc(X1, 0.0, None, X1, M2)  # out = X1
    assert float(((X1 - ref).abs() / bound).max()) < 1e-14


def test_update_tc_zero_rows_and_columns():
    import torch
    S, D, k = 2, 300, 16
    X1 = rand_block(S, D, k, seed=21)
    X1[:, 5] = 0
    X1[1, 7:200] = 0
    M1 = rand_block(S, k, k, seed=22)
    M1[0, :, 3] = 0
    out = torch.full_like(X1, 5.0)
    update_tc(out, 0.0, None, X1, M1)
    ref = X1 @ M1
    assert float(out[:, 5].abs().max()) == 0.0
    assert float(out[1, 7:200].abs().max()) == 0.0
    assert float(out[0, :, 3].abs().max()) == 0.0
    assert float(((out - ref).abs() / (X1.abs() @ M1.abs()).clamp_min(1e-300)).max()) < 1e-14


def test_update_tc_on_blocks_larger_than_l2():
    """4 sectors x 400,000 rows x 16 columns (410 MB per block), a two-term update."""
    import torch
    S, D, k = 4, 400000, 16
    X = rand_block(S, D, k, seed=31)
    Y = rand_block(S, D, k, seed=32)
    M1 = rand_block(S, k, k, seed=33)
    M2 = rand_block(S, k, k, seed=34)
    out = torch.empty_like(X)
    update_tc(out, 1.0, Y, X, M1, Y, M2)
    ref = Y + X @ M1 + Y @ M2
    bound = Y.abs() + X.abs() @ M1.abs() + Y.abs() @ M2.abs()
    assert float(((out - ref).abs() / bound).max()) < 1e-14


def test_update_tc_deterministic():
    import torch
    X = rand_block(2, 50000, 16, seed=41)
    M = rand_block(2, 16, 16, seed=42)
    a = update_tc(torch.empty_like(X), 0.0, None, X, M)
    b = update_tc(torch.empty_like(X), 0.0, None, X, M)
    assert torch.equal(a, b)


def test_invalid_shapes_are_rejected_tc():
    import torch
    X = rand_block(1, 10, 17, seed=0)
    rc = N.lib().ls_gpu_block_update_tc(1, 10, 17, 0.0, None, X.data_ptr(), X.data_ptr(), None, None,
                                        X.data_ptr(), None)
    assert rc == -1
    assert "k <= 16" in N.lib().ls_gpu_last_error().decode()
    rc = N.lib().ls_gpu_block_update_tc(1, 10, 4, 1.0, None, X.data_ptr(), X.data_ptr(), None, None,
                                        X.data_ptr(), None)
    assert rc == -1
    assert "NULL" in N.lib().ls_gpu_last_error().decode()


def test_sector_lanczos_tensor_equals_fp64():
    """The same 60 block-Lanczos steps with tensor-core and with FP64 dense products: every
    sector's lowest Ritz value agrees to 1e-12 relative."""
    n = 18
    expr = LAT.xxz(LAT.chain_bonds(n), 1.0, 1.5)
    ops = []
    for kk in (0, 3, 9):
        b = ls.SpinBasis(n, n // 2, 1, ls.Symmetries(LAT.chain_symmetries(n, kk)))
        b.build(exact_norms=True)
        ops.append(ls.Operator(b, expr))
    batch = ls.SectorBatch(ops, k=8)
    e_tc = lanczos.sector_ground_states(batch, steps=60, seed=2, graph=True, dense="tensor")
    e_fp64 = lanczos.sector_ground_states(batch, steps=60, seed=2, graph=True, dense="fp64")
    assert np.abs(e_tc - e_fp64).max() <= 1e-12 * np.abs(e_fp64).max()


def gram_tc(X, Y):
    import torch
    S, D, k = X.shape
    G = torch.empty((S, k, k), dtype=torch.complex128, device="cuda")
    rc = N.lib().ls_gpu_block_gram_tc(S, D, k, X.data_ptr(), Y.data_ptr(), G.data_ptr(),
                                      torch.cuda.current_stream().cuda_stream)
    N.check(rc, "block Gram (tensor cores)")
    torch.cuda.synchronize()
    return G


@pytest.mark.parametrize("S,D,k", [(1, 1, 1), (2, 129, 16), (3, 1000, 8), (1, 257, 5), (2, 300, 12),
                                   (1, 128, 16), (3, 70001, 16), (5, 3000, 9)])
def test_gram_tc_exact_on_small_integers(S, D, k):
    import torch
    X = int_block((S, D, k), 6, 1000)
    Y = int_block((S, D, k), 7, 1000)
    assert torch.equal(gram_tc(X, Y), X.mH @ Y)
    assert torch.equal(gram_tc(X, X), X.mH @ X)


def accurate_gram(A, B, rows=20000):
    """X^H Y with every product rounded once and the sums over rows taken by tree reductions
    (error ~ log2(D) u, where a GEMM's running sums give ~ sqrt(D) u)."""
    import torch
    S, D, k = A.shape
    out = torch.zeros((S, k, k), dtype=torch.complex128, device="cuda")
    for r0 in range(0, D, rows):
        a, b = A[:, r0:r0 + rows], B[:, r0:r0 + rows]
        out += (a.conj()[..., :, None] * b[..., None, :]).sum(dim=1)
    return out


@pytest.mark.parametrize("S,D,k,scale,spread", [
    (1, 1000, 16, 1.0, 0.0), (3, 777, 8, 1e-6, 0.0), (2, 33, 3, 1e5, 0.0), (5, 4097, 16, 1.0, 3.0),
    (2, 70001, 16, 1e-3, 0.0), (1, 200000, 5, 1.0, 1.0), (4, 31, 12, 1.0, 0.0),
])
def test_gram_tc_matches_fp64(S, D, k, scale, spread):
    X = rand_block(S, D, k, seed=D + k, scale=scale, spread=spread)
    Y = rand_block(S, D, k, seed=D + k + 1, scale=1.0 / scale, spread=spread)
    for A, B in ((X, Y), (X, X)):
        G = gram_tc(A, B)
        ref = accurate_gram(A, B)
        bound = A.abs().mT @ B.abs()
        # FP64-level: 4e-15 of the sum of magnitudes (the FP32-pair kernel: 1e-13)
        assert float(((G - ref).abs() / bound).max()) <= 4e-15


def test_gram_tc_orthonormal_block_near_identity():
    """The Gram of an orthonormal block: off-diagonal entries cancel to ~1e-16 (an absolute bound
    that the FP32-pair kernel only meets to ~3e-14)."""
    import torch
    S, D, k = 3, 50000, 16
    W = rand_block(S, D, k, seed=51)
    Q = torch.linalg.qr(W)[0].contiguous()  # row-major [S, D, k], as the library expects
    G = gram_tc(Q, Q)
    eye = torch.eye(k, dtype=torch.complex128, device="cuda")
    assert float((G - eye).abs().max()) < 5e-15


def test_gram_tc_on_blocks_larger_than_l2_and_deterministic():
    import torch
    S, D, k = 4, 400000, 16
    X = rand_block(S, D, k, seed=61)
    Y = rand_block(S, D, k, seed=62)
    G = gram_tc(X, Y)
    ref = accurate_gram(X, Y)
    assert float(((G - ref).abs() / (X.abs().mT @ Y.abs())).max()) <= 4e-15
    assert torch.equal(G, gram_tc(X, Y))


def test_gram_tc_empty_and_invalid():
    import torch
    X = torch.empty((3, 0, 4), dtype=torch.complex128, device="cuda")
    G = torch.full((3, 4, 4), 7.0 + 1j, dtype=torch.complex128, device="cuda")
    rc = N.lib().ls_gpu_block_gram_tc(3, 0, 4, X.data_ptr(), X.data_ptr(), G.data_ptr(),
                                      torch.cuda.current_stream().cuda_stream)
    N.check(rc, "block Gram (tensor cores)")
    torch.cuda.synchronize()
    assert float(G.abs().max()) == 0.0
    Z = rand_block(1, 10, 17, seed=0)
    rc = N.lib().ls_gpu_block_gram_tc(1, 10, 17, Z.data_ptr(), Z.data_ptr(), Z.data_ptr(), None)
    assert rc == -1
    assert "k <= 16" in N.lib().ls_gpu_last_error().decode()
