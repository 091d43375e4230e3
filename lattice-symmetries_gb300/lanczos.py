"""Block Lanczos on the GPU for many symmetry sectors at once.

This replaces the eigensolver drivers that sit on top of the reference's matvec (scipy's eigsh
over Operator._matvec in python/lattice_symmetries/__init__.py:751-752, and the PRIMME driver of
chapel/src/Diagonalize.chpl): every step applies H to a block of k vectors in every sector with
ONE batched matvec (SectorBatch), then orthogonalises all sectors together with batched dense
algebra.  One step (matvec + orthogonalisation) is recorded in a CUDA graph and replayed.

Recurrence (per sector, blocks of k columns, Q_0 orthonormal, Q_{-1} = 0, B_{-1} = 0):

    W   = H Q_j
    A_j = Q_j^H W
    W  <- W - Q_j A_j - Q_{j-1} B_{j-1}^H        (+ one local re-orthogonalisation against Q_j)
    W   = Q_{j+1} B_j                             (Cholesky QR, two passes)

and the eigenvalues of the block-tridiagonal T (diagonal blocks A_j, sub-diagonal blocks B_j)
approximate the extremal eigenvalues of H.  There is no global re-orthogonalisation, so converged
Ritz values can repeat ("ghosts"); the lowest ones are reliable.

Dense products (`dense=`): "tensor" (default on the GPU for k <= 16) runs the tall-skinny Gram
matrices and block updates through the library's tensor-core kernels (ls_gpu_block_gram_tc /
ls_gpu_block_update_tc: FP64 storage, values cut into fixed-point bf16 digits whose products are
summed exactly by tcgen05 MMAs, FP64-level results); "paired" through its FP32-pair kernels
(ls_gpu_block_gram / ls_gpu_block_update: below 2^-45 relative error per product); "fp64" uses
torch's FP64 GEMMs (GB300's FP64 pipe is narrow: several times slower).
CPU tensors always take the torch path.
"""

from __future__ import annotations

from typing import Callable, List, Optional, Tuple

import numpy as np


DENSE_MODES = ("tensor", "paired", "fp64")
DENSE_DEFAULT = "tensor"


def _mode(X, dense) -> str:
    """The dense-product arithmetic for block X: 'tensor' / 'paired' (the library's kernels) need
    a CUDA complex128 [S, D, k] block with k <= 16, else torch FP64 GEMMs run."""
    import torch

    mode = DENSE_DEFAULT if dense is None else dense
    if mode not in DENSE_MODES:
        raise ValueError("dense must be one of " + ", ".join(repr(m) for m in DENSE_MODES))
    native = X.is_cuda and X.dtype == torch.complex128 and X.dim() == 3 and X.shape[-1] <= 16
    return mode if native else "fp64"


def _library(X, dense) -> bool:
    """True when the library's dense kernels (tensor-core or FP32-pair) take block X."""
    return _mode(X, dense) != "fp64"


def _native():
    from . import _native as N

    return N, N.lib()


def _gram(X, Y, dense=None, blocks: int = 256, min_rows: int = 64):
    """X^H Y for [S, D, k] blocks as [S, k, k].

    tensor: one call of ls_gpu_block_gram_tc; paired: ls_gpu_block_gram.  fp64 (torch): a single GEMM with inner dimension D
    (hundreds of thousands) and a 16 x 16 output leaves most of the GPU idle, so the rows are split
    into `blocks` equal row blocks (S * blocks GEMMs whose partial results are summed) plus the
    remaining D mod blocks rows."""
    import torch

    S, D, k = X.shape
    if _library(X, dense):
        N, lib = _native()
        X = X.contiguous()
        Y = Y.contiguous()
        G = torch.empty((S, k, k), dtype=X.dtype, device=X.device)
        stream = torch.cuda.current_stream(X.device).cuda_stream
        fn = lib.ls_gpu_block_gram_tc if _mode(X, dense) == "tensor" else lib.ls_gpu_block_gram
        N.check(fn(S, D, k, X.data_ptr(), Y.data_ptr(), G.data_ptr(), stream), "block Gram")
        return G
    c = blocks
    while c > 1 and D // c < min_rows:
        c //= 2
    m = D // c
    if c <= 1:
        return X.mH @ Y
    main = (X[:, :c * m].reshape(S, c, m, k).mH @ Y[:, :c * m].reshape(S, c, m, k)).sum(1)
    if c * m == D:
        return main
    return main + X[:, c * m:].mH @ Y[:, c * m:]


def _update(out, beta: float, W, X1, M1, X2=None, M2=None, dense=None):
    """out = beta W + X1 M1 (+ X2 M2) for [S, D, k] blocks and [S, k, k] matrices; out may be W, X1
    or X2 (tensor: one call of ls_gpu_block_update_tc; paired: ls_gpu_block_update; fp64: torch
    GEMMs)."""
    import torch

    S, D, k = X1.shape
    if _library(X1, dense) and out.is_contiguous():
        N, lib = _native()
        X1 = X1.contiguous()
        M1 = M1.contiguous()
        if X2 is not None:
            X2 = X2.contiguous()
            M2 = M2.contiguous()
        if W is not None and beta != 0.0:
            W = W.contiguous()
        stream = torch.cuda.current_stream(X1.device).cuda_stream
        fn = lib.ls_gpu_block_update_tc if _mode(X1, dense) == "tensor" else lib.ls_gpu_block_update
        rc = fn(S, D, k, float(beta), W.data_ptr() if (W is not None and beta != 0.0) else None,
                X1.data_ptr(), M1.data_ptr(), X2.data_ptr() if X2 is not None else None,
                M2.data_ptr() if M2 is not None else None, out.data_ptr(), stream)
        N.check(rc, "block update")
        return out
    if beta != 0.0 and out is W and X1 is not out and X2 is not out:
        if beta != 1.0:
            out.mul_(beta)
        out.baddbmm_(X1, M1)
        if X2 is not None:
            out.baddbmm_(X2, M2)
        return out
    res = torch.matmul(X1, M1)
    if X2 is not None:
        res = res + torch.matmul(X2, M2)
    if beta != 0.0:
        res = res + beta * W
    out.copy_(res)
    return out


def _chol_factor(G, eps: float = 1e-15):
    """Upper Cholesky factor R of the (symmetrised, slightly shifted) Gram matrix G = R^H R and
    its inverse, batched over the leading dimension."""
    import torch

    k = G.shape[-1]
    eye = torch.eye(k, dtype=G.dtype, device=G.device)
    G = 0.5 * (G + G.mH)
    scale = torch.diagonal(G, dim1=-2, dim2=-1).real.mean(-1).clamp_min(1e-300)
    G = G + (eps * scale)[..., None, None] * eye
    L, _ = torch.linalg.cholesky_ex(G)
    R = L.mH
    return R, torch.linalg.solve_triangular(R, eye.expand_as(R), upper=True)


def _cholqr(W, eps: float = 1e-15, passes: int = 2, dense=None, out=None):
    """W = Q R with Q orthonormal (batched over the leading dimension): two Cholesky-QR passes.
    A tiny diagonal shift keeps exhausted blocks (W ~ 0) finite instead of NaN.  The k x k factor
    is inverted explicitly, so that applying it is a GEMM rather than a triangular solve over D.
    With `out`, Q is written there and W serves as scratch for the intermediate passes."""
    import torch

    k = W.shape[-1]
    R = None
    Q = W
    for p in range(passes):
        Rp, Rinv = _chol_factor(_gram(Q, Q, dense), eps)
        if out is None:
            target = torch.empty_like(Q)
        else:
            target = out if p == passes - 1 else W
        Q = _update(target, 0.0, None, Q, Rinv, dense=dense)
        R = Rp if R is None else Rp @ R
    return Q, R


def lanczos_step(apply: Callable[[], None], Q, W, Qp, Bp, A_out, B_out, lean: bool = False,
                 dense=None) -> None:
    """One block-Lanczos step on preallocated tensors ([S, D, k] blocks, [S, k, k] coefficients).

    `apply()` must compute W = H Q in place.  On return Q holds Q_{j+1}, Qp holds Q_j,
    Bp = B_out = B_j and A_out = A_j; W is scratch.  Everything is stream-ordered (no host
    synchronisation), so the step can be captured in a CUDA graph.  lean=True skips the local
    re-orthogonalisation and uses one Cholesky-QR pass: 4 tall-skinny products per step instead
    of 7 (the full step folds the re-orthogonalisation update into the first Cholesky-QR
    update)."""
    apply()
    A = _gram(Q, W, dense)
    _update(W, 1.0, W, Q, -A, Qp, -Bp.mH, dense=dense)  # W -= Q A + Q_{j-1} B_{j-1}^H
    if lean:
        A = 0.5 * (A + A.mH)
        Qp.copy_(Q)
        _, B = _cholqr(W, passes=1, dense=dense, out=Q)
    else:
        # Local re-orthogonalisation against the current block, W' = W - Q C with C = Q^H W,
        # folded into the first Cholesky-QR pass: W'^H W' = W^H W - C^H C (Q^H Q = I), and
        # (W - Q C) R^-1 = W R^-1 - Q (C R^-1) is one two-term update.
        C = _gram(Q, W, dense)
        G = _gram(W, W, dense) - C.mH @ C
        A = A + C
        A = 0.5 * (A + A.mH)
        Qp.copy_(Q)
        R1, R1inv = _chol_factor(G)
        _update(W, 0.0, None, W, R1inv, Q, -(C @ R1inv), dense=dense)
        _, R2 = _cholqr(W, passes=1, dense=dense, out=Q)  # second pass
        B = R2 @ R1
    Bp.copy_(B)
    A_out.copy_(A)
    B_out.copy_(B)


def block_tridiagonal(A: List, B: List):
    """Assembles T [S, n k, n k] from A_0..A_{n-1} and B_0..B_{n-2} ([S, k, k] each)."""
    import torch

    n = len(A)
    S, k, _ = A[0].shape
    T = torch.zeros((S, n * k, n * k), dtype=A[0].dtype, device=A[0].device)
    for j in range(n):
        T[:, j * k:(j + 1) * k, j * k:(j + 1) * k] = A[j]
        if j + 1 < n:
            T[:, (j + 1) * k:(j + 2) * k, j * k:(j + 1) * k] = B[j]
            T[:, j * k:(j + 1) * k, (j + 1) * k:(j + 2) * k] = B[j].mH
    return T


def block_lanczos(apply: Callable[[], None], Q, W, steps: int, graph: bool = False,
                  timer: Optional[dict] = None, lean: bool = False, dense=None):
    """Runs `steps` block-Lanczos steps with W = H Q computed by `apply()`; Q must hold an
    orthonormal starting block.  Returns the eigenvalues of T per sector ([S, steps * k],
    ascending).  With graph=True one step is captured in a CUDA graph after a warm-up step
    (which is itself step 0) and replayed for the rest."""
    import torch

    S, D, k = Q.shape
    Qp = torch.zeros_like(Q)
    Bp = torch.zeros((S, k, k), dtype=Q.dtype, device=Q.device)
    A_cur = torch.zeros_like(Bp)
    B_cur = torch.zeros_like(Bp)
    A_hist, B_hist = [], []

    def record():
        A_hist.append(A_cur.clone())
        B_hist.append(B_cur.clone())

    use_graph = graph and Q.is_cuda
    g = None
    if use_graph:
        side = torch.cuda.Stream(Q.device)
        side.wait_stream(torch.cuda.current_stream(Q.device))
        with torch.cuda.stream(side):
            lanczos_step(apply, Q, W, Qp, Bp, A_cur, B_cur, lean, dense)  # step 0, also the warm-up
        torch.cuda.current_stream(Q.device).wait_stream(side)
        record()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            lanczos_step(apply, Q, W, Qp, Bp, A_cur, B_cur, lean, dense)
        # capture does not execute: step 1 runs at the first replay below
    start = end = None
    if timer is not None and Q.is_cuda:
        torch.cuda.synchronize(Q.device)
        start = torch.cuda.Event(enable_timing=True)
        end = torch.cuda.Event(enable_timing=True)
        start.record()
    j0 = len(A_hist)
    for _ in range(j0, steps):
        if g is not None:
            g.replay()
        else:
            lanczos_step(apply, Q, W, Qp, Bp, A_cur, B_cur, lean, dense)
        record()
    if start is not None:
        end.record()
        torch.cuda.synchronize(Q.device)
        timer["ms"] = start.elapsed_time(end)
        timer["steps"] = steps - j0
    T = block_tridiagonal(A_hist, B_hist)
    return torch.linalg.eigvalsh(T)


def random_start(batch, seed: int = 0, dense=None):
    """Fills batch.X with an orthonormal random block per sector (zero padding rows)."""
    import torch

    gen = torch.Generator(device="cpu").manual_seed(seed)
    for s in range(batch.number_sectors):
        d = batch.sizes[s]
        x = torch.randn((d, batch.k), dtype=torch.float64, generator=gen) + \
            1j * torch.randn((d, batch.k), dtype=torch.float64, generator=gen)
        batch.X[s].zero_()
        batch.X[s, :d].copy_(x.to(torch.complex128))
    Q, _ = _cholqr(batch.X, dense=dense)
    batch.X.copy_(Q)
    return batch.X


def sector_ground_states(batch, steps: int, seed: int = 0, graph: bool = True,
                         timer: Optional[dict] = None, lean: bool = False, dense=None) -> np.ndarray:
    """Lowest eigenvalue of every sector of a SectorBatch after `steps` block-Lanczos steps."""
    random_start(batch, seed, dense)
    ev = block_lanczos(lambda: batch.run(), batch.X, batch.Y, steps, graph=graph, timer=timer, lean=lean,
                       dense=dense)
    batch.check_errors()
    return ev[:, 0].cpu().numpy()


def ground_state(apply: Callable[[], None], Q, W, steps: int, graph: bool = False,
                 timer: Optional[dict] = None, dense=None):
    """Lowest eigenpair by block Lanczos with the Krylov blocks kept for the Ritz vector.

    Q, W: [1, D, k] blocks (Q orthonormal on entry), `apply()` computes W = H Q.  Returns
    (E0, psi0) with psi0 a unit vector [D] (complex128, on Q's device).  Memory: steps blocks of
    [D, k]."""
    import torch

    S, D, k = Q.shape
    if S != 1:
        raise ValueError("ground_state handles one sector")
    Qp = torch.zeros_like(Q)
    Bp = torch.zeros((S, k, k), dtype=Q.dtype, device=Q.device)
    A_cur = torch.zeros_like(Bp)
    B_cur = torch.zeros_like(Bp)
    A_hist, B_hist, blocks = [], [], []

    def step_and_record(run):
        blocks.append(Q[0].clone())
        run()
        A_hist.append(A_cur.clone())
        B_hist.append(B_cur.clone())

    def eager():
        lanczos_step(apply, Q, W, Qp, Bp, A_cur, B_cur, dense=dense)

    g = None
    if graph and Q.is_cuda:
        side = torch.cuda.Stream(Q.device)
        side.wait_stream(torch.cuda.current_stream(Q.device))
        with torch.cuda.stream(side):
            blocks.append(Q[0].clone())
            lanczos_step(apply, Q, W, Qp, Bp, A_cur, B_cur, dense=dense)
        torch.cuda.current_stream(Q.device).wait_stream(side)
        A_hist.append(A_cur.clone())
        B_hist.append(B_cur.clone())
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            lanczos_step(apply, Q, W, Qp, Bp, A_cur, B_cur, dense=dense)
    start = end = None
    if timer is not None and Q.is_cuda:
        torch.cuda.synchronize(Q.device)
        start = torch.cuda.Event(enable_timing=True)
        end = torch.cuda.Event(enable_timing=True)
        start.record()
    j0 = len(A_hist)
    for _ in range(j0, steps):
        step_and_record(g.replay if g is not None else eager)
    if start is not None:
        end.record()
        torch.cuda.synchronize(Q.device)
        timer["ms"] = start.elapsed_time(end)
        timer["steps"] = steps - j0
    T = block_tridiagonal(A_hist, B_hist)[0]
    evals, evecs = torch.linalg.eigh(T)
    y = evecs[:, 0].reshape(len(blocks), k)
    psi = torch.zeros(D, dtype=Q.dtype, device=Q.device)
    for j, blk in enumerate(blocks):
        psi += blk @ y[j]
    psi /= torch.linalg.vector_norm(psi)
    return float(evals[0].real), psi


def _energy_function():
    import torch

    class GroundStateEnergy(torch.autograd.Function):
        """E0(theta) of a ParametrizedOperator; backward by Hellmann-Feynman:
        dE0/dtheta_c = <psi0| H_c |psi0> (real for Hermitian H_c), from the fused coupling
        products or one matvec per coupling."""

        @staticmethod
        def forward(ctx, theta, pop, k, steps, seed, graph, dense):
            import numpy as np
            pop.set_theta(theta.detach().cpu().numpy())
            op = pop.operator
            D = op.basis.number_states
            dev = torch.device("cuda", torch.cuda.current_device())
            gen = torch.Generator(device="cpu").manual_seed(seed)
            Q = (torch.randn((1, D, k), generator=gen, dtype=torch.float64)
                 + 1j * torch.randn((1, D, k), generator=gen, dtype=torch.float64)).to(dev)
            Q, _ = _cholqr(Q, dense=dense)
            W = torch.empty_like(Q)
            Q = Q.contiguous()

            def apply():
                op.apply_device(Q[0], out=W[0], check=False)

            e0, psi = ground_state(apply, Q, W, steps, graph=graph, dense=dense)
            op.check_errors()
            ctx.pop = pop
            ctx.psi = psi
            ctx.save_for_backward(theta)
            return torch.tensor(e0, dtype=torch.float64)

        @staticmethod
        def backward(ctx, grad):
            (theta,) = ctx.saved_tensors
            hf = ctx.pop.coupling_products(ctx.psi, ctx.psi).real
            return ((grad.to(hf.device) * hf).to(dtype=theta.dtype, device=theta.device),
                    None, None, None, None, None, None)

    return GroundStateEnergy


_GSE = None


def ground_state_energy(pop, theta, k: int = 8, steps: int = 60, seed: int = 0, graph: bool = True,
                        dense=None):
    """E0(theta) of a ParametrizedOperator by k-RHS block Lanczos, differentiable in theta."""
    import torch

    global _GSE
    if _GSE is None:
        _GSE = _energy_function()
    if not isinstance(theta, torch.Tensor):
        theta = torch.as_tensor(theta, dtype=torch.float64)
    return _GSE.apply(theta, pop, k, steps, seed, graph, dense)
