"""Host logic of the block-Lanczos driver on CPU tensors (dense Hermitian test matrices)."""

import importlib

import numpy as np
import pytest

torch = pytest.importorskip("torch")
lanczos = importlib.import_module("lattice-symmetries_gb300.lanczos")


def random_hermitian(S, D, seed):
    g = torch.Generator().manual_seed(seed)
    a = torch.randn((S, D, D), generator=g, dtype=torch.float64) + 1j * torch.randn((S, D, D), generator=g,
                                                                                   dtype=torch.float64)
    return (a + a.mH) / 2


def test_cholqr_orthonormal_and_exact():
    g = torch.Generator().manual_seed(0)
    W = (torch.randn((3, 50, 6), generator=g, dtype=torch.float64) + 0j).to(torch.complex128)
    Q, R = lanczos._cholqr(W)
    eye = torch.eye(6, dtype=torch.complex128)
    assert float((Q.mH @ Q - eye).abs().max()) < 1e-13
    assert float((Q @ R - W).abs().max()) < 1e-12 * float(W.abs().max())
    assert float(torch.tril(R, -1).abs().max()) == 0.0


def test_block_tridiagonal_layout():
    A = [torch.full((1, 2, 2), float(j), dtype=torch.complex128) for j in range(3)]
    B = [torch.full((1, 2, 2), 10.0 + j, dtype=torch.complex128) + 1j for j in range(2)]
    T = lanczos.block_tridiagonal(A, B)
    assert T.shape == (1, 6, 6)
    assert complex(T[0, 2, 0]) == 10 + 1j and complex(T[0, 0, 2]) == 10 - 1j
    assert complex(T[0, 4, 3]) == 11 + 1j and complex(T[0, 5, 0]) == 0


@pytest.mark.parametrize("S,D,k", [(3, 40, 4), (2, 33, 3)])
def test_block_lanczos_reaches_extremal_eigenvalues(S, D, k):
    H = random_hermitian(S, D, seed=S * 100 + D)
    g = torch.Generator().manual_seed(7)
    Q = torch.randn((S, D, k), generator=g, dtype=torch.float64).to(torch.complex128)
    Q, _ = lanczos._cholqr(Q)
    W = torch.empty_like(Q)
    steps = (D + k - 1) // k + 2
    ev = lanczos.block_lanczos(lambda: W.copy_(H @ Q), Q, W, steps)
    ref = torch.linalg.eigvalsh(H)
    assert float((ev[:, 0] - ref[:, 0]).abs().max()) < 1e-9
    assert float((ev[:, -1] - ref[:, -1]).abs().max()) < 1e-9


def test_block_lanczos_padded_sectors_are_independent():
    # two sectors of different size padded into one [S, D, k] block: padding rows stay zero
    D = 30
    H = random_hermitian(2, D, seed=5)
    H[1, 20:, :] = 0
    H[1, :, 20:] = 0
    g = torch.Generator().manual_seed(3)
    Q = torch.randn((2, D, 2), generator=g, dtype=torch.float64).to(torch.complex128)
    Q[1, 20:] = 0
    Q, _ = lanczos._cholqr(Q)
    W = torch.empty_like(Q)
    ev = lanczos.block_lanczos(lambda: W.copy_(H @ Q), Q, W, 12)
    assert float(Q[1, 20:].abs().max()) == 0.0
    ref1 = np.linalg.eigvalsh(H[1, :20, :20].numpy())
    assert abs(float(ev[1, 0]) - ref1[0]) < 1e-9


def test_ground_state_ritz_vector():
    D, k = 50, 3
    H = random_hermitian(1, D, seed=11)
    g = torch.Generator().manual_seed(2)
    Q = torch.randn((1, D, k), generator=g, dtype=torch.float64).to(torch.complex128)
    Q, _ = lanczos._cholqr(Q)
    W = torch.empty_like(Q)
    e0, psi = lanczos.ground_state(lambda: W.copy_(H @ Q), Q, W, steps=20)
    ref = torch.linalg.eigvalsh(H)[0, 0]
    assert abs(e0 - float(ref)) < 1e-9
    r = H[0] @ psi - e0 * psi
    assert float(torch.linalg.vector_norm(r)) < 1e-6


def test_lean_steps_reach_the_same_extremal_eigenvalues():
    H = random_hermitian(2, 60, seed=21)
    ref = torch.linalg.eigvalsh(H)
    for lean in (False, True):
        g = torch.Generator().manual_seed(9)
        Q = torch.randn((2, 60, 4), generator=g, dtype=torch.float64).to(torch.complex128)
        Q, _ = lanczos._cholqr(Q)
        W = torch.empty_like(Q)
        ev = lanczos.block_lanczos(lambda: W.copy_(H @ Q), Q, W, 14, lean=lean)
        assert float((ev[:, 0] - ref[:, 0]).abs().max()) < 1e-8


def test_dense_mode_validation_and_update_forms():
    """CPU tensors take the torch path in every mode; an unknown mode is an error; _update's
    in-place and aliasing forms agree with the plain expression."""
    g = torch.Generator().manual_seed(5)
    S, D, k = 2, 30, 4
    W = (torch.randn((S, D, k), generator=g, dtype=torch.float64) + 0j).to(torch.complex128)
    X = torch.randn((S, D, k), generator=g, dtype=torch.complex128)
    M = torch.randn((S, k, k), generator=g, dtype=torch.complex128)
    with pytest.raises(ValueError):
        lanczos._gram(W, W, dense="fp32")
    for mode in (None, "paired", "fp64"):
        assert torch.allclose(lanczos._gram(W, X, dense=mode), W.mH @ X)
    ref = W + X @ M
    out = W.clone()
    lanczos._update(out, 1.0, out, X, M, dense="paired")
    assert torch.allclose(out, ref)
    out = X.clone()
    lanczos._update(out, 0.0, None, out, M)  # out aliases X1
    assert torch.allclose(out, X @ M)
    out = torch.empty_like(W)
    lanczos._update(out, -0.5, W, X, M, X, M)
    assert torch.allclose(out, -0.5 * W + 2 * (X @ M))
