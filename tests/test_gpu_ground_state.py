"""Ground state of a symmetric Hubbard sector by 8-RHS block Lanczos (CUDA graph) and dE0/d(t, U)
by Hellmann-Feynman through autograd, against dense diagonalisation and finite differences."""

import importlib

import numpy as np
import pytest

from ls_helpers import LAT, ls

pytestmark = pytest.mark.gpu
ag = importlib.import_module("lattice-symmetries_gb300.autograd")
lanczos = importlib.import_module("lattice-symmetries_gb300.lanczos")


def dense_e0(pop, theta):
    import torch
    pop.set_theta(theta)
    D = pop.basis.number_states
    h = pop.operator.apply_device(torch.eye(D, dtype=torch.complex128, device="cuda")).cpu().numpy()
    return np.linalg.eigvalsh(h)[0]


def test_hubbard_ground_state_energy_and_gradient():
    import torch
    L = 3
    syms = ls.Symmetries(LAT.square_symmetries(L, 0, 0, True))
    basis = ls.SpinfulFermionBasis(L * L, (3, 3), symmetries=syms)
    basis.build()
    pop = ag.ParametrizedOperator(basis, list(LAT.hubbard_parts(LAT.square_bonds(L), L * L)), theta=[1.0, 4.0])
    theta = torch.tensor([1.0, 4.0], dtype=torch.float64, requires_grad=True)
    e0 = lanczos.ground_state_energy(pop, theta, k=8, steps=25, seed=3, graph=True)
    ref = dense_e0(pop, [1.0, 4.0])
    assert abs(e0.item() - ref) < 1e-9
    e0.backward()
    h = 1e-5
    fd = []
    for c in range(2):
        tp, tm = np.array([1.0, 4.0]), np.array([1.0, 4.0])
        tp[c] += h
        tm[c] -= h
        fd.append((dense_e0(pop, tp) - dense_e0(pop, tm)) / (2 * h))
    assert np.abs(theta.grad.numpy() - np.array(fd)).max() < 1e-6, (theta.grad, fd)
    # Hellmann-Feynman identity: E0 = t dE/dt + U dE/dU (H is linear in theta)
    assert abs(float(theta.grad @ theta.detach()) - ref) < 1e-8
