"""Gradients of y = H(theta) x on the GPU: the fused per-coupling inner products, the adjoint
matvec behind dL/dx, central finite differences (h = 1e-6) and torch.autograd.gradcheck.

Workload family of the differentiation benchmark: spin-1/2 ladder with leg, rung and
Dzyaloshinskii-Moriya couplings (imaginary sigma+ sigma- coefficients, a non-real matrix),
leg translations x leg exchange."""

import importlib

import numpy as np
import pytest

from ls_helpers import LAT, Case, ls, oracle_terms

pytestmark = pytest.mark.gpu
ag = importlib.import_module("lattice-symmetries_gb300.autograd")
THETA = [1.0, 0.7, 0.2]


def ladder_parts(n_rungs):
    legs, rungs = LAT.ladder(n_rungs)
    return [LAT.heisenberg(legs, 0.25), LAT.heisenberg(rungs, 0.25), LAT.dm_z(legs, 1.0)]


def ladder_pop(n_rungs, k=0, exchange=0, symmetric=True):
    syms = ls.Symmetries(LAT.ladder_symmetries(n_rungs, k, exchange)) if symmetric else None
    basis = ls.SpinBasis(2 * n_rungs, n_rungs, None, syms)
    basis.build()
    return ag.ParametrizedOperator(basis, ladder_parts(n_rungs), theta=THETA)


def rand(D, seed, k=None):
    import torch
    rng = np.random.default_rng(seed)
    shape = (D,) if k is None else (D, k)
    return torch.from_numpy(rng.normal(size=shape) + 1j * rng.normal(size=shape)).cuda()


@pytest.mark.parametrize("n_rungs,k,exchange", [(8, 0, 0), (8, 3, 1), (10, 5, 0)])
def test_fused_coupling_products_match_per_coupling_matvecs_and_oracle(n_rungs, k, exchange):
    pop = ladder_pop(n_rungs, k, exchange)
    D = pop.basis.number_states
    g, x = rand(D, 1), rand(D, 2)
    fused = pop.coupling_products(g, x, fused=True).cpu().numpy()
    split = pop.coupling_products(g, x, fused=False).cpu().numpy()
    assert np.abs(fused - split).max() <= 1e-12 * np.abs(split).max()
    # oracle: per-coupling scatter matvecs assembled on the CPU
    states = np.asarray(pop.basis.states)
    gn, xn = g.cpu().numpy(), x.cpu().numpy()
    for c, sub in enumerate(pop._sub_operators()):
        case = Case(pop.basis, ladder_parts(n_rungs)[c])
        case.off, case.diag = oracle_terms(sub)
        yc = case.oracle_matvec(states, xn, complex_=True)
        ref = np.vdot(gn, yc)
        assert abs(fused[c] - ref) <= 1e-12 * max(1.0, abs(ref)), (c, fused[c], ref)


def test_backward_matches_finite_differences_and_adjoint():
    import torch
    pop = ladder_pop(8, 2, 0)
    D = pop.basis.number_states
    v, x0 = rand(D, 3), rand(D, 4)
    theta = torch.tensor(THETA, dtype=torch.float64, requires_grad=True)
    x = x0.clone().requires_grad_(True)
    loss = torch.real(torch.vdot(v, pop.apply(theta, x)))
    loss.backward()
    # dL/dtheta_c = Re <v, H_c x>
    exact = pop.coupling_products(v, x0, fused=False).real.cpu().numpy()
    assert np.abs(theta.grad.numpy() - exact).max() <= 1e-12 * np.abs(exact).max()
    # central finite differences, h = 1e-6
    h = 1e-6
    fd = []
    for c in range(3):
        tp, tm = np.array(THETA), np.array(THETA)
        tp[c] += h
        tm[c] -= h
        lp = float(torch.real(torch.vdot(v, pop.apply(torch.tensor(tp), x0))))
        lm = float(torch.real(torch.vdot(v, pop.apply(torch.tensor(tm), x0))))
        fd.append((lp - lm) / (2 * h))
    assert np.abs(theta.grad.numpy() - np.array(fd)).max() <= 1e-6 * max(1.0, np.abs(fd).max())
    # dL/dx = H(theta)^dagger v
    pop.set_theta(THETA)
    hv = pop.operator.apply_device(v, adjoint=True)
    assert float((x.grad - hv).abs().max()) <= 1e-12 * float(hv.abs().max())


def test_gradcheck_small_ladder():
    import torch
    pop = ladder_pop(4, 1, 0)
    D = pop.basis.number_states
    theta = torch.tensor(THETA, dtype=torch.float64, requires_grad=True)
    x = rand(D, 5).requires_grad_(True)
    assert torch.autograd.gradcheck(lambda t, y: pop.apply(t, y), (theta, x), eps=1e-6, atol=1e-8, rtol=1e-6)


def test_block_inputs_and_unprojected_fallback():
    import torch
    pop = ladder_pop(6, 0, 0, symmetric=False)  # no lattice symmetries: per-coupling path
    D = pop.basis.number_states
    g, x = rand(D, 6, k=3), rand(D, 7, k=3)
    out = pop.coupling_products(g, x).cpu().numpy()
    ref = np.zeros(3, dtype=complex)
    for c, sub in enumerate(pop._sub_operators()):
        ref[c] = np.vdot(g.cpu().numpy(), sub.apply_device(x).cpu().numpy())
    assert np.abs(out - ref).max() <= 1e-12 * np.abs(ref).max()
    theta = torch.tensor(THETA, dtype=torch.float64, requires_grad=True)
    loss = torch.real(torch.sum(g.conj() * pop.apply(theta, x)))
    loss.backward()
    assert np.abs(theta.grad.numpy() - out.real).max() <= 1e-12 * np.abs(out.real).max()
