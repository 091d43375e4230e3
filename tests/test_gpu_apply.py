"""Per-state term application on device batches (ls_gpu_operator_apply_{diag,off_diag}) against the
host functions with the reference's semantics (ls_internal_operator_apply_*_x1, themselves
compared with the compiled reference.c in test_abi.py): identical targets, order and offsets."""

import ctypes

import numpy as np
import pytest

from ls_helpers import LAT, ls

pytestmark = pytest.mark.gpu


def host_apply(op, alphas):
    lib = ls._native.lib()
    B = len(alphas)
    T = op.number_off_diag_terms
    a = np.ascontiguousarray(alphas, dtype=np.uint64)
    betas = np.zeros(max(B * T, 1), dtype=np.uint64)
    coeffs = np.zeros(max(B * T, 1), dtype=np.complex128)
    offsets = np.zeros(B + 1, dtype=np.int64)
    P = ctypes.POINTER
    lib.ls_internal_operator_apply_off_diag_x1(
        op._payload, B, a.ctypes.data_as(P(ctypes.c_uint64)), betas.ctypes.data_as(P(ctypes.c_uint64)),
        coeffs.ctypes.data_as(P(ctypes.c_double)), offsets.ctypes.data_as(P(ctypes.c_ssize_t)), None)
    ys = np.zeros(B, dtype=np.float64)
    lib.ls_internal_operator_apply_diag_x1(op._payload, B, a.ctypes.data_as(P(ctypes.c_uint64)),
                                           ys.ctypes.data_as(P(ctypes.c_double)), None)
    n = offsets[-1]
    return betas[:n], coeffs[:n], offsets, ys


@pytest.mark.parametrize("kind", ["spin", "fermion", "dm"])
def test_device_apply_matches_host(kind):
    import torch
    rng = np.random.default_rng(4)
    if kind == "spin":
        basis = ls.SpinBasis(20)
        expr = LAT.xxz(LAT.chain_bonds(20), 1.0, 0.3)
        alphas = rng.integers(0, 1 << 20, size=5000, dtype=np.uint64)
    elif kind == "dm":
        legs, rungs = LAT.ladder(8)
        basis = ls.SpinBasis(16)
        expr = LAT.heisenberg(legs + rungs) + LAT.dm_z(legs, 0.4)
        alphas = rng.integers(0, 1 << 16, size=3000, dtype=np.uint64)
    else:
        basis = ls.SpinfulFermionBasis(9)
        expr = LAT.hubbard(LAT.square_bonds(3), 1.0, 4.0, number_sites=9)
        alphas = rng.integers(0, 1 << 18, size=4000, dtype=np.uint64)
    op = ls.Operator(basis, expr)
    hb, hc, ho, hy = host_apply(op, alphas)
    d = torch.from_numpy(alphas.view(np.int64)).cuda()
    b, c, o = op.apply_off_diag_batch(d)
    y = op.apply_diag_batch(d)
    torch.cuda.synchronize()
    assert np.array_equal(o.cpu().numpy(), ho)
    assert np.array_equal(b.cpu().numpy().view(np.uint64), hb)
    assert np.array_equal(c.cpu().numpy(), hc)
    assert np.array_equal(y.cpu().numpy(), hy)


def test_empty_batch():
    import torch
    op = ls.Operator(ls.SpinBasis(8), LAT.heisenberg(LAT.chain_bonds(8)))
    b, c, o = op.apply_off_diag_batch(torch.zeros(0, dtype=torch.int64, device="cuda"))
    assert o.shape == (1,) and int(o[0]) == 0 and b.numel() == 0


@pytest.mark.parametrize("k", [2, 3, 5, 16])
def test_reference_call_with_several_vectors(k):
    """ls_chpl_matrix_vector_product with num_vectors = k equals k one-vector calls."""
    from ls_helpers import chain_case, square_case
    for case in (chain_case(16, 0, 0, 1), chain_case(16, 3), square_case(4, 2, 2, 1, J2=0.5)):
        case.basis.build()
        D = case.basis.number_states
        X = np.random.default_rng(k).normal(size=(k, D))
        Y = case.op.apply_to_state_vectors(X)
        ref = np.stack([case.op.apply_to_state_vector(X[v].copy()) for v in range(k)])
        assert np.abs(Y - ref).max() <= 1e-13 * np.abs(ref).max()
