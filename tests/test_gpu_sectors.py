"""Batched multi-sector matvec (SectorBatch / ls_gpu_sector_plan_*) and the block-Lanczos driver
on the GPU.

The batched kernel must reproduce the single-sector matvec (itself checked against the oracle in
test_gpu_parity.py) sector by sector; the union of the sector spectra it produces must equal the
spectrum of the unsymmetrised Hamiltonian (complex characters: the reference truncates these, so
the sum-over-sectors identity is the pin); block Lanczos must find every sector's ground state.
"""

import importlib

import numpy as np
import pytest

from ls_helpers import LAT, ls

pytestmark = pytest.mark.gpu
lanczos = importlib.import_module("lattice-symmetries_gb300.lanczos")


def xxz_sector_ops(n, delta=1.5, inversions=(1, -1), momenta=None, exact=False):
    ops = []
    expr = LAT.xxz(LAT.chain_bonds(n), 1.0, delta)
    for k in (range(n) if momenta is None else momenta):
        for z in inversions:
            basis = ls.SpinBasis(n, n // 2, z, ls.Symmetries(LAT.chain_symmetries(n, k)))
            basis.build(exact_norms=exact)
            if basis.number_states == 0:
                continue
            ops.append(ls.Operator(basis, expr))
    return ops


def fill_random(batch, seed):
    import torch
    g = torch.Generator(device="cpu").manual_seed(seed)
    batch.X.zero_()
    for s in range(batch.number_sectors):
        d = batch.sizes[s]
        x = torch.randn((d, batch.k), generator=g, dtype=torch.float64) + \
            1j * torch.randn((d, batch.k), generator=g, dtype=torch.float64)
        batch.X[s, :d].copy_(x)


def assert_matches_single(batch, ops, adjoint=False):
    for s, op in enumerate(ops):
        ref = op.apply_device(batch.x(s).contiguous(), adjoint=adjoint)
        got = batch.y(s)
        err = float((got - ref).abs().max())
        scale = float(ref.abs().max()) + 1e-300
        assert err <= 1e-13 * scale, (s, err, scale)


@pytest.mark.parametrize("k", [1, 4, 5, 16])
def test_batched_equals_single_sector(k):
    ops = xxz_sector_ops(16)
    batch = ls.SectorBatch(ops, k=k)
    assert batch.batched
    fill_random(batch, 10 + k)
    batch.run(check=True)
    assert_matches_single(batch, ops)
    # padding rows stay zero
    for s in range(batch.number_sectors):
        assert float(batch.Y[s, batch.sizes[s]:].abs().sum()) == 0.0


def test_batched_adjoint_and_graph_replay():
    import torch
    ops = xxz_sector_ops(14, delta=0.7)
    batch = ls.SectorBatch(ops, k=8, adjoint=True)
    assert batch.batched
    fill_random(batch, 3)
    batch.run(check=True)
    assert_matches_single(batch, ops, adjoint=True)
    first = batch.Y.clone()
    batch.capture()
    batch.Y.zero_()
    batch.replay()
    torch.cuda.synchronize()
    assert torch.equal(batch.Y, first)
    fill_random(batch, 4)  # a graph replays on the batch's own buffers: new inputs, new outputs
    batch.replay()
    torch.cuda.synchronize()
    assert_matches_single(batch, ops, adjoint=True)


def test_unshareable_sectors_fall_back_to_per_sector_launches():
    n = 12
    ops = []
    for k, J in [(0, 1.0), (3, 0.5), (6, 2.0)]:
        basis = ls.SpinBasis(n, n // 2, None, ls.Symmetries(LAT.chain_symmetries(n, k)))
        basis.build()
        ops.append(ls.Operator(basis, LAT.heisenberg(LAT.chain_bonds(n), J)))
    batch = ls.SectorBatch(ops, k=4)
    assert not batch.batched
    fill_random(batch, 5)
    batch.run(check=True)
    assert_matches_single(batch, ops)


def test_union_of_sector_spectra_equals_full_spectrum():
    import torch
    n, delta = 12, 1.5
    ops = xxz_sector_ops(n, delta, exact=True)
    dmax = max(op.basis.number_states for op in ops)
    batch = ls.SectorBatch(ops, k=16)
    dense = [np.zeros((op.basis.number_states,) * 2, dtype=complex) for op in ops]
    for c0 in range(0, dmax, 16):  # H applied to identity columns, 16 at a time, all sectors at once
        batch.X.zero_()
        for s, op in enumerate(ops):
            d = op.basis.number_states
            for c in range(c0, min(c0 + 16, d)):
                batch.X[s, c, c - c0] = 1.0
        batch.run(check=True)
        for s, op in enumerate(ops):
            d = op.basis.number_states
            m = min(c0 + 16, d) - c0
            if m > 0:
                dense[s][:, c0:c0 + m] = batch.y(s)[:, :m].cpu().numpy()
    spectra = []
    for h in dense:
        assert np.abs(h - h.conj().T).max() < 1e-12
        spectra.append(np.linalg.eigvalsh(h))
    union = np.sort(np.concatenate(spectra))
    full = ls.SpinBasis(n, n // 2)
    full.build()
    op = ls.Operator(full, LAT.xxz(LAT.chain_bonds(n), 1.0, delta))
    eye = torch.eye(full.number_states, dtype=torch.complex128, device="cuda")
    hf = op.apply_device(eye).cpu().numpy()
    ref = np.linalg.eigvalsh(hf)
    assert union.shape == ref.shape
    assert np.abs(union - ref).max() < 1e-10


def test_block_lanczos_finds_sector_ground_states():
    import torch
    n = 16
    ops = xxz_sector_ops(n, 1.5, momenta=[0, 1, 5, 8], exact=True)
    batch = ls.SectorBatch(ops, k=4)
    timer = {}
    e0 = lanczos.sector_ground_states(batch, steps=40, seed=1, graph=True, timer=timer)
    assert timer["steps"] == 39
    for s, op in enumerate(ops):
        d = op.basis.number_states
        eye = torch.eye(d, dtype=torch.complex128, device="cuda")
        h = op.apply_device(eye).cpu().numpy()
        ref = np.linalg.eigvalsh(h)[0]
        assert abs(e0[s] - ref) < 1e-8 * max(1.0, abs(ref)), (s, e0[s], ref)


def test_zero_norm_states_are_zero_rows_and_columns(oracle):
    """N = 16, k = 1, z = -1: the reference's floating rule keeps four representatives whose
    exact norm is zero.  They must be zero rows and columns, and the rest of H must equal H on the
    exact-rule basis (and the oracle)."""
    import torch
    from ls_helpers import Case
    n = 16
    expr = LAT.xxz(LAT.chain_bonds(n), 1.0, 1.5)
    bref = ls.SpinBasis(n, n // 2, -1, ls.Symmetries(LAT.chain_symmetries(n, 1)))
    bref.build()
    bex = ls.SpinBasis(n, n // 2, -1, ls.Symmetries(LAT.chain_symmetries(n, 1)))
    bex.build(exact_norms=True)
    ref_states, ex_states = np.asarray(bref.states), np.asarray(bex.states)
    case = Case(bref, expr)
    norms = case.oracle_norms_exact(ref_states)
    noise = norms == 0
    assert noise.sum() == 4
    assert np.array_equal(ref_states[~noise], ex_states)
    rng = np.random.default_rng(0)
    x = rng.normal(size=len(ref_states)) + 1j * rng.normal(size=len(ref_states))
    y_ref = ls.Operator(bref, expr).apply_device(torch.from_numpy(x).cuda()).cpu().numpy()
    assert np.all(y_ref[noise] == 0)
    y_ex = ls.Operator(bex, expr).apply_device(torch.from_numpy(x[~noise]).cuda()).cpu().numpy()
    assert np.abs(y_ref[~noise] - y_ex).max() <= 1e-13 * np.abs(y_ex).max()
    y_or = case.oracle_matvec(ref_states, x, complex_=True, exact_norms=True)
    assert np.linalg.norm(y_ref - y_or) <= 1e-12 * np.linalg.norm(y_or)


def test_first_matvec_on_a_fresh_basis_sees_its_norms():
    """The orbit norms of a basis are computed lazily by its first matvec; that first product,
    enqueued on the caller's stream, must already see them (one vector, fresh bases in turn)."""
    import torch
    from ls_helpers import Case
    n = 16
    expr = LAT.xxz(LAT.chain_bonds(n), 1.0, 1.5)
    for k, z in [(1, -1), (3, 1), (5, -1)]:
        b = ls.SpinBasis(n, n // 2, z, ls.Symmetries(LAT.chain_symmetries(n, k)))
        b.build(exact_norms=True)
        st = np.asarray(b.states)
        x = np.random.default_rng(k).normal(size=len(st)) + 0.5j
        y = ls.Operator(b, expr).apply_device(torch.from_numpy(x).cuda()).cpu().numpy()
        yo = Case(b, expr).oracle_matvec(st, x, complex_=True, exact_norms=True)
        assert np.linalg.norm(y - yo) <= 1e-12 * np.linalg.norm(yo)


def test_plan_forms_and_autotune():
    """Both forms of a plan (one launch over all sectors, one launch per sector) give the same
    result; the autotuner times both and keeps one; a plan that cannot batch refuses the form."""
    import torch
    ops = xxz_sector_ops(16)
    batch = ls.SectorBatch(ops, k=16)
    assert batch.batched
    fill_random(batch, 21)
    y1 = batch.run(check=True).clone()
    batch.set_batched(False)
    assert not batch.batched
    y2 = batch.run(check=True).clone()
    assert float((y1 - y2).abs().max()) <= 1e-14 * float(y1.abs().max())
    t = batch.autotune()
    assert t["ms_batched"] > 0 and t["ms_per_sector"] > 0
    assert batch.batched == t["batched"]
    y3 = batch.replay().clone()
    torch.cuda.synchronize()
    assert float((y3 - y1).abs().max()) <= 1e-14 * float(y1.abs().max())
