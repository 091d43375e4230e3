"""Spinful fermions with lattice symmetries on the GPU (no reference counterpart: its fermionic
bases have no symmetries, Basis.hs:713-723).  The oracle is the dense restatement
oracle/fermion_symmetry.py, itself pinned by test_fermion_oracle.py (union of sector spectra =
unsymmetrised spectrum, HPhi ground-state energy of test/04_hubbard_square)."""

import ctypes
import itertools

import numpy as np
import pytest

import fermion_symmetry as FS
from ls_helpers import LAT, ls

pytestmark = pytest.mark.gpu


def elements_of(symmetries):
    re, im = symmetries.characters
    return FS.group_elements(symmetries.permutations, re, im)


def hubbard_4x2(goldens):
    g = [h for h in goldens["hphi"] if h["name"] == "04_hubbard_square"][0]
    expr = None
    for t in g["terms"]:
        e = ls.Expr(t["expression"], sites=t["sites"])
        expr = e if expr is None else expr + e
    return expr, g["energy"]


def sparse_h(states, op):
    import scipy.sparse as sp
    index = {int(a): i for i, a in enumerate(states)}
    rows, cols, vals = [], [], []
    for arrays in (op._off_arrays, op._diag_arrays):
        v, m, l, r, x, s = arrays
        for j, a in enumerate(states):
            for t in range(len(v)):
                if (a & int(m[t])) != int(r[t]):
                    continue
                sign = -1.0 if bin(a & int(s[t])).count("1") & 1 else 1.0
                rows.append(index[a ^ int(x[t])])
                cols.append(j)
                vals.append(v[t] * sign)
    D = len(states)
    return sp.csr_matrix((vals, (rows, cols)), shape=(D, D))


def check_sector(basis, expr, states_full, H, seed):
    import torch
    basis.build()
    reps, norms, P = FS.symmetric_basis(states_full, elements_of(basis.symmetries), fermionic=True)
    got = np.asarray(basis.states)
    assert np.array_equal(got, reps)
    if len(reps) == 0:
        return None
    dn = torch.as_tensor(basis.device_norms(), device="cuda").cpu().numpy()
    assert np.abs(dn - norms).max() < 1e-14
    op = ls.Operator(basis, expr)
    rng = np.random.default_rng(seed)
    x = rng.normal(size=len(reps)) + 1j * rng.normal(size=len(reps))
    y = op.apply_device(torch.from_numpy(x).cuda()).cpu().numpy()
    ref = P.conj().T @ (H @ (P @ x))
    assert np.linalg.norm(y - ref) <= 1e-12 * np.linalg.norm(ref)
    # block of right-hand sides (the 8-RHS kernel) and the adjoint
    X = rng.normal(size=(len(reps), 8)) + 1j * rng.normal(size=(len(reps), 8))
    Y = op.apply_device(torch.from_numpy(X).cuda()).cpu().numpy()
    REF = P.conj().T @ (H @ (P @ X))
    assert np.linalg.norm(Y - REF) <= 1e-12 * np.linalg.norm(REF)
    Ya = op.apply_device(torch.from_numpy(x).cuda(), adjoint=True).cpu().numpy()
    refa = P.conj().T @ (H.conj().T @ (P @ x))
    assert np.linalg.norm(Ya - refa) <= 1e-12 * np.linalg.norm(refa)
    return op


def test_hubbard_4x2_all_momentum_sectors(goldens):
    import torch
    expr, e_hphi = hubbard_4x2(goldens)
    states = FS.fixed_occupation_states(8, 4, 4)
    full = ls.SpinfulFermionBasis(8, (4, 4))
    H = sparse_h(states, ls.Operator(full, expr))
    tx = [4 * (i // 4) + (i % 4 + 1) % 4 for i in range(8)]
    ty = [(i + 4) % 8 for i in range(8)]
    e0 = []
    for kx, ky in itertools.product(range(4), range(2)):
        b = ls.SpinfulFermionBasis(8, (4, 4), symmetries=ls.Symmetries([ls.Symmetry(tx, kx), ls.Symmetry(ty, ky)]))
        op = check_sector(b, expr, states, H, seed=10 * kx + ky)
        D = b.number_states
        h = op.apply_device(torch.eye(D, dtype=torch.complex128, device="cuda")).cpu().numpy()
        assert np.abs(h - h.conj().T).max() < 1e-12
        e0.append(np.linalg.eigvalsh(h)[0])
    assert abs(min(e0) - e_hphi) < 1e-9


@pytest.mark.parametrize("kx,ky,point_group", [(0, 0, True), (1, 2, False)])
def test_hubbard_3x3_with_point_group(kx, ky, point_group):
    L = 3
    syms = ls.Symmetries(LAT.square_symmetries(L, kx, ky, point_group))
    expr = LAT.hubbard(LAT.square_bonds(L), t=1.0, U=4.0, number_sites=L * L)
    states = FS.fixed_occupation_states(L * L, 3, 3)
    H = sparse_h(states, ls.Operator(ls.SpinfulFermionBasis(L * L, (3, 3)), expr))
    b = ls.SpinfulFermionBasis(L * L, (3, 3), symmetries=syms)
    check_sector(b, expr, states, H, seed=7)


def test_fermionic_noalloc_enumeration_and_state_info():
    import torch
    L = 3
    syms = ls.Symmetries(LAT.square_symmetries(L, 0, 0, True))
    b = ls.SpinfulFermionBasis(L * L, (3, 2), symmetries=syms)
    b.build()
    n = b.number_states
    lib = ls._native.lib()
    out = torch.zeros(n, dtype=torch.int64, device="cuda")
    count = ctypes.c_int64(0)
    rc = lib.ls_gpu_enumerate_noalloc(b._payload, out.data_ptr(), n, ctypes.byref(count),
                                      torch.cuda.current_stream().cuda_stream)
    assert rc == 0 and count.value == n
    assert np.array_equal(out.cpu().numpy().view(np.uint64), np.asarray(b.states))
    # state_info of arbitrary states: representative and character x fermionic sign
    states = np.array(FS.fixed_occupation_states(L * L, 3, 2), dtype=np.uint64)
    reps, chars, norms = b.state_info(states)
    els = elements_of(b.symmetries)
    rep_set = set(int(r) for r in np.asarray(b.states))
    for a, r, ch in list(zip(states, reps, chars))[::7]:
        a = int(a)
        images = [(FS.apply_perm(p, a), c * FS.fermion_sign(p, a)) for p, c in els]
        rmin = min(i for i, _ in images)
        assert int(r) == rmin
        if rmin in rep_set:  # orbits with a nonzero norm: every minimising element agrees
            vals = {complex(round(c.real, 12), round(c.imag, 12)) for i, c in images if i == rmin}
            assert len(vals) == 1
            assert abs(ch - vals.pop()) < 1e-12
