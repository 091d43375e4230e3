"""Pins of the dense symmetry-adapted restatement (oracle/fermion_symmetry.py), on CPU.

* spins: it reproduces the C restatement of the reference (representatives, exact norms and
  the complex H*x of a momentum sector), which fixes its conventions;
* spinful fermions without symmetries: its H equals the C oracle's (pinned by the reference's
  Hubbard goldens) and gives the HPhi ground-state energy of test/04_hubbard_square;
* spinful fermions with lattice symmetries: the union of all momentum-sector spectra equals the
  unsymmetrised spectrum, which only holds with the fermionic permutation signs.
"""

import itertools

import numpy as np
import pytest

import fermion_symmetry as FS
from ls_helpers import LAT, Case, ls, oracle_terms


def elements_of(symmetries):
    re, im = symmetries.characters
    return FS.group_elements(symmetries.permutations, re, im)


def test_spin_sector_matches_c_oracle():
    n, k = 8, 1
    c = Case(ls.SpinBasis(n, n // 2, None, ls.Symmetries(LAT.chain_symmetries(n, k))),
             LAT.xxz(LAT.chain_bonds(n), 1.0, 0.7))
    states_ref = c.oracle_states()
    exact = c.oracle_norms_exact(states_ref)
    reps_c = states_ref[exact > 0]
    full = [s for s in range(1 << n) if bin(s).count("1") == n // 2]
    reps, norms, P = FS.symmetric_basis(full, elements_of(c.basis.symmetries), fermionic=False)
    assert np.array_equal(reps, reps_c)
    assert np.allclose(norms, exact[exact > 0], rtol=0, atol=1e-14)
    H = FS.hamiltonian(full, c.op._off_arrays) + FS.hamiltonian(full, c.op._diag_arrays)
    Hs = P.conj().T @ H @ P
    rng = np.random.default_rng(0)
    x = rng.normal(size=len(reps)) + 1j * rng.normal(size=len(reps))
    y = c.oracle_matvec(reps, x, complex_=True, exact_norms=True)
    assert np.linalg.norm(Hs @ x - y) <= 1e-12 * np.linalg.norm(y)


def hubbard_4x2(goldens):
    g = [h for h in goldens["hphi"] if h["name"] == "04_hubbard_square"][0]
    expr = None
    for t in g["terms"]:
        e = ls.Expr(t["expression"], sites=t["sites"])
        expr = e if expr is None else expr + e
    return expr, g["energy"]


def translations_4x2():
    tx = [4 * (i // 4) + (i % 4 + 1) % 4 for i in range(8)]
    ty = [(i + 4) % 8 for i in range(8)]
    return tx, ty


def test_fermion_hamiltonian_and_hphi_energy(goldens):
    expr, e_hphi = hubbard_4x2(goldens)
    basis = ls.SpinfulFermionBasis(8, (4, 4))
    c = Case(basis, expr)
    states = FS.fixed_occupation_states(8, 4, 4)
    H = FS.hamiltonian(states, c.op._off_arrays) + FS.hamiltonian(states, c.op._diag_arrays)
    assert np.abs(H - H.conj().T).max() < 1e-12
    rng = np.random.default_rng(1)
    x = rng.normal(size=len(states))
    y = c.oracle_matvec(np.array(states, dtype=np.uint64), x.astype(complex), complex_=True)
    assert np.linalg.norm(H @ x - y) <= 1e-12 * np.linalg.norm(y)
    e0 = np.linalg.eigvalsh(H.real)[0]
    assert abs(e0 - e_hphi) < 1e-9


def test_fermion_sector_spectra_union_equals_full_spectrum(goldens):
    expr, e_hphi = hubbard_4x2(goldens)
    states = FS.fixed_occupation_states(8, 4, 4)
    full = ls.SpinfulFermionBasis(8, (4, 4))
    cf = Case(full, expr)
    H = FS.hamiltonian(states, cf.op._off_arrays) + FS.hamiltonian(states, cf.op._diag_arrays)
    ref = np.linalg.eigvalsh(H.real)
    tx, ty = translations_4x2()
    spectra = []
    for kx, ky in itertools.product(range(4), range(2)):
        syms = ls.Symmetries([ls.Symmetry(tx, kx), ls.Symmetry(ty, ky)])
        b = ls.SpinfulFermionBasis(8, (4, 4), symmetries=syms)
        reps, norms, P = FS.symmetric_basis(states, elements_of(b.symmetries), fermionic=True)
        Hs = P.conj().T @ H @ P
        assert np.abs(Hs - Hs.conj().T).max() < 1e-12
        spectra.append(np.linalg.eigvalsh(Hs))
    union = np.sort(np.concatenate(spectra))
    assert union.shape == ref.shape
    assert np.abs(union - ref).max() < 1e-9
    assert abs(union[0] - e_hphi) < 1e-9
