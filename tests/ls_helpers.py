"""Shared builders for the tests: the product objects and the matching oracle inputs."""

from __future__ import annotations

import importlib

import numpy as np

import oracle as O

ls = importlib.import_module("lattice-symmetries_gb300")
E = importlib.import_module("lattice-symmetries_gb300._expr")
LAT = importlib.import_module("lattice-symmetries_gb300.lattices")


def oracle_group(symmetries, spin_inversion):
    """Oracle group from the independent closure, with the product's Benes masks for the
    baseline path."""
    gens = [(s.permutation, s.sector) for s in symmetries.generators]
    el = O.close_group(gens)
    re, im = O.characters(el)
    masks, shifts = symmetries.network()
    perms = np.array([e[0] for e in el], dtype=np.int32)
    return O.Group(perms, re, im, spin_inversion, symmetries.number_bits, masks, shifts)


def oracle_terms(op):
    return O.Terms(*op._off_arrays), O.Terms(*op._diag_arrays)


class Case:
    """A basis + operator pair with its oracle twin."""

    def __init__(self, basis, expr, name=""):
        self.name = name
        self.basis = basis
        self.expr = expr
        self.op = ls.Operator(basis, expr)
        self.inv = basis._c.spin_inversion
        self.nbits = basis.number_bits
        if basis.has_permutation_symmetries:
            self.group = oracle_group(basis.symmetries, self.inv)
            self.projection = 2
        else:
            self.group = None
            self.projection = 1 if self.inv != 0 else 0
        self.off, self.diag = oracle_terms(self.op)

    def oracle_states(self):
        lo, hi = self.basis._estimates()
        b = self.basis
        if self.projection == 2:
            return O.enumerate_projected(self.group, lo, hi, hamming_fixed=b._c.number_up >= 0)
        if isinstance(b, ls.SpinfulFermionBasis) and isinstance(b.occupation, tuple):
            return O.enumerate_spinful(b.number_sites, lo, hi)
        fixed = (b._c.number_up >= 0) if isinstance(b, ls.SpinBasis) else (b._c.number_particles >= 0)
        return O.enumerate_unprojected(b.number_bits if not isinstance(b, ls.SpinBasis) else b.number_spins,
                                       self.inv, fixed, lo, hi)

    def oracle_norms(self, reps):
        if self.projection == 2:
            return O.state_info(self.group, reps)[2]
        return np.ones(len(reps))

    def oracle_norms_exact(self, reps):
        if self.projection == 2:
            _, cnt = O.orbit_exact(self.group, reps)
            return np.sqrt(cnt / (self.group.order * (2 if self.inv else 1)))
        return np.ones(len(reps))

    def oracle_matvec(self, reps, x, complex_=False, exact_norms=True):
        """The reference's scatter algorithm; by default with exact stabiliser norms (identical to
        the reference's floating norms in real sectors)."""
        norms = self.oracle_norms_exact(reps) if exact_norms else self.oracle_norms(reps)
        y, st = O.matvec(self.group, self.projection, self.inv, self.nbits, reps, norms, self.off, self.diag, x,
                         complex_=complex_, identity_index=bool(self.basis._c.state_index_is_identity),
                         exact_norms=exact_norms)
        assert st == 0
        return y


def chain_case(n, k=0, p=None, inv=None, h="half", J=1.0):
    """h: Hamming weight, "half" for n // 2 (none under spin inversion), None for all weights."""
    syms = ls.Symmetries(LAT.chain_symmetries(n, k, p))
    if h == "half":
        h = n // 2 if inv is None else None
    basis = ls.SpinBasis(n, hamming_weight=h, spin_inversion=inv, symmetries=syms)
    return Case(basis, LAT.heisenberg(LAT.chain_bonds(n), J), "chain{}".format(n))


def config1_case(goldens):
    """BASELINE config 1 = chapel/data/heisenberg_chain_24_symm.yaml."""
    c = goldens["chapel_configs"]["heisenberg_chain_24_symm"]
    b = c["basis"]
    syms = ls.Symmetries([ls.Symmetry(s["permutation"], s["sector"]) for s in b["symmetries"]])
    basis = ls.SpinBasis(b["number_spins"], b["hamming_weight"], b["spin_inversion"], syms)
    expr = None
    for t in c["terms"]:
        e = ls.Expr(t["expression"], sites=t["sites"])
        expr = e if expr is None else expr + e
    return Case(basis, expr, "config1")


def square_case(L, kx=0, ky=0, inv=1, J2=0.0, h=None, point_group=True):
    syms = ls.Symmetries(LAT.square_symmetries(L, kx, ky, point_group))
    n = L * L
    basis = ls.SpinBasis(n, hamming_weight=h if h is not None else n // 2, spin_inversion=inv, symmetries=syms)
    expr = LAT.heisenberg(LAT.square_bonds(L))
    if J2 != 0.0:
        expr = expr + LAT.heisenberg(LAT.square_bonds(L, diagonal=True), J2)
    return Case(basis, expr, "square{}".format(L))
