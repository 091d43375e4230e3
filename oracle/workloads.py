"""Benchmark workloads restated for the oracle (TEST INFRASTRUCTURE ONLY; see ls_oracle.c).

`bench.py --impl reference` times the CPU restatement of the reference's algorithm without
loading anything of the product: the lattice, its symmetry generators, the Benes networks
(benes.py), the group closure (oracle.close_group) and the non-branching term tables below are
all built here from plain data.

Term tables follow the reference's format (kernels/lattice_symmetries_types.h:140-151; applied as
kernels/reference.c:67-134): for a column state a and term t the element exists when
(a & m_t) == r_t; the target is a ^ x_t with coefficient v_t (-1)^popcount(a & s_t).  A bond
(i, j) of sigma.sigma = 2 (s+_i s-_j + s-_i s+_j) + sz_i sz_j gives two off-diagonal terms
(v = 2J, m = x = bits i and j, r = the bit that is set before the flip, l = the other one) and one
diagonal term (v = J, s = bits i and j).
"""

from __future__ import annotations

from typing import Dict, List, Sequence, Tuple

import numpy as np

import benes
import oracle as O


def square_index(x: int, y: int, L: int) -> int:
    return (y % L) * L + (x % L)


def square_bonds(L: int, diagonal: bool = False) -> List[Tuple[int, int]]:
    out = []
    for y in range(L):
        for x in range(L):
            i = square_index(x, y, L)
            if diagonal:
                out += [(i, square_index(x + 1, y + 1, L)), (i, square_index(x + 1, y - 1, L))]
            else:
                out += [(i, square_index(x + 1, y, L)), (i, square_index(x, y + 1, L))]
    return out


def square_generators(L: int, kx: int, ky: int) -> List[Tuple[List[int], int]]:
    """Translations (sectors kx, ky), both mirrors and the 90-degree rotation (sector 0): the
    generators of chapel/data/heisenberg_square_6x6.yaml with the momentum changed."""
    n = L * L
    tx = [square_index(i % L + 1, i // L, L) for i in range(n)]
    ty = [square_index(i % L, i // L + 1, L) for i in range(n)]
    rx = [square_index(L - 1 - i % L, i // L, L) for i in range(n)]
    ry = [square_index(i % L, L - 1 - i // L, L) for i in range(n)]
    rot = [square_index(L - 1 - i // L, i % L, L) for i in range(n)]
    return [(tx, kx), (ty, ky), (rx, 0), (ry, 0), (rot, 0)]


def chain_generators(n: int, k: int, parity: int) -> List[Tuple[List[int], int]]:
    return [([(i + 1) % n for i in range(n)], k), (list(range(n))[::-1], parity)]


def heisenberg_terms(bonds: Sequence[Tuple[int, int]], J: Sequence[float]):
    """(off-diagonal, diagonal) term tables of sum_b J_b sigma_i . sigma_j, as oracle.Terms."""
    off = {k: [] for k in "vmlrxs"}
    diag = {k: [] for k in "vmlrxs"}
    for (i, j), c in zip(bonds, J):
        bi, bj = 1 << i, 1 << j
        for r, l in ((bj, bi), (bi, bj)):
            for k, v in zip("vmlrxs", (2.0 * c, bi | bj, l, r, bi | bj, 0)):
                off[k].append(v)
        for k, v in zip("vmlrxs", (c, 0, 0, 0, 0, bi | bj)):
            diag[k].append(v)

    def terms(d):
        return O.Terms(np.array(d["v"], dtype=np.complex128), *(np.array(d[k], dtype=np.uint64) for k in "mlrxs"))

    return terms(off), terms(diag)


class Workload:
    """A projected spin sector: group (with its Benes network), sector range and Hamiltonian."""

    def __init__(self, name: str, number_sites: int, hamming: int, spin_inversion: int,
                 generators: Sequence[Tuple[List[int], int]], bonds, couplings, seed: int):
        self.name = name
        self.n = number_sites
        self.h = hamming
        self.inv = spin_inversion
        self.seed = seed
        el = O.close_group(generators)
        re, im = O.characters(el)
        perms = np.array([e[0] for e in el], dtype=np.int32)
        masks, shifts = benes.group_network([list(p) for p in perms])
        self.group = O.Group(perms, re, im, spin_inversion, number_sites, masks, shifts)
        self.off, self.diag = heisenberg_terms(bonds, couplings)

    def estimates(self) -> Tuple[int, int]:
        """Range of candidate representatives (haskell/src/LatticeSymmetries/Basis.hs:734-774)."""
        lo = (1 << self.h) - 1
        hi = lo << (self.n - self.h - (1 if self.inv != 0 else 0))
        return lo, hi


def workload(name: str) -> Workload:
    if name == "j1j2_6x6":
        L = 6
        bonds = square_bonds(L) + square_bonds(L, diagonal=True)
        J = [1.0] * (2 * L * L) + [0.5] * (2 * L * L)
        return Workload(name, L * L, L * L // 2, 1, square_generators(L, 3, 3), bonds, J, seed=2)
    if name == "chain24":
        n = 24
        bonds = [(i, (i + 1) % n) for i in range(n)]
        return Workload(name, n, n // 2, 1, chain_generators(n, 0, 0), bonds, [1.0] * n, seed=1)
    raise KeyError(name)


WORKLOADS: Dict[str, str] = {"j1j2_6x6": "J1-J2 6x6 (pi, pi)", "chain24": "Heisenberg chain N=24"}
