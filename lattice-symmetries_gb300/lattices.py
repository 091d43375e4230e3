"""Lattices, symmetry generators and Hamiltonians of the standard workloads.

These play the role of the reference's chapel/data/*.yaml configs: plain descriptions from which
``Symmetries``, bases and ``Expr`` objects are built.
"""

from __future__ import annotations

from typing import List, Sequence, Tuple

from ._expr import Expr
from ._group import Symmetries, Symmetry


def chain_bonds(n: int) -> List[Tuple[int, int]]:
    return [(i, (i + 1) % n) for i in range(n)]


def chain_symmetries(n: int, momentum: int = 0, parity: int = None) -> List[Symmetry]:
    gens = [Symmetry([(i + 1) % n for i in range(n)], momentum)]
    if parity is not None:
        gens.append(Symmetry(list(range(n))[::-1], parity))
    return gens


def square_index(x: int, y: int, L: int) -> int:
    return (y % L) * L + (x % L)


def square_bonds(L: int, diagonal: bool = False) -> List[Tuple[int, int]]:
    """Nearest-neighbour (or next-nearest, diagonal=True) bonds of an L x L torus."""
    out = []
    for y in range(L):
        for x in range(L):
            i = square_index(x, y, L)
            if not diagonal:
                out.append((i, square_index(x + 1, y, L)))
                out.append((i, square_index(x, y + 1, L)))
            else:
                out.append((i, square_index(x + 1, y + 1, L)))
                out.append((i, square_index(x + 1, y - 1, L)))
    return out


def square_symmetries(L: int, kx: int = 0, ky: int = 0, point_group: bool = True) -> List[Symmetry]:
    """Translations (sectors kx, ky), the two reflections and the 90-degree rotation of an L x L
    torus (the generator set of chapel/data/heisenberg_square_6x6.yaml).  The point group is only
    compatible with momenta it maps to themselves (e.g. 0 or (pi, pi)); point_group=False keeps
    the translations only."""
    tx = [square_index(i % L + 1, i // L, L) for i in range(L * L)]
    ty = [square_index(i % L, i // L + 1, L) for i in range(L * L)]
    if not point_group:
        return [Symmetry(tx, kx), Symmetry(ty, ky)]
    rx = [square_index(L - 1 - i % L, i // L, L) for i in range(L * L)]
    ry = [square_index(i % L, L - 1 - i // L, L) for i in range(L * L)]
    rot = [square_index(L - 1 - i // L, i % L, L) for i in range(L * L)]
    return [Symmetry(tx, kx), Symmetry(ty, ky), Symmetry(rx, 0), Symmetry(ry, 0), Symmetry(rot, 0)]


def triangular_index(x: int, y: int, L: int) -> int:
    """Site x * a1 + y * a2 of an L x L triangular torus (a1 = (1, 0), a2 = (1/2, sqrt(3)/2))."""
    return (y % L) * L + (x % L)


def triangular_bonds(L: int) -> List[Tuple[int, int]]:
    """Nearest-neighbour bonds of an L x L triangular torus (directions a1, a2, a2 - a1)."""
    out = []
    for y in range(L):
        for x in range(L):
            i = triangular_index(x, y, L)
            out.append((i, triangular_index(x + 1, y, L)))
            out.append((i, triangular_index(x, y + 1, L)))
            out.append((i, triangular_index(x - 1, y + 1, L)))
    return out


def triangular_symmetries(L: int, k1: int = 0, k2: int = 0, rotation: int = 0, reflection: int = None
                          ) -> List[Symmetry]:
    """Translations (sectors k1, k2), the 60-degree rotation (x, y) -> (-y, x + y) with sector
    `rotation` (of 6) and, unless reflection is None, the mirror (x, y) -> (y, x) with that sector:
    the group T x C6 (6 L^2 elements) or T x C6v (12 L^2).  As on the square torus, the point group
    only combines with momenta it maps to themselves."""
    n = L * L
    t1 = [triangular_index(i % L + 1, i // L, L) for i in range(n)]
    t2 = [triangular_index(i % L, i // L + 1, L) for i in range(n)]
    rot = [triangular_index(-(i // L), i % L + i // L, L) for i in range(n)]
    gens = [Symmetry(t1, k1), Symmetry(t2, k2), Symmetry(rot, rotation)]
    if reflection is not None:
        gens.append(Symmetry([triangular_index(i // L, i % L, L) for i in range(n)], reflection))
    return gens


def hypercube_bonds(dim: int) -> List[Tuple[int, int]]:
    """Edges of the dim-dimensional hypercube (sites = dim-bit labels differing in one bit); for
    dim = 4 this is the 4 x 4 square torus with its sites relabelled."""
    return [(v, v ^ (1 << b)) for v in range(1 << dim) for b in range(dim) if v < v ^ (1 << b)]


def hypercube_symmetries(dim: int, odd_permutations: int = 0, even_only: bool = False) -> List[Symmetry]:
    """Automorphisms of the hypercube: the flip of label bit 0 and the permutations of the label
    bits (2^dim * dim! elements), or only the even permutations of the label bits with
    even_only=True.  odd_permutations=1 selects the representation that is -1 on odd permutations
    of the label bits (else trivial)."""
    n = 1 << dim

    def relabel(p):  # site v -> the label whose bit p[b] is bit b of v
        return [sum(((v >> b) & 1) << p[b] for b in range(dim)) for v in range(n)]

    flip = Symmetry([v ^ 1 for v in range(n)], 0)
    if even_only:
        c1 = [1, 2, 0] + list(range(3, dim))
        c2 = [0, 2, 3, 1] + list(range(4, dim))
        return [flip, Symmetry(relabel(c1), 0), Symmetry(relabel(c2), 0)]
    swap = [1, 0] + list(range(2, dim))
    cycle = list(range(1, dim)) + [0]
    # a dim-cycle is odd for even dim: sector dim/2 of its dim gives -1
    return [flip, Symmetry(relabel(swap), odd_permutations),
            Symmetry(relabel(cycle), (dim // 2) * odd_permutations if dim % 2 == 0 else 0)]


def heisenberg(bonds: Sequence[Tuple[int, int]], J=1.0) -> Expr:
    """J * sum (σˣσˣ + σʸσʸ + σᶻσᶻ) over bonds (the form of chapel/data/heisenberg_*.yaml)."""
    e = Expr("σˣ₀ σˣ₁ + σʸ₀ σʸ₁ + σᶻ₀ σᶻ₁", sites=[list(b) for b in bonds])
    return e.scale(J) if J != 1.0 else e


def xxz(bonds, Jxy=1.0, delta=1.0) -> Expr:
    exy = Expr("σˣ₀ σˣ₁ + σʸ₀ σʸ₁", sites=[list(b) for b in bonds]).scale(Jxy)
    ez = Expr("σᶻ₀ σᶻ₁", sites=[list(b) for b in bonds]).scale(delta)
    return exy + ez


def dm_z(bonds, D=1.0) -> Expr:
    """D * sum ẑ·(S_i × S_j) = D * sum (Sˣ_i Sʸ_j - Sʸ_i Sˣ_j) (imaginary σ⁺σ⁻ coefficients)."""
    e = Expr("Sˣ₀ Sʸ₁ - Sʸ₀ Sˣ₁", sites=[list(b) for b in bonds])
    return e.scale(D)


def ladder(n_rungs: int):
    """2-leg ladder, site (leg, r) -> leg * n_rungs + r; returns (leg bonds, rung bonds)."""
    legs = [(l * n_rungs + r, l * n_rungs + (r + 1) % n_rungs) for l in (0, 1) for r in range(n_rungs)]
    rungs = [(r, n_rungs + r) for r in range(n_rungs)]
    return legs, rungs


def ladder_symmetries(n_rungs: int, k: int = 0, exchange: int = 0) -> List[Symmetry]:
    n = 2 * n_rungs
    t = [(i // n_rungs) * n_rungs + (i % n_rungs + 1) % n_rungs for i in range(n)]
    ex = [(i + n_rungs) % n for i in range(n)]
    return [Symmetry(t, k), Symmetry(ex, exchange)]


def hubbard_parts(bonds, number_sites=None):
    """(hopping with t = 1, on-site interaction with U = 1): H = t * hopping + U * interaction."""
    hop = Expr("c†₀↑ c₁↑ + c†₁↑ c₀↑ + c†₀↓ c₁↓ + c†₁↓ c₀↓", sites=[list(b) for b in bonds]).scale(-1.0)
    n = number_sites if number_sites is not None else 1 + max(max(b) for b in bonds)
    onsite = Expr("n₀↑ n₀↓", sites=[[i] for i in range(n)])
    return hop, onsite


def hubbard(bonds, t=1.0, U=1.0, number_sites=None) -> Expr:
    hop = Expr("c†₀↑ c₁↑ + c†₁↑ c₀↑ + c†₀↓ c₁↓ + c†₁↓ c₀↓", sites=[list(b) for b in bonds]).scale(-t)
    n = number_sites if number_sites is not None else 1 + max(max(b) for b in bonds)
    onsite = Expr("n₀↑ n₀↓", sites=[[i] for i in range(n)]).scale(U)
    return hop + onsite
