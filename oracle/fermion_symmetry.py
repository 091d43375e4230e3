"""Dense restatement of symmetry-adapted bases, spins and spinful fermions (test infrastructure:
only tests may import this module; nothing in the product calls it).

The reference has no fermionic bases with lattice symmetries (haskell/src/LatticeSymmetries/
Basis.hs:713-723), so this module restates the standard construction for small systems with
dense linear algebra, to check the GPU path:

* a group element with site permutation p acts on a basis state x by "bit i of g.x = bit p[i] of
  x" (haskell/src/LatticeSymmetries/Benes.hs:338-345); on spinful fermions p acts on the up
  orbitals [0, n) and on the down orbitals [n, 2n) alike, and the Fock-space operator
  g |x> = c^dag_{g(k1)} c^dag_{g(k2)} ... |0> (k1 < k2 < ... occupied, g(k) = p^-1(k)) equals
  (-1)^inv |g.x>, inv = #{(k < l) occupied : g(k) > g(l)};
* the symmetric basis vector of a representative r is |r~> = sum_g chi_g g|r> / (|G| n_r) with
  n_r = || sum_g chi_g g|r> || / |G| (representatives with n_r = 0 are dropped), and
  H~ = P^dagger H P for the matrix P of these vectors;
* H itself is assembled from the non-branching terms, T|a> = v [(a & m) == r] (-1)^popcount(a & s)
  |a ^ x> (kernels/reference.c:97-135).

The characters chi_g and the choice chi_g (not its conjugate) are fixed by the spin case, which must
reproduce the oracle's C restatement of the reference (checked in the tests).
"""

from __future__ import annotations

from typing import Dict, List, Sequence, Tuple

import numpy as np


def apply_perm(perm: Sequence[int], x: int) -> int:
    y = 0
    for i, pi in enumerate(perm):
        if (x >> pi) & 1:
            y |= 1 << i
    return y


def fermion_sign(perm: Sequence[int], x: int) -> int:
    """(-1)^inv for the orbital map g(k) = position of k in perm."""
    pos = {int(k): i for i, k in enumerate(perm)}
    occ = [k for k in range(len(perm)) if (x >> k) & 1]
    images = [pos[k] for k in occ]
    inv = 0
    for a in range(len(images)):
        for b in range(a + 1, len(images)):
            if images[a] > images[b]:
                inv += 1
    return -1 if inv & 1 else 1


def hamiltonian(states: Sequence[int], terms) -> np.ndarray:
    """Dense H on the span of `states` from (v, m, l, r, x, s) arrays (off-diagonal and diagonal
    terms alike); states outside the span must not be generated."""
    index: Dict[int, int] = {int(a): i for i, a in enumerate(states)}
    D = len(states)
    H = np.zeros((D, D), dtype=complex)
    v, m, l, r, x, s = terms
    for j, a in enumerate(states):
        a = int(a)
        for t in range(len(v)):
            if (a & int(m[t])) != int(r[t]):
                continue
            sign = -1.0 if bin(a & int(s[t])).count("1") & 1 else 1.0
            b = a ^ int(x[t])
            H[index[b], j] += v[t] * sign
    return H


def symmetric_basis(states: Sequence[int], elements: List[Tuple[Sequence[int], complex]],
                    fermionic: bool) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Representatives (ascending), their norms n_r and the matrix P [len(states), len(reps)]."""
    index = {int(a): i for i, a in enumerate(states)}
    G = len(elements)
    seen = set()
    reps, norms, cols = [], [], []
    for a in sorted(int(z) for z in states):
        if a in seen:
            continue
        vec = np.zeros(len(states), dtype=complex)
        orbit = []
        for perm, chi in elements:
            b = apply_perm(perm, a)
            sg = fermion_sign(perm, a) if fermionic else 1
            vec[index[b]] += chi * sg
            orbit.append(b)
        seen.update(orbit)
        r = min(orbit)
        if r != a:
            continue  # a is not the orbit minimum (its orbit was entered through a smaller state)
        nrm = np.linalg.norm(vec) / G
        if nrm < 1e-12:
            continue
        reps.append(a)
        norms.append(nrm)
        cols.append(vec / (G * nrm))
    P = np.array(cols).T if cols else np.zeros((len(states), 0), dtype=complex)
    return np.array(reps, dtype=np.uint64), np.array(norms), P


def group_elements(permutations: np.ndarray, chars_re: np.ndarray, chars_im: np.ndarray):
    return [(list(map(int, p)), complex(cr, ci)) for p, cr, ci in zip(permutations, chars_re, chars_im)]


def fixed_occupation_states(n_sites: int, n_up: int, n_down: int) -> List[int]:
    """All spinful-fermion states with the given particle numbers (up bits low), ascending."""
    from itertools import combinations
    ups = [sum(1 << k for k in c) for c in combinations(range(n_sites), n_up)]
    downs = [sum(1 << k for k in c) for c in combinations(range(n_sites), n_down)]
    return sorted((d << n_sites) | u for d in downs for u in ups)
