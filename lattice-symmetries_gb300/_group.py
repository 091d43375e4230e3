"""Permutation groups, characters and Benes networks (host side).

This module produces the inputs of the GPU orbit-scan kernels: the closed group of lattice
symmetries, one character per group element, and one Benes network per element batched into a
``[depth][|G|]`` mask matrix.  It follows the semantics of the reference's Haskell host layer:

* permutation convention: bit ``i`` of ``g.x`` is bit ``p[i]`` of ``x``
  (haskell/src/LatticeSymmetries/Benes.hs:338-345, ``permuteBits'``);
* composition ``(a <> b)[i] = b[a[i]]`` (Benes.hs:100-101) and phases add modulo one
  (Group.hs:95-96);
* closure by breadth-first products with the generators, returned in ascending order of
  ``(permutation, phase)`` (Group.hs:174-183, ``fromGenerators``);
* the consistency check that every product is in the set and has an integer sector
  (Group.hs:124-132);
* characters ``cos(-2*pi*phi)`` and ``sin(-2*pi*phi)`` with ``phi = sector/periodicity``
  (Group.hs:115-116);
* Benes networks on the bit count padded to a power of two, with stage distances
  ``1, 2, ..., n/2, ..., 2, 1`` (Benes.hs:295-336) and the mask layout ``[stage][element]``
  (Benes.hs:356-377).

The routing that chooses the masks is this module's own (the classic looping algorithm on
adjacent pairs); any valid routing yields the same permutation, which is what the kernels and
the tests rely on.
"""

from __future__ import annotations

import math
from fractions import Fraction
from typing import List, Sequence, Tuple

import numpy as np

Permutation = Tuple[int, ...]


def _check_permutation(p: Sequence[int]) -> Permutation:
    p = tuple(int(i) for i in p)
    if len(p) == 0 or sorted(p) != list(range(len(p))):
        raise ValueError("invalid permutation: {}".format(list(p)))
    return p


def compose(a: Permutation, b: Permutation) -> Permutation:
    """``(a <> b)[i] = b[a[i]]`` (Benes.hs:100-101)."""
    return tuple(b[i] for i in a)


def periodicity(p: Permutation) -> int:
    """Smallest n >= 1 with p^n = identity (Group.hs:47-53)."""
    identity = tuple(range(len(p)))
    n, q = 1, p
    while q != identity:
        q = compose(p, q)
        n += 1
    return n


def permute_bits(p: Permutation, x: int) -> int:
    """Bit i of the result is bit p[i] of x (Benes.hs:338-345)."""
    y = 0
    for i, pi in enumerate(p):
        if (x >> pi) & 1:
            y |= 1 << i
    return y


class Symmetry:
    """A permutation together with a sector (Group.hs:58-85).

    ``phase = sector / periodicity``; 0 <= sector < periodicity.
    """

    __slots__ = ("permutation", "phase")

    def __init__(self, permutation: Sequence[int], sector: int):
        p = _check_permutation(permutation)
        n = periodicity(p)
        sector = int(sector)
        if sector < 0 or sector >= n:
            raise ValueError(
                "invalid sector: {}; permutation has periodicity {}".format(sector, n))
        self.permutation = p
        self.phase = Fraction(sector, n)

    @classmethod
    def _from_phase(cls, p: Permutation, phase: Fraction) -> "Symmetry":
        s = cls.__new__(cls)
        s.permutation = p
        s.phase = phase
        return s

    @property
    def periodicity(self) -> int:
        return periodicity(self.permutation)

    @property
    def sector(self) -> int:
        s = self.phase * self.periodicity
        if s.denominator != 1:
            raise ValueError("invalid symmetry: phase {} is not a multiple of 1/{}".format(
                self.phase, self.periodicity))
        return int(s)

    def __mul__(self, other: "Symmetry") -> "Symmetry":
        """Semigroup product ``self <> other`` (Group.hs:95-96)."""
        phase = self.phase + other.phase
        if phase >= 1:
            phase -= phase.numerator // phase.denominator
        return Symmetry._from_phase(compose(self.permutation, other.permutation), phase)

    def _key(self):
        return (self.permutation, self.phase)

    def __eq__(self, other):
        return isinstance(other, Symmetry) and self._key() == other._key()

    def __lt__(self, other):
        return self._key() < other._key()

    def __hash__(self):
        return hash(self._key())

    def __len__(self):
        return len(self.permutation)

    def __repr__(self):
        return "Symmetry({}, sector={})".format(list(self.permutation), self.sector)

    def json_object(self):
        return {"permutation": list(self.permutation), "sector": self.sector}


def close_group(generators: Sequence[Symmetry]) -> List[Symmetry]:
    """Group closure in ascending (permutation, phase) order (Group.hs:174-183)."""
    if len(generators) == 0:
        return []
    n = len(generators[0])
    identity = Symmetry(tuple(range(n)), 0)
    interior = set()
    boundary = {identity}
    while boundary:
        interior |= boundary
        nxt = set()
        for h in boundary:
            for g in generators:
                nxt.add(h * g)
        boundary = nxt - interior
    return sorted(interior)


def character(phase: Fraction) -> Tuple[float, float]:
    """(cos(-2 pi phi), sin(-2 pi phi)) with phi the phase as a double (Group.hs:115-116)."""
    phi = float(phase)
    angle = -2 * math.pi * phi
    return (math.cos(angle), math.sin(angle))


# ---------------------------------------------------------------------------------------------
# Benes networks
# ---------------------------------------------------------------------------------------------


def padded_size(number_bits: int) -> int:
    """2**ceil(log2(n)) as in Benes.hs:308-314."""
    n = 1
    while n < number_bits:
        n *= 2
    return n


def benes_shifts(number_bits: int) -> List[int]:
    """Stage distances 1, 2, ..., n/2, ..., 2, 1 for the padded size n (Benes.hs:295-306)."""
    n = padded_size(number_bits)
    up = []
    d = 1
    while 2 * d <= n:
        up.append(d)
        d *= 2
    return up + list(reversed(up[:-1]))


def _route(p: List[int]) -> List[List[int]]:
    """Masks (as lists of swapped lower positions) of a Benes network realising out[i] = in[p[i]].

    Returns one list per stage, outermost stages first/last, for size len(p) = 2**k: the
    network is stage A (pairs (2j, 2j+1)), two half-size networks on the even and the odd
    positions, stage B (pairs (2j, 2j+1)).
    """
    n = len(p)
    if n == 1:
        return []
    if n == 2:
        return [[0] if p[0] == 1 else []]
    pinv = [0] * n
    for i, e in enumerate(p):
        pinv[e] = i
    via_even = [None] * n  # routing of each element (input position)
    for start in range(0, n, 2):
        if via_even[p[start]] is not None:
            continue
        # Output `out` takes its element through the even sub-network; follow the cycle.
        out = start
        while True:
            e = p[out]
            if via_even[e] is not None:
                break
            via_even[e] = True
            partner = e ^ 1                       # the other element of e's input pair
            via_even[partner] = False             # ... goes through the odd sub-network
            q = pinv[partner]                     # output that needs the partner
            out = q ^ 1                           # its output partner must use the even one
            if via_even[p[out]] is not None:
                break
    stage_a = [2 * k for k in range(n // 2) if not via_even[2 * k]]
    stage_b = [2 * j for j in range(n // 2) if not via_even[p[2 * j]]]
    sigma_even = [0] * (n // 2)
    sigma_odd = [0] * (n // 2)
    for i in range(n):
        e = p[i]
        if via_even[e]:
            sigma_even[i // 2] = e // 2
        else:
            sigma_odd[i // 2] = e // 2
    inner_even = _route(sigma_even)
    inner_odd = _route(sigma_odd)
    inner = []
    for se, so in zip(inner_even, inner_odd):
        inner.append(sorted([2 * i for i in se] + [2 * i + 1 for i in so]))
    return [stage_a] + inner + [stage_b]


def benes_network(p: Sequence[int]) -> Tuple[List[int], List[int]]:
    """(masks, shifts) of one permutation, padded to a power of two (Benes.hs:316-323)."""
    p = list(_check_permutation(p))
    n = padded_size(len(p))
    p = p + list(range(len(p), n))
    stages = _route(p)
    shifts = benes_shifts(len(p)) if n > 1 else []
    assert len(stages) == len(shifts)
    masks = []
    for positions in stages:
        m = 0
        for i in positions:
            m |= 1 << i
        masks.append(m)
    return masks, shifts


def bit_permute_step(x: int, m: int, d: int) -> int:
    """generator.cpp:5-8 / Benes.hs:325-328: swap bits i and i+d for every i set in m."""
    y = ((x >> d) ^ x) & m
    return x ^ y ^ (y << d)


def apply_network(masks: Sequence[int], shifts: Sequence[int], x: int) -> int:
    for m, d in zip(masks, shifts):
        x = bit_permute_step(x, m, d)
    return x


class Symmetries:
    """The closed group generated by a list of symmetries (Group.hs:98-133)."""

    def __init__(self, generators: Sequence[Symmetry] = ()):
        generators = list(generators)
        self._generators = generators
        if len(generators) == 0:
            self.elements: List[Symmetry] = []
            self.number_bits = 0
        else:
            n = len(generators[0])
            if any(len(g) != n for g in generators):
                raise ValueError("symmetries have different number of sites")
            self.elements = close_group(generators)
            self.number_bits = n
            present = set(self.elements)
            for s1 in self.elements:
                for s2 in self.elements:
                    s3 = s1 * s2
                    if s3 not in present or (s3.phase * periodicity(s3.permutation)).denominator != 1:
                        raise ValueError("incompatible symmetries")
        self._network = None

    @property
    def generators(self) -> List[Symmetry]:
        return self._generators

    def __len__(self) -> int:
        return len(self._generators)

    @property
    def order(self) -> int:
        return len(self.elements)

    def json_object(self):
        return [g.json_object() for g in self._generators]

    @property
    def permutations(self) -> np.ndarray:
        return np.array([s.permutation for s in self.elements], dtype=np.int32).reshape(
            len(self.elements), self.number_bits)

    @property
    def characters(self) -> Tuple[np.ndarray, np.ndarray]:
        ch = [character(s.phase) for s in self.elements]
        re = np.array([c[0] for c in ch], dtype=np.float64)
        im = np.array([c[1] for c in ch], dtype=np.float64)
        return re, im

    @property
    def phases(self) -> List[Fraction]:
        return [s.phase for s in self.elements]

    def is_real(self) -> bool:
        """Group.hs:155-156: all imaginary parts of the characters are exactly zero."""
        return bool(np.all(self.characters[1] == 0))

    def doubled(self) -> "Symmetries":
        """The same group acting on spinful-fermion orbitals: site permutation p becomes
        p on the up orbitals [0, n) and p + n on the down orbitals [n, 2n); elements keep their
        order and characters."""
        n = self.number_bits
        gens = [Symmetry(list(g.permutation) + [n + int(i) for i in g.permutation], g.sector)
                for g in self._generators]
        return Symmetries(gens)

    def network(self) -> Tuple[np.ndarray, np.ndarray]:
        """Batched Benes network: masks [depth][|G|] (uint64) and shifts [depth] (uint64)."""
        if self._network is None:
            if not self.elements:
                self._network = (np.zeros((0, 0), dtype=np.uint64), np.zeros(0, dtype=np.uint64))
            else:
                per = [benes_network(s.permutation) for s in self.elements]
                shifts = per[0][1]
                depth = len(shifts)
                masks = np.zeros((depth, len(per)), dtype=np.uint64)
                for j, (m, sh) in enumerate(per):
                    assert sh == shifts
                    for k in range(depth):
                        masks[k, j] = m[k]
                self._network = (masks, np.array(shifts, dtype=np.uint64))
        return self._network
