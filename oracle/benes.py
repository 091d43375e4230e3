"""Benes networks for the oracle (TEST INFRASTRUCTURE ONLY; see ls_oracle.c).

The reference applies every group element as a Benes network of delta swaps
(haskell/src/LatticeSymmetries/Benes.hs:295-377; one step is kernels/generator.cpp:5-8):

    y = ((x >> d) ^ x) & m;   x = x ^ y ^ (y << d)

which exchanges bits p and p + d wherever bit p of m is set.  This module routes a permutation
into such a network by the classical looping algorithm (Benes 1964; Waksman 1968), written here
from the algorithm's description and independent of the product's router.  The network on
n = 2^k positions has 2k - 1 stages with shifts 1, 2, ..., n/2, ..., 2, 1: the outer stages
exchange the pairs (2j, 2j + 1), the inner stages keep the parity of a position and route the
even and the odd positions as two networks on n/2 positions.

Semantics as in Benes.hs:338-345: bit i of the image is bit perm[i] of the input.
"""

from __future__ import annotations

from typing import List, Sequence, Tuple

import numpy as np


def _route(perm: List[int]) -> Tuple[List[int], List[int]]:
    """(masks, shifts) of a network on len(perm) = 2^k positions; masks as Python ints."""
    n = len(perm)
    if n == 2:
        return [1 if perm[0] == 1 else 0], [1]
    # colour c[p] of input position p: the sub-network (0 even, 1 odd) its element passes through.
    # Input pairs (2j, 2j+1) and the inputs of output pairs (perm[2i], perm[2i+1]) get different
    # colours; following the constraints alternately closes loops.
    where = [0] * n  # output position of input p
    for o, p in enumerate(perm):
        where[p] = o
    c = [-1] * n
    for start in range(n):
        if c[start] >= 0:
            continue
        p, col = start, 0
        while c[p] < 0:
            c[p] = col
            c[p ^ 1] = 1 - col
            # the output partner of p ^ 1's output takes the other colour than p ^ 1, i.e. col
            q = perm[where[p ^ 1] ^ 1]
            p = q
    first = 0  # swap input pair j when its even element goes to the odd network
    for j in range(n // 2):
        if c[2 * j] == 1:
            first |= 1 << (2 * j)
    last = 0  # swap output pair i when output 2i's element comes out of the odd network
    t = [0] * (n // 2)
    for i in range(n // 2):
        t[i] = c[perm[2 * i]]
        if t[i]:
            last |= 1 << (2 * i)
    subs = [[0] * (n // 2), [0] * (n // 2)]
    for o in range(n):
        e = c[perm[o]]
        q = o ^ t[o >> 1]  # position before the last stage (parity e)
        subs[e][q >> 1] = perm[o] >> 1
    inner = [_route(subs[0]), _route(subs[1])]
    masks = [first]
    shifts = [1]
    for s in range(len(inner[0][0])):
        m = 0
        for e in (0, 1):
            sub = inner[e][0][s]
            for b in range(n // 2):
                if (sub >> b) & 1:
                    m |= 1 << (2 * b + e)
        masks.append(m)
        shifts.append(2 * inner[0][1][s])
    masks.append(last)
    shifts.append(1)
    return masks, shifts


def network(perm: Sequence[int]) -> Tuple[List[int], List[int]]:
    """(masks, shifts) realising `perm` on 64-bit words (positions beyond len(perm) fixed); the
    size is padded to the next power of two (at least 2), as Benes.hs:308-314 does."""
    n = len(perm)
    size = 2
    while size < n:
        size *= 2
    full = list(perm) + list(range(n, size))
    return _route(full)


def group_network(perms: Sequence[Sequence[int]]) -> Tuple[np.ndarray, np.ndarray]:
    """Masks [depth][n_elems] (the layout of kernels/kernels.c:157-167) and shifts [depth] for a
    list of permutations of the same size."""
    nets = [network(p) for p in perms]
    shifts = nets[0][1]
    assert all(s == shifts for _, s in nets)
    masks = np.array([[m[k] for m, _ in nets] for k in range(len(shifts))], dtype=np.uint64)
    return masks, np.array(shifts, dtype=np.uint64)


def apply(masks: Sequence[int], shifts: Sequence[int], x: int) -> int:
    for m, d in zip(masks, shifts):
        y = ((x >> d) ^ x) & m
        x = x ^ y ^ ((y << d) & 0xFFFFFFFFFFFFFFFF)
    return x


def permute_bits(perm: Sequence[int], x: int) -> int:
    return sum(((x >> p) & 1) << i for i, p in enumerate(perm))
