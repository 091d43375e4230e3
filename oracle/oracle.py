"""Python side of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs import this module.  It wraps
oracle/_build/liboracle.so (this repository's C restatement of the reference's algorithms,
ls_oracle.c) and oracle/_ref/libls_ref.so (the reference's own kernels/indexing.c and
kernels/reference.c compiled where they lie, when the reference tree is present), and adds two
independent pure-Python restatements used to cross-check the product's host layer:

* ``close_group`` -- group closure and characters (Group.hs:106-133, :174-183), written without
  the product's code;
* ``apply_product`` -- the action of a product of spin/fermion generators on a basis state,
  evaluated bit by bit with Jordan-Wigner signs (no non-branching tables), used to build dense
  matrices for small systems.
"""

from __future__ import annotations

import ctypes
import math
import os
import subprocess
from ctypes import POINTER, Structure, c_double, c_int, c_int32, c_int64, c_uint8, c_uint64, c_void_p
from fractions import Fraction
from typing import Dict, List, Sequence, Tuple

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libls_ref.so")


def build(ref: bool = False) -> None:
    targets = ["all"] + (["ref"] if ref else [])
    subprocess.run(["make", "-s", "-C", HERE] + targets, check=True)


class lso_group(Structure):
    _fields_ = [("n_bits", c_int), ("n_elems", c_int), ("spin_inversion", c_int),
                ("perms", POINTER(c_int32)), ("chars_re", POINTER(c_double)),
                ("chars_im", POINTER(c_double)), ("depth", c_int), ("masks", POINTER(c_uint64)),
                ("shifts", POINTER(c_uint64))]


class lso_terms(Structure):
    _fields_ = [("n", c_int), ("v", POINTER(c_double)), ("m", POINTER(c_uint64)),
                ("l", POINTER(c_uint64)), ("r", POINTER(c_uint64)), ("x", POINTER(c_uint64)),
                ("s", POINTER(c_uint64))]


class lso_projection(Structure):
    _fields_ = [("projection", c_int), ("spin_inversion", c_int), ("n_bits", c_int),
                ("state_index_identity", c_int)]


LSO_COMPLEX, LSO_BENES, LSO_PREFIX_INDEX, LSO_ATOMIC, LSO_EXACT_NORMS = 1, 2, 4, 8, 16

_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        L.lso_state_info.argtypes = [POINTER(lso_group), c_int, c_int, c_int64, POINTER(c_uint64),
                                     POINTER(c_uint64), POINTER(c_double), POINTER(c_double)]
        L.lso_is_representative.argtypes = [POINTER(lso_group), c_int, c_int, c_int64, POINTER(c_uint64),
                                            POINTER(c_uint8), POINTER(c_double)]
        L.lso_orbit_exact.argtypes = [POINTER(lso_group), c_int64, POINTER(c_uint64), POINTER(c_uint64),
                                      POINTER(c_int32)]
        L.lso_fixed_hamming_state_to_index.restype = c_int64
        L.lso_fixed_hamming_state_to_index.argtypes = [c_uint64]
        L.lso_fixed_hamming_index_to_state.restype = c_uint64
        L.lso_fixed_hamming_index_to_state.argtypes = [c_int64, c_int]
        L.lso_enumerate_projected.restype = c_int64
        L.lso_enumerate_projected.argtypes = [POINTER(lso_group), c_int, c_int, c_int, c_uint64, c_uint64,
                                              POINTER(c_uint64), c_int64]
        L.lso_enumerate_unprojected.restype = c_int64
        L.lso_enumerate_unprojected.argtypes = [c_int, c_int, c_int, c_uint64, c_uint64, POINTER(c_uint64), c_int64]
        L.lso_enumerate_spinful.restype = c_int64
        L.lso_enumerate_spinful.argtypes = [c_int, c_uint64, c_uint64, POINTER(c_uint64), c_int64]
        L.lso_matvec.restype = c_int
        L.lso_matvec.argtypes = [POINTER(lso_group), POINTER(lso_projection), c_int64, POINTER(c_uint64),
                                 POINTER(c_double), POINTER(lso_terms), POINTER(lso_terms), c_int,
                                 POINTER(c_double), POINTER(c_double), c_int64, c_int64, POINTER(c_int64)]
        L.lso_enumerate_projected_par.restype = c_int64
        L.lso_enumerate_projected_par.argtypes = [POINTER(lso_group), c_int, c_int, c_int, c_uint64, c_uint64,
                                                  POINTER(c_uint64), c_int64]
        L.lso_index_create.restype = c_void_p
        L.lso_index_create.argtypes = [POINTER(c_uint64), c_int64, c_int, c_int]
        L.lso_index_destroy.argtypes = [c_void_p]
        L.lso_matvec_columns.restype = c_int
        L.lso_matvec_columns.argtypes = [POINTER(lso_group), POINTER(lso_projection), c_int64, POINTER(c_uint64),
                                         c_void_p, POINTER(lso_terms), POINTER(lso_terms), c_int, c_int64,
                                         POINTER(c_int64), POINTER(c_double), POINTER(c_int64), POINTER(c_double),
                                         POINTER(c_int64)]
        L.lso_matvec_sample.restype = c_int
        L.lso_matvec_sample.argtypes = [POINTER(lso_group), POINTER(lso_projection), c_int64, POINTER(c_uint64),
                                        c_void_p, POINTER(lso_terms), POINTER(lso_terms), c_int, c_int64,
                                        POINTER(c_int64), POINTER(c_double), POINTER(c_double), POINTER(c_double),
                                        POINTER(c_int64)]
        L.lso_max_threads.restype = c_int
        L.lso_set_threads.argtypes = [c_int]
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(POINTER(t))


class Group:
    """A closed group for the oracle: permutations (bit i of g.x = bit perm[i] of x), characters,
    spin inversion, and optionally the Benes network used by the baseline path."""

    def __init__(self, perms, chars_re, chars_im, spin_inversion=0, n_bits=None, masks=None, shifts=None):
        n_elems = len(chars_re)
        perms = np.asarray(perms, dtype=np.int32)
        self.perms = np.ascontiguousarray(perms.reshape(n_elems, -1) if n_elems > 0 else np.zeros((0, 1), np.int32))
        self.chars_re = np.ascontiguousarray(chars_re, dtype=np.float64)
        self.chars_im = np.ascontiguousarray(chars_im, dtype=np.float64)
        self.spin_inversion = int(spin_inversion)
        self.n_bits = int(n_bits if n_bits is not None else self.perms.shape[1])
        self.masks = None if masks is None else np.ascontiguousarray(masks, dtype=np.uint64)
        self.shifts = None if shifts is None else np.ascontiguousarray(shifts, dtype=np.uint64)
        c = lso_group()
        c.n_bits = self.n_bits
        c.n_elems = len(self.chars_re)
        c.spin_inversion = self.spin_inversion
        c.perms = _p(self.perms, c_int32)
        c.chars_re = _p(self.chars_re, c_double)
        c.chars_im = _p(self.chars_im, c_double)
        if self.masks is not None:
            c.depth = int(self.masks.shape[0])
            c.masks = _p(self.masks, c_uint64)
            c.shifts = _p(self.shifts, c_uint64)
        else:
            c.depth = 0
        self.c = c

    @property
    def order(self):
        return len(self.chars_re)


def state_info(g: Group, xs, lane_width=8, use_benes=False):
    xs = np.ascontiguousarray(xs, dtype=np.uint64)
    n = xs.shape[0]
    reps = np.zeros(n, dtype=np.uint64)
    chars = np.zeros(2 * n, dtype=np.float64)
    norms = np.zeros(n, dtype=np.float64)
    lib().lso_state_info(ctypes.byref(g.c), lane_width, int(use_benes), n, _p(xs, c_uint64),
                         _p(reps, c_uint64), _p(chars, c_double), _p(norms, c_double))
    return reps, chars[0::2] + 1j * chars[1::2], norms


def is_representative(g: Group, xs, lane_width=4, use_benes=False):
    xs = np.ascontiguousarray(xs, dtype=np.uint64)
    n = xs.shape[0]
    flags = np.zeros(n, dtype=np.uint8)
    norms = np.zeros(n, dtype=np.float64)
    lib().lso_is_representative(ctypes.byref(g.c), lane_width, int(use_benes), n, _p(xs, c_uint64),
                                _p(flags, c_uint8), _p(norms, c_double))
    return flags, norms


def orbit_exact(g: Group, xs):
    xs = np.ascontiguousarray(xs, dtype=np.uint64)
    n = xs.shape[0]
    reps = np.zeros(n, dtype=np.uint64)
    cnt = np.zeros(n, dtype=np.int32)
    lib().lso_orbit_exact(ctypes.byref(g.c), n, _p(xs, c_uint64), _p(reps, c_uint64), _p(cnt, c_int32))
    return reps, cnt


def rank(state: int) -> int:
    return int(lib().lso_fixed_hamming_state_to_index(state))


def unrank(index: int, h: int) -> int:
    return int(lib().lso_fixed_hamming_index_to_state(index, h))


def enumerate_projected(g: Group, lower, upper, hamming_fixed=True, lane_width=4, use_benes=False, cap=None):
    if cap is None:
        n_cand = rank(upper) - rank(lower) + 1 if hamming_fixed else upper - lower + 1
        cap = max(16, int(n_cand // max(1, g.order) * 4) + 4096)
        cap = min(cap, int(n_cand) + 1)
    out = np.zeros(cap, dtype=np.uint64)
    n = lib().lso_enumerate_projected(ctypes.byref(g.c), lane_width, int(use_benes), int(hamming_fixed),
                                      lower, upper, _p(out, c_uint64), cap)
    if n > cap:
        return enumerate_projected(g, lower, upper, hamming_fixed, lane_width, use_benes, cap=int(n))
    return out[:n]


def enumerate_projected_par(g: Group, lower, upper, hamming_fixed=True, lane_width=8, use_benes=True, cap=None):
    """Projected enumeration on all threads (ls_oracle.c lso_enumerate_projected_par): the same
    states as enumerate_projected, with the candidate range split among threads by rank."""
    if cap is None:
        n_cand = rank(upper) - rank(lower) + 1 if hamming_fixed else upper - lower + 1
        cap = max(16, int(n_cand // max(1, g.order) * 3 // (2 if g.spin_inversion else 1)) + 4096)
        cap = min(cap, int(n_cand) + 1)
    out = np.zeros(cap, dtype=np.uint64)
    n = lib().lso_enumerate_projected_par(ctypes.byref(g.c), lane_width, int(use_benes), int(hamming_fixed),
                                          lower, upper, _p(out, c_uint64), cap)
    if n > cap:
        return enumerate_projected_par(g, lower, upper, hamming_fixed, lane_width, use_benes, cap=int(n))
    return out[:n]


class Index:
    """The reference's prefix-table index over sorted representatives (kernels/indexing.c:45-117),
    built once; keeps a reference to the array it indexes."""

    def __init__(self, reps, number_bits, prefix_bits=22):
        self.reps = np.ascontiguousarray(reps, dtype=np.uint64)
        self.ptr = lib().lso_index_create(_p(self.reps, c_uint64), self.reps.shape[0], int(number_bits),
                                          int(prefix_bits))

    def __del__(self):
        if getattr(self, "ptr", None):
            lib().lso_index_destroy(self.ptr)
            self.ptr = None


def _projection(projection, spin_inversion, n_bits, identity_index=False):
    pr = lso_projection()
    pr.projection = projection
    pr.spin_inversion = spin_inversion
    pr.n_bits = n_bits
    pr.state_index_identity = int(identity_index)
    return pr


def matvec_columns(g, projection, spin_inversion, n_bits, reps, cols, col_norms, off: "Terms", diag: "Terms",
                   baseline=False, exact_norms=True, index: "Index" = None, identity_index=False):
    """Columns `cols` of H as sparse lists (ls_oracle.c lso_matvec_columns): returns a list of
    (rows, values) per column, complex values, the diagonal element first, duplicates not merged.
    baseline: Benes orbit scan (else the bit-by-bit permutations)."""
    reps = np.ascontiguousarray(reps, dtype=np.uint64)
    cols = np.ascontiguousarray(cols, dtype=np.int64)
    nc = cols.shape[0]
    norms = np.ascontiguousarray(np.ones(nc) if col_norms is None else col_norms, dtype=np.float64)
    stride = off.c.n + 1
    rows = np.zeros(nc * stride, dtype=np.int64)
    vals = np.zeros(2 * nc * stride, dtype=np.float64)
    counts = np.zeros(nc, dtype=np.int64)
    if g is None:
        g = Group(np.zeros((0, 1)), [], [], 0, n_bits)
    pr = _projection(projection, spin_inversion, n_bits, identity_index)
    mode = (LSO_BENES if baseline else 0) | (LSO_EXACT_NORMS if exact_norms else 0)
    st = lib().lso_matvec_columns(ctypes.byref(g.c), ctypes.byref(pr), reps.shape[0], _p(reps, c_uint64),
                                  index.ptr if index is not None else None, ctypes.byref(off.c),
                                  ctypes.byref(diag.c), mode, nc, _p(cols, c_int64), _p(norms, c_double),
                                  _p(rows, c_int64), _p(vals, c_double), _p(counts, c_int64))
    if st != 0:
        raise RuntimeError("an element of a sampled column left the basis")
    v = vals.view(np.complex128)
    return [(rows[c * stride:c * stride + counts[c]].copy(), v[c * stride:c * stride + counts[c]].copy())
            for c in range(nc)]


def matvec_sample(g, projection, spin_inversion, n_bits, reps, cols, col_norms, off: "Terms", diag: "Terms", x, y,
                  index: "Index", exact_norms=False):
    """y += H[:, cols] x over a sample of columns by the reference's scatter algorithm with atomics
    (ls_oracle.c lso_matvec_sample), Benes orbit scan and prefix index; x complex [len(cols)],
    y complex [D] (not cleared).  Returns the number of off-diagonal elements generated."""
    reps = index.reps if index is not None else np.ascontiguousarray(reps, dtype=np.uint64)
    cols = np.ascontiguousarray(cols, dtype=np.int64)
    norms = np.ascontiguousarray(col_norms, dtype=np.float64)
    xv = np.ascontiguousarray(x, dtype=np.complex128).view(np.float64)
    assert y.dtype == np.complex128 and y.flags.c_contiguous and y.shape[0] == reps.shape[0]
    pr = _projection(projection, spin_inversion, n_bits)
    mode = LSO_BENES | LSO_PREFIX_INDEX | LSO_ATOMIC | (LSO_EXACT_NORMS if exact_norms else 0)
    nnz = c_int64(0)
    st = lib().lso_matvec_sample(ctypes.byref(g.c), ctypes.byref(pr), reps.shape[0], _p(reps, c_uint64),
                                 index.ptr if index is not None else None, ctypes.byref(off.c), ctypes.byref(diag.c),
                                 mode, cols.shape[0], _p(cols, c_int64), _p(norms, c_double), _p(xv, c_double),
                                 _p(y.view(np.float64), c_double), ctypes.byref(nnz))
    if st != 0:
        raise RuntimeError("an element of a sampled column left the basis")
    return int(nnz.value)


def enumerate_unprojected(number_sites, spin_inversion, hamming_fixed, low, high):
    n_max = (rank(high) - rank(low) + 1) if hamming_fixed else (high - low + 1)
    out = np.zeros(max(int(n_max), 1), dtype=np.uint64)
    n = lib().lso_enumerate_unprojected(number_sites, spin_inversion, int(hamming_fixed), low, high,
                                        _p(out, c_uint64), out.shape[0])
    return out[:n]


def enumerate_spinful(number_sites, lower, upper):
    mask = (1 << number_sites) - 1
    na = rank(upper & mask) - rank(lower & mask) + 1
    nb = rank((upper >> number_sites) & mask) - rank((lower >> number_sites) & mask) + 1
    out = np.zeros(max(na * nb, 1), dtype=np.uint64)
    n = lib().lso_enumerate_spinful(number_sites, lower, upper, _p(out, c_uint64), out.shape[0])
    return out[:n]


class Terms:
    def __init__(self, v, m, l, r, x, s):
        self.v = np.ascontiguousarray(np.asarray(v, dtype=np.complex128).view(np.float64))
        self.arrs = [np.ascontiguousarray(a, dtype=np.uint64) for a in (m, l, r, x, s)]
        c = lso_terms()
        c.n = len(self.arrs[0])
        c.v = _p(self.v, c_double)
        c.m, c.l, c.r, c.x, c.s = (_p(a, c_uint64) for a in self.arrs)
        self.c = c


def matvec(g, projection, spin_inversion, n_bits, reps, rep_norms, off: Terms, diag: Terms, x,
           complex_=False, baseline=False, cols=None, identity_index=False, return_nnz=False,
           exact_norms=False):
    """y = H x by the reference's scatter algorithm (ls_oracle.c lso_matvec).

    exact_norms: norms of generated states from the exact stabiliser sum instead of the
    reference's floating sum of characters (they differ only for orbits whose stabiliser
    character is non-trivial in complex sectors, where the reference's sum is rounding noise
    and its driver halts on the resulting index miss).

    Returns (y, status), or (y, status, nnz) with return_nnz: the off-diagonal elements that the
    processed columns contributed."""
    reps = np.ascontiguousarray(reps, dtype=np.uint64)
    D = reps.shape[0]
    if rep_norms is None:
        rep_norms = np.ones(D)
    rep_norms = np.ascontiguousarray(rep_norms, dtype=np.float64)
    pr = lso_projection()
    pr.projection = projection
    pr.spin_inversion = spin_inversion
    pr.n_bits = n_bits
    pr.state_index_identity = int(identity_index)
    if complex_:
        xv = np.ascontiguousarray(np.asarray(x, dtype=np.complex128)).view(np.float64)
        y = np.zeros(2 * D, dtype=np.float64)
    else:
        xv = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros(D, dtype=np.float64)
    mode = (LSO_COMPLEX if complex_ else 0) | ((LSO_BENES | LSO_PREFIX_INDEX | LSO_ATOMIC) if baseline else 0)
    mode |= LSO_EXACT_NORMS if exact_norms else 0
    if g is None:
        g = Group(np.zeros((0, 1)), [], [], 0, n_bits)
    gc = ctypes.byref(g.c)
    c0, c1 = (-1, -1) if cols is None else cols
    nnz = c_int64(0)
    st = lib().lso_matvec(gc, ctypes.byref(pr), D, _p(reps, c_uint64), _p(rep_norms, c_double),
                          ctypes.byref(off.c), ctypes.byref(diag.c), mode, _p(xv, c_double), _p(y, c_double),
                          c0, c1, ctypes.byref(nnz))
    if complex_:
        y = y.view(np.complex128)
    if return_nnz:
        return y, st, int(nnz.value)
    return y, st


def set_threads(n: int):
    lib().lso_set_threads(int(n))


def max_threads() -> int:
    return int(lib().lso_max_threads())


# ----------------------------------------------------------------------------------------------
# Independent restatements (pure Python)
# ----------------------------------------------------------------------------------------------

def close_group(generators: Sequence[Tuple[Sequence[int], int]]):
    """[(perm tuple, Fraction phase)] in ascending order (Group.hs:174-183).

    generators: (permutation, sector) pairs.  Composition (a <> b)[i] = b[a[i]], phases add mod 1.
    """
    if not generators:
        return []
    gens = []
    for p, sector in generators:
        p = tuple(int(i) for i in p)
        n, q = 1, p
        ident = tuple(range(len(p)))
        while q != ident:
            q = tuple(q[i] for i in p)
            n += 1
        gens.append((p, Fraction(int(sector), n)))
    ident = (tuple(range(len(gens[0][0]))), Fraction(0))
    seen = {ident}
    frontier = [ident]
    while frontier:
        new = []
        for (pa, fa) in frontier:
            for (pb, fb) in gens:
                pc = tuple(pb[i] for i in pa)
                fc = fa + fb
                if fc >= 1:
                    fc -= 1
                e = (pc, fc)
                if e not in seen:
                    seen.add(e)
                    new.append(e)
        frontier = new
    return sorted(seen)


def characters(elements):
    re = np.array([math.cos(-2 * math.pi * float(f)) for _, f in elements])
    im = np.array([math.sin(-2 * math.pi * float(f)) for _, f in elements])
    return re, im


def apply_product(product, state: int, number_sites: int):
    """Apply a product of generators (rightmost first) to a basis state bit by bit.

    product: sequence of (kind, site) with kinds '1', 'z', '+', '-' (Pauli spins) or 'f1', 'n',
    'c+', 'c' (fermions; site is an int or (spin, k) with spin 0 = up in bits [0, n), 1 = down in
    bits [n, 2n)).  Returns (coefficient, new_state) or (0, None).
    """
    c = 1
    s = state
    for kind, site in reversed(list(product)):
        if isinstance(site, tuple):
            spin, k = site
            b = k + (number_sites if spin == 1 else 0)
        else:
            b = site
        bit = (s >> b) & 1
        if kind in ("1", "f1"):
            continue
        if kind == "z":
            c *= 1 if bit else -1
        elif kind == "+":
            if bit:
                return 0, None
            s |= 1 << b
        elif kind == "-":
            if not bit:
                return 0, None
            s &= ~(1 << b)
        elif kind == "n":
            if not bit:
                return 0, None
        elif kind in ("c+", "c"):
            if (kind == "c+") == bool(bit):
                return 0, None
            sign = bin(s & ((1 << b) - 1)).count("1") % 2
            c *= -1 if sign else 1
            s ^= 1 << b
        else:
            raise ValueError(kind)
    return c, s


def dense_from_products(terms, states: Sequence[int], number_sites: int) -> np.ndarray:
    """Dense <a|H|b> over `states` for H = sum_k coeff_k * product_k (coefficients complex)."""
    idx = {int(s): i for i, s in enumerate(states)}
    n = len(states)
    H = np.zeros((n, n), dtype=np.complex128)
    for coeff, product in terms:
        for j, b in enumerate(states):
            c, a = apply_product(product, int(b), number_sites)
            if a is None or c == 0:
                continue
            if a in idx:
                H[idx[a], j] += complex(coeff) * c
    return H
