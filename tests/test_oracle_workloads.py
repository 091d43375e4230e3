"""The oracle-side restatement of the benchmark workloads (oracle/workloads.py, oracle/benes.py),
which `bench.py --impl reference` uses without loading the product: its Benes networks realise
the permutations, its group and term tables equal the product's for the same workload, and its
threaded enumeration reproduces the single-threaded one and the config-1 basis size."""

import random

import numpy as np
import pytest

import benes
import oracle as O
import workloads as W
from ls_helpers import LAT, ls


def test_benes_router_realises_random_permutations():
    rnd = random.Random(5)
    for n in (2, 3, 7, 16, 24, 36, 49, 64):
        for _ in range(10):
            p = list(range(n))
            rnd.shuffle(p)
            masks, shifts = benes.network(p)
            assert len(shifts) == 2 * max(1, (n - 1).bit_length()) - 1
            for _ in range(10):
                x = rnd.getrandbits(n)
                assert benes.apply(masks, shifts, x) == benes.permute_bits(p, x)


def _as_set(terms):
    v = terms.v.view(np.complex128)
    return sorted(zip(v.real.round(15), v.imag.round(15), *(a.tolist() for a in terms.arrs)))


def test_j1j2_workload_matches_the_product_description():
    w = W.workload("j1j2_6x6")
    basis = ls.SpinBasis(36, 18, 1, ls.Symmetries(LAT.square_symmetries(6, 3, 3)))
    expr = LAT.heisenberg(LAT.square_bonds(6)) + LAT.heisenberg(LAT.square_bonds(6, diagonal=True), 0.5)
    op = ls.Operator(basis, expr)
    assert _as_set(w.off) == _as_set(O.Terms(*op._off_arrays))
    assert _as_set(w.diag) == _as_set(O.Terms(*op._diag_arrays))
    assert w.group.order == basis.symmetries.order == 288
    assert w.estimates() == basis._estimates()
    # same group elements and characters
    ours = {tuple(p): (round(a, 12), round(b, 12)) for p, a, b in zip(w.group.perms.tolist(), w.group.chars_re,
                                                                        w.group.chars_im)}
    re, im = basis.symmetries.characters
    theirs = {tuple(p): (round(a, 12), round(b, 12)) for p, a, b in zip(basis.symmetries.permutations.tolist(),
                                                                        re, im)}
    assert ours == theirs
    # the oracle's own Benes network gives the same images as the bit-by-bit permutations
    rng = np.random.default_rng(3)
    xs = np.array([O.unrank(int(r), 18) for r in rng.integers(0, 9075135300, size=300)], dtype=np.uint64)
    a = O.state_info(w.group, xs, use_benes=True)
    b = O.state_info(w.group, xs, use_benes=False)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])


def test_threaded_enumeration_matches_serial_on_a_candidate_range():
    w = W.workload("j1j2_6x6")
    lo, _ = w.estimates()
    hi = O.unrank(O.rank(lo) + 400_000, 18)
    serial = O.enumerate_projected(w.group, lo, hi, lane_width=8, use_benes=True)
    threaded = O.enumerate_projected_par(w.group, lo, hi, lane_width=8, use_benes=True)
    assert len(serial) > 1000
    assert np.array_equal(serial, threaded)


def test_chain24_workload_is_config1(goldens):
    w = W.workload("chain24")
    lo, hi = w.estimates()
    reps = O.enumerate_projected_par(w.group, lo, hi, lane_width=8, use_benes=True)
    assert len(reps) == 28968


def test_sampled_columns_equal_full_scatter():
    """lso_matvec_columns / lso_matvec_sample reproduce lso_matvec on the columns they cover."""
    w = W.workload("chain24")
    lo, hi = w.estimates()
    reps = O.enumerate_projected_par(w.group, lo, hi)
    D = len(reps)
    norms = O.state_info(w.group, reps, use_benes=True)[2]
    rng = np.random.default_rng(4)
    cols = np.sort(rng.choice(D, size=300, replace=False))
    x = np.zeros(D, dtype=np.complex128)
    x[cols] = rng.normal(size=300) + 1j * rng.normal(size=300)
    y_full, st = O.matvec(w.group, 2, 1, 24, reps, norms, w.off, w.diag, x, complex_=True, baseline=True)
    assert st == 0
    idx = O.Index(reps, 24)
    y = np.zeros(D, dtype=np.complex128)
    nnz = O.matvec_sample(w.group, 2, 1, 24, reps, cols, norms[cols], w.off, w.diag, x[cols], y, idx)
    assert nnz > 300
    assert np.abs(y - y_full).max() <= 1e-12 * np.abs(y_full).max()
    y2 = np.zeros(D, dtype=np.complex128)
    for c, (rows, vals) in zip(cols, O.matvec_columns(w.group, 2, 1, 24, reps, cols, norms[cols], w.off, w.diag,
                                                       baseline=True, exact_norms=False, index=idx)):
        np.add.at(y2, rows, vals * x[c])
    assert np.abs(y2 - y_full).max() <= 1e-12 * np.abs(y_full).max()
