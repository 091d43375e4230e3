"""Parity of every packed-kernel instantiation the dispatcher can select.

The packed projected kernel is compiled for 1, 2, 3, 4, 6, 9, 12 and 16 group elements per lane
(slots), each with and without spin inversion.  The chain and square cases of the other files
reach 1-4 slots; the groups here reach the rest:

    slots  group (elements)                                   sites
      6    triangular 4x4 T x C6v (192), hypercube Q4 even (192),
           square 6x6 T x C4 (144, complex)                   16 / 16 / 36
      9    square 6x6 T x C4v (288), triangular 6x6 T x C6 (216, complex)     36
     12    hypercube Q4 = square 4x4 torus automorphisms (384)                16
     16    triangular 6x6 T x C6v (432)                                       36

Small Hamming weights keep the 36-site bases small enough for the oracle's full matvec.  The
full-size cases (the J1-J2 6x6 (pi, pi) sector of the headline benchmark and the triangular 6x6
Sz = 0 sector with inversion) compare sampled columns of H with the oracle's scatter of the same
columns (chapel/src/BatchedOperator.chpl:207-253, DistributedMatrixVector.chpl:91-143): the exact
set of non-zero rows and the values to relative L2 <= 1e-12, through the 16-column block kernel,
the one-vector kernel and the adjoint kernel, and through the reference-facing host-pointer call.
"""

import numpy as np
import pytest

import oracle as O
from ls_helpers import LAT, Case, ls

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def rel_l2(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-300)


def _square_c4(L, rotation):
    """Translations x the 90-degree rotation (no mirrors) of an L x L torus."""
    rot = [LAT.square_index(L - 1 - i // L, i % L, L) for i in range(L * L)]
    return LAT.square_symmetries(L, 0, 0, point_group=False) + [ls.Symmetry(rot, rotation)]


def _case(name):
    S = ls.Symmetries
    if name == "tri4_c6v_z1":
        b = ls.SpinBasis(16, 8, 1, S(LAT.triangular_symmetries(4, 0, 0, 0, 0)))
        return Case(b, LAT.heisenberg(LAT.triangular_bonds(4)), name), 6
    if name == "q4even_zm1":
        b = ls.SpinBasis(16, 8, -1, S(LAT.hypercube_symmetries(4, even_only=True)))
        return Case(b, LAT.heisenberg(LAT.hypercube_bonds(4)), name), 6
    if name == "sq6_c4_rot1_h5":
        b = ls.SpinBasis(36, 5, None, S(_square_c4(6, 1)))
        return Case(b, LAT.heisenberg(LAT.square_bonds(6)) + LAT.heisenberg(LAT.square_bonds(6, True), 0.5), name), 6
    if name == "sq6_c4v_pipi_h5":
        b = ls.SpinBasis(36, 5, None, S(LAT.square_symmetries(6, 3, 3)))
        return Case(b, LAT.heisenberg(LAT.square_bonds(6)) + LAT.heisenberg(LAT.square_bonds(6, True), 0.5), name), 9
    if name == "tri6_c6_rot1_h5":
        b = ls.SpinBasis(36, 5, None, S(LAT.triangular_symmetries(6, 0, 0, 1)))
        return Case(b, LAT.heisenberg(LAT.triangular_bonds(6)), name), 9
    if name == "q4_z1":
        b = ls.SpinBasis(16, 8, 1, S(LAT.hypercube_symmetries(4)))
        return Case(b, LAT.heisenberg(LAT.hypercube_bonds(4)), name), 12
    if name == "q4sign_zm1":
        b = ls.SpinBasis(16, 8, -1, S(LAT.hypercube_symmetries(4, odd_permutations=1)))
        return Case(b, LAT.heisenberg(LAT.hypercube_bonds(4)), name), 12
    if name == "q4_h6":
        b = ls.SpinBasis(16, 6, None, S(LAT.hypercube_symmetries(4)))
        return Case(b, LAT.heisenberg(LAT.hypercube_bonds(4)), name), 12
    if name == "tri6_c6v_h5":
        b = ls.SpinBasis(36, 5, None, S(LAT.triangular_symmetries(6, 0, 0, 0, 0)))
        return Case(b, LAT.heisenberg(LAT.triangular_bonds(6)), name), 16
    raise KeyError(name)


SMALL = ["tri4_c6v_z1", "q4even_zm1", "sq6_c4_rot1_h5", "sq6_c4v_pipi_h5", "tri6_c6_rot1_h5", "q4_z1",
         "q4sign_zm1", "q4_h6", "tri6_c6v_h5"]


@pytest.fixture(scope="module")
def small_cases():
    out = {}
    for name in SMALL:
        c, slots = _case(name)
        c.basis.build()
        out[name] = (c, slots)
    return out


@pytest.mark.parametrize("name", SMALL)
def test_slots_kernel_and_enumeration(small_cases, name):
    c, slots = small_cases[name]
    assert c.op.kernel_info() == ("packed", slots)
    states = c.basis.states
    assert len(states) >= 10
    assert np.array_equal(states, c.oracle_states())


@pytest.mark.parametrize("name", SMALL)
def test_slots_matvec_complex_block_adjoint(small_cases, name):
    import torch
    c, _ = small_cases[name]
    states = c.basis.states
    D = len(states)
    rng = np.random.default_rng(11)
    x = rng.normal(size=D) + 1j * rng.normal(size=D)
    yo = c.oracle_matvec(states, x, complex_=True)
    y = c.op.apply_device(torch.from_numpy(x).cuda()).cpu().numpy()
    assert rel_l2(y, yo) <= RTOL
    # H is Hermitian: the adjoint kernel (adjoint term table) gives the same vector
    ya = c.op.apply_device(torch.from_numpy(x).cuda(), adjoint=True).cpu().numpy()
    assert rel_l2(ya, yo) <= RTOL
    # 16-column block: every column against the oracle
    X = rng.normal(size=(D, 16)) + 1j * rng.normal(size=(D, 16))
    Y = c.op.apply_device(torch.from_numpy(X).cuda()).cpu().numpy()
    for col in range(16):
        assert rel_l2(Y[:, col], c.oracle_matvec(states, X[:, col], complex_=True)) <= RTOL


@pytest.mark.parametrize("name", SMALL)
def test_slots_reference_facing_real_matvec(small_cases, name):
    """ls_chpl_matrix_vector_product (host buffers, real x and y, real part of the elements)."""
    c, _ = small_cases[name]
    states = c.basis.states
    x = np.random.default_rng(12).normal(size=len(states))
    y = c.op.apply_to_state_vector(x)
    assert rel_l2(y, c.oracle_matvec(states, x)) <= RTOL


# ------------------------------------------------------------------------------------------------
# Full-size sectors: sampled columns
# ------------------------------------------------------------------------------------------------
def _merge(rows, vals, tol):
    u, inv = np.unique(rows, return_inverse=True)
    v = np.zeros(len(u), dtype=np.complex128)
    np.add.at(v, inv, vals)
    keep = np.abs(v) > tol
    return u[keep], v[keep]


def _nonzero_rows(y, tol):
    import torch
    idx = torch.nonzero(torch.abs(y) > tol).flatten()
    return idx.cpu().numpy(), y[idx].cpu().numpy()


def sampled_columns(case, n_cols=32, seed=0):
    """GPU columns of H (block, one-vector, adjoint, host-pointer paths) against the oracle's
    scatter of the same columns.  Returns the sample's per-column non-zero counts."""
    import torch
    b = case.basis
    states = b.states
    D = len(states)
    rng = np.random.default_rng(seed)
    cols = np.sort(rng.choice(D, size=n_cols, replace=False)).astype(np.int64)
    norms = O.state_info(case.group, states[cols])[2]
    ref = O.matvec_columns(case.group, 2, case.inv, case.nbits, states, cols, norms, case.off, case.diag,
                           exact_norms=True)
    scale = max(np.abs(v).max() for _, v in ref)
    tol = 1e-12 * scale
    ref = [_merge(r, v, tol) for r, v in ref]
    counts = []
    # block kernel: H e_j for 16 columns at a time
    for c0 in range(0, n_cols, 16):
        X = torch.zeros((D, 16), dtype=torch.complex128, device="cuda")
        for k in range(16):
            X[int(cols[c0 + k]), k] = 1.0
        Y = case.op.apply_device(X)
        for k in range(16):
            rows, vals = _nonzero_rows(Y[:, k], tol)
            r_rows, r_vals = ref[c0 + k]
            assert np.array_equal(rows, r_rows), "column {}: rows differ".format(int(cols[c0 + k]))
            assert rel_l2(vals, r_vals) <= RTOL
            counts.append(len(rows))
        del X, Y
    # one-vector kernel and adjoint kernel on a random combination of the sampled columns
    coef = rng.normal(size=n_cols) + 1j * rng.normal(size=n_cols)
    expected = {}
    for (r_rows, r_vals), a in zip(ref, coef):
        for r, v in zip(r_rows.tolist(), r_vals.tolist()):
            expected[r] = expected.get(r, 0.0) + a * v
    e_rows = np.array(sorted(expected), dtype=np.int64)
    e_vals = np.array([expected[r] for r in e_rows.tolist()])
    x = torch.zeros(D, dtype=torch.complex128, device="cuda")
    x[torch.from_numpy(cols).cuda()] = torch.from_numpy(coef).cuda()
    for adjoint in (False, True):
        y = case.op.apply_device(x, adjoint=adjoint)
        got = y[torch.from_numpy(e_rows).cuda()].cpu().numpy()
        assert rel_l2(got, e_vals) <= RTOL
        # nothing outside the expected rows
        y[torch.from_numpy(e_rows).cuda()] = 0
        assert float(torch.abs(y).max()) <= 1e-12 * float(np.abs(e_vals).max())
    # the reference-facing call with host buffers (real x, real y)
    xr = np.zeros(D)
    xr[cols] = coef.real
    yr = case.op.apply_to_state_vector(xr)
    er = np.zeros(D)
    for (r_rows, r_vals), a in zip(ref, coef.real):
        np.add.at(er, r_rows, (a * r_vals).real)
    assert rel_l2(yr, er) <= RTOL
    return counts


def check_enumeration_pin(basis, key):
    """The GPU enumeration equals the oracle's full enumeration of the sector (count and SHA-256,
    tests/golden/enumeration_pins.json, made by tests/golden/make_enumeration_pins.py), and a
    random candidate range re-enumerated by the oracle here."""
    import hashlib
    import json
    import os
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "enumeration_pins.json")) as f:
        pin = json.load(f)[key]
    states = np.ascontiguousarray(basis.states)
    assert len(states) == pin["count"]
    assert states[:4].tolist() == pin["first"] and states[-4:].tolist() == pin["last"]
    assert hashlib.sha256(states.astype("<u8").tobytes()).hexdigest() == pin["sha256"]
    lo, hi = basis._estimates()
    r0, r1 = O.rank(lo), O.rank(hi)
    from ls_helpers import oracle_group
    group = oracle_group(basis.symmetries, basis._c.spin_inversion)
    # the start of the range (dense in representatives) and a random window in its first 5 %
    for start in (r0, int(np.random.default_rng(1).integers(r0, r0 + (r1 - r0) // 20))):
        a, b = O.unrank(start, 18), O.unrank(start + 1_000_000, 18)
        got = O.enumerate_projected_par(group, a, b)
        inside = states[(states >= np.uint64(a)) & (states <= np.uint64(b))]
        assert np.array_equal(got, inside)


def test_headline_j1j2_6x6_pipi_sampled_columns():
    """The bench's default workload, at full size: J1-J2 6x6 (pi, pi), T x C4v x Z2."""
    syms = ls.Symmetries(LAT.square_symmetries(6, 3, 3))
    basis = ls.SpinBasis(36, 18, 1, syms)
    expr = LAT.heisenberg(LAT.square_bonds(6)) + LAT.heisenberg(LAT.square_bonds(6, diagonal=True), 0.5)
    case = Case(basis, expr, "j1j2_6x6")
    basis.build()
    assert basis.number_states == 15741359
    check_enumeration_pin(basis, "square6_pipi_z1")
    assert case.op.kernel_info() == ("packed", 9)
    counts = sampled_columns(case, 32, seed=2)
    assert min(counts) >= 1 and max(counts) <= 289


def test_triangular_6x6_inversion_sampled_columns():
    """16 slots with spin inversion: triangular 6x6, T x C6v x Z2, Sz = 0."""
    syms = ls.Symmetries(LAT.triangular_symmetries(6, 0, 0, 0, 0))
    basis = ls.SpinBasis(36, 18, 1, syms)
    case = Case(basis, LAT.heisenberg(LAT.triangular_bonds(6)), "tri6")
    basis.build()
    assert basis.number_states > 5_000_000
    check_enumeration_pin(basis, "triangular6_c6v_z1")
    assert case.op.kernel_info() == ("packed", 16)
    sampled_columns(case, 32, seed=3)
