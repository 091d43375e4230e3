"""The oracle and the host layer pinned against the reference's own known answers (CPU)."""

import importlib
import os

import numpy as np
import pytest

import oracle as O
from ls_helpers import Case, E, LAT, chain_case, config1_case, ls, oracle_group, square_case

G = importlib.import_module("lattice-symmetries_gb300._group")


def test_benes_known_answers(goldens):
    """haskell/test/LatticeSymmetries/BenesSpec.hs:33-41."""
    for kat in goldens["benes_kats"]:
        masks, shifts = G.benes_network(kat["permutation"])
        assert G.apply_network(masks, shifts, kat["x"]) == kat["y"]
        assert G.permute_bits(tuple(kat["permutation"]), kat["x"]) == kat["y"]


def test_benes_property():
    """BenesSpec.hs:24-28: the network reproduces permuteBits' for random permutations."""
    rng = np.random.default_rng(0)
    for _ in range(200):
        n = int(rng.integers(1, 65))
        p = list(rng.permutation(n))
        masks, shifts = G.benes_network(p)
        assert shifts == G.benes_shifts(n) if n > 1 else shifts == []
        for x in rng.integers(0, 1 << min(n, 62), size=10):
            x = int(x) & ((1 << n) - 1)
            assert G.apply_network(masks, shifts, x) == G.permute_bits(tuple(p), x)


@pytest.mark.parametrize("gens", [
    [([(i + 1) % 10 for i in range(10)], 5), (list(range(10))[::-1], 1)],
    [([(i + 1) % 24 for i in range(24)], 0), (list(range(24))[::-1], 0)],
    [([2, 10, 0, 4, 3, 7, 11, 5, 9, 8, 1, 6], 1)],  # kagome right_shift, python/test/test_api.py:50
    [([(i + 1) % 28 for i in range(28)], 3)],
])
def test_group_closure_matches_independent_restatement(gens):
    S = ls.Symmetries([ls.Symmetry(p, s) for p, s in gens])
    el = O.close_group(gens)
    assert [e[0] for e in el] == [s.permutation for s in S.elements]
    re, im = O.characters(el)
    r2, i2 = S.characters
    assert np.array_equal(re, r2) and np.array_equal(im, i2)
    masks, shifts = S.network()
    rng = np.random.default_rng(1)
    n = S.number_bits
    for j, s in enumerate(S.elements):
        for x in rng.integers(0, 1 << n, size=5):
            y = G.apply_network([int(m) for m in masks[:, j]], [int(d) for d in shifts], int(x))
            assert y == G.permute_bits(s.permutation, int(x))


def test_square_pi_pi_sector_is_consistent():
    S = ls.Symmetries(LAT.square_symmetries(6, 3, 3))
    assert S.order == 288


def test_n10_chain_ground_state(goldens):
    """python/example/getting_started.py:9-51: E0 = -18.06178542."""
    g = goldens["n10_chain"]
    syms = ls.Symmetries([ls.Symmetry(s["permutation"], s["sector"]) for s in g["symmetries"]])
    basis = ls.SpinBasis(g["number_spins"], spin_inversion=g["spin_inversion"], symmetries=syms)
    case = Case(basis, ls.Expr(g["expression"], sites=g["sites"]))
    reps = case.oracle_states()
    D = len(reps)
    H = np.zeros((D, D))
    for j in range(D):
        e = np.zeros(D)
        e[j] = 1
        H[:, j] = case.oracle_matvec(reps, e)
    assert np.allclose(H, H.T, atol=1e-13)
    assert np.isclose(np.linalg.eigvalsh(H)[0], g["energy"], atol=1e-8)


def _hubbard_2site(t, U):
    e = ls.Expr("c†↑₀ c↑₁", sites=[(0, 1)]).scale(-t)
    e = e - ls.Expr("c†↑₁ c↑₀", sites=[(0, 1)]).scale(t)
    e = e - ls.Expr("c†↓₁ c↓₀", sites=[(0, 1)]).scale(t)
    e = e - ls.Expr("c†↓₀ c↓₁", sites=[(0, 1)]).scale(t)
    e = e + ls.Expr("n↑₀ n↓₀", sites=[(0,)]).scale(U)
    e = e + ls.Expr("n↑₁ n↓₁", sites=[(1,)]).scale(U)
    return e


@pytest.mark.parametrize("name", ["test_hubbard_hamiltonian_matrix",
                                  "test_hubbard_hamiltonian_matrix_with_defined_particle_number"])
def test_hubbard_2site_golden_matrices(goldens, name):
    """python/run_tests.py:128-175."""
    h = goldens["hubbard_2site"]
    expected = np.array(h["matrices"][name], dtype=float)
    args = h["bases"][name]
    basis = ls.SpinfulFermionBasis(*args) if len(args) == 1 else ls.SpinfulFermionBasis(args[0], args[1])
    case = Case(basis, _hubbard_2site(h["t"], h["U"]))
    states = case.oracle_states()
    D = len(states)
    H = np.zeros((D, D))
    for j in range(D):
        x = np.zeros(D)
        x[j] = 1
        H[:, j] = case.oracle_matvec(states, x)
    assert np.array_equal(H, expected)
    # independent bit-level action of the generator products
    prods = [(v.to_complex(), p) for v, p in case.expr.terms]
    Hd = O.dense_from_products(prods, [int(s) for s in states], 2)
    assert np.array_equal(Hd.real, expected) and not Hd.imag.any()


def _hphi_case(entry):
    b = entry["basis"]
    if b.get("particle") == "spinful-fermion":
        basis = ls.SpinfulFermionBasis(b["number_sites"], b.get("number_particles"))
        if isinstance(b.get("number_particles"), list):
            basis = ls.SpinfulFermionBasis(b["number_sites"], tuple(b["number_particles"]))
    else:
        basis = ls.SpinBasis(b["number_spins"], b.get("hamming_weight"), b.get("spin_inversion"))
    expr = None
    for t in entry["terms"]:
        e = ls.Expr(t["expression"], sites=t["sites"])
        expr = e if expr is None else expr + e
    return Case(basis, expr, entry["name"])


@pytest.mark.parametrize("idx", range(5))
def test_hphi_ground_state_energies(goldens, idx):
    """test/0[1-5]_*/HPhi/output/zvo_energy.dat against dense diagonalisation of the oracle's H."""
    entry = goldens["hphi"][idx]
    case = _hphi_case(entry)
    states = case.oracle_states()
    D = len(states)
    H = np.zeros((D, D), dtype=np.complex128)
    for j in range(D):
        x = np.zeros(D, dtype=np.complex128)
        x[j] = 1
        H[:, j] = case.oracle_matvec(states, x, complex_=True)
    assert np.allclose(H, H.conj().T, atol=1e-12)
    e0 = np.linalg.eigvalsh(H)[0]
    assert abs(e0 - entry["energy"]) < 1e-9


def test_config1_representative_count(goldens):
    """BASELINE config 1 (chapel/data/heisenberg_chain_24_symm.yaml): 28,968 representatives."""
    case = config1_case(goldens)
    reps = case.oracle_states()
    assert len(reps) == 28968
    assert np.all(np.diff(reps.astype(np.int64)) > 0)


def test_reference_index_kernel_outputs(ref_kernels):
    """The oracle's prefix-table search against outputs of the reference's own indexing.c."""
    for name in ("idx_a", "idx_b", "idx_c"):
        states = ref_kernels[name + "_states"]
        needles = ref_kernels[name + "_needles"]
        expected = ref_kernels[name + "_indices"]
        nbits, prefix = (int(v) for v in ref_kernels[name + "_meta"])
        got = np.searchsorted(states, needles)
        got = np.where((got < len(states)) & (states[np.minimum(got, len(states) - 1)] == needles), got, -1)
        assert np.array_equal(got, expected)


def test_reference_term_generation_outputs(ref_kernels):
    """The product's and the oracle's term semantics against the reference's own reference.c."""
    r = ref_kernels
    alphas, xs = r["apply_alphas"], r["apply_xs"]
    off = (r["apply_off_m"], r["apply_off_l"], r["apply_off_r"], r["apply_off_x"], r["apply_off_s"])
    v = r["apply_off_v"]
    betas, coeffs, offsets = [], [], [0]
    for a, xv in zip(alphas, xs):
        for t in range(len(v)):
            m, l, rr, x, s = (int(arr[t]) for arr in off)
            if (int(a) & m) == rr:
                sign = -1 if bin(int(a) & s).count("1") % 2 else 1
                betas.append(int(a) ^ x)
                coeffs.append(v[t] * sign * xv)
        offsets.append(len(betas))
    assert np.array_equal(np.array(betas, dtype=np.uint64), r["apply_betas"])
    assert np.array_equal(np.array(coeffs), r["apply_coeffs"])
    assert np.array_equal(np.array(offsets), r["apply_offsets"])


@pytest.mark.skipif(not os.path.exists(O.REF_LIB), reason="reference kernels not built here")
def test_oracle_index_against_compiled_reference(ref_kernels):
    """Direct call into the compiled reference (only where the reference tree exists)."""
    import ctypes
    L = ctypes.CDLL(O.REF_LIB)
    assert hasattr(L, "ls_hs_state_index_binary_search_kernel")


@pytest.mark.parametrize("make", [lambda g: config1_case(g), lambda g: chain_case(16, k=8, p=1, inv=-1),
                                  lambda g: square_case(4, 2, 2, inv=1, J2=0.5)])
def test_exact_norms_equal_reference_norms_in_real_sectors(goldens, make):
    """In real sectors the reference's floating stabiliser sums are exact, so the exact-norm
    checker reproduces the reference's scatter bit for bit."""
    case = make(goldens)
    reps = case.oracle_states()
    rng = np.random.default_rng(6)
    x = rng.normal(size=len(reps))
    y_ref = case.oracle_matvec(reps, x, exact_norms=False)
    y_exact = case.oracle_matvec(reps, x, exact_norms=True)
    assert np.array_equal(y_ref, y_exact)


@pytest.mark.parametrize("n,k", [(14, 3), (13, 5), (16, 4), (20, 3)])
def test_reference_rule_basis_has_no_noise_states(n, k):
    """The reference keeps a state iff its floating stabiliser sum is > 0; in these complex
    sectors that decision agrees with the exact one (no state with a non-trivial stabiliser
    character survives), so the bit-exact basis is also the correct one."""
    case = chain_case(n, k=k, h=n // 2)
    reps = case.oracle_states()
    _, cnt = O.orbit_exact(case.group, reps)
    assert np.all(cnt > 0)


def test_oracle_baseline_path_equals_checker():
    """The Benes/prefix-index/atomic baseline path computes the same H x as the checker path."""
    case = chain_case(16, k=0, p=0, inv=1)
    reps = case.oracle_states()
    rng = np.random.default_rng(3)
    x = rng.normal(size=len(reps))
    y1 = case.oracle_matvec(reps, x)
    norms = case.oracle_norms(reps)
    y2, st = O.matvec(case.group, 2, case.inv, case.nbits, reps, norms, case.off, case.diag, x, baseline=True)
    assert st == 0
    assert np.linalg.norm(y1 - y2) <= 1e-13 * np.linalg.norm(y1)


def test_gather_formula_equals_reference_scatter():
    """Dense check of the gather identity used by the GPU kernels on a complex sector:
    H[i, j] = sum_t [a_i & m == l] v (-1)^pop(beta & s) conj(chi) n_j / n_i."""
    n = 12
    case = chain_case(n, k=3, p=None, inv=None, h=6)
    reps = case.oracle_states()
    D = len(reps)
    H = np.zeros((D, D), dtype=np.complex128)
    for j in range(D):
        x = np.zeros(D, dtype=np.complex128)
        x[j] = 1
        H[:, j] = case.oracle_matvec(reps, x, complex_=True)
    reps_l = [int(r) for r in reps]
    idx = {r: i for i, r in enumerate(reps_l)}
    _, chars, norms = O.state_info(case.group, reps)
    v, m, l, rr, xx, s = case.op._off_arrays
    Hg = np.zeros_like(H)
    for i, a in enumerate(reps_l):
        for t in range(len(v)):
            if (a & int(m[t])) != int(l[t]):
                continue
            beta = a ^ int(xx[t])
            sign = -1 if bin(beta & int(s[t])).count("1") % 2 else 1
            rep, chi, nb = O.state_info(case.group, np.array([beta], dtype=np.uint64))
            if nb[0] == 0 or int(rep[0]) not in idx:
                continue
            j = idx[int(rep[0])]
            Hg[i, j] += v[t] * sign * np.conj(chi[0]) * nb[0] / norms[i]
    dv, dm, dl, dr, dx, ds = case.op._diag_arrays
    for i, a in enumerate(reps_l):
        for t in range(len(dv)):
            if (a & int(dm[t])) == int(dr[t]):
                Hg[i, i] += dv[t] * (-1 if bin(a & int(ds[t])).count("1") % 2 else 1)
    assert np.abs(H - Hg).max() < 1e-12
    assert np.abs(H - H.conj().T).max() < 1e-12
