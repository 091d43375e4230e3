"""GPU parity: libls_gb300.so (through the C ABI and the Python binding) against the CPU oracle.

Integer outputs (representatives, indices, characters, flags) are compared bit for bit; H*x to
relative L2 <= 1e-12 (the FP64 tolerance of the hot path).
"""

import numpy as np
import pytest

import oracle as O
from ls_helpers import LAT, Case, chain_case, config1_case, ls, square_case

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def rel_l2(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _cases(goldens):
    out = [
        ("config1", lambda: config1_case(goldens)),
        ("chain16_k0_p0_z1", lambda: chain_case(16, k=0, p=0, inv=1)),
        ("chain16_k8_p1_zm1", lambda: chain_case(16, k=8, p=1, inv=-1)),
        ("chain14_k3_h7", lambda: chain_case(14, k=3, h=7)),          # complex sector
        ("chain13_k5_h6", lambda: chain_case(13, k=5, h=6)),          # odd length, complex
        ("square4_pipi_z1", lambda: square_case(4, 2, 2, inv=1, J2=0.5)),
        ("square4_k10_h8", lambda: square_case(4, 1, 0, inv=None, J2=0.5, point_group=False)),
        ("chain12_noh", lambda: chain_case(12, k=0, p=0, inv=None, h=None)),
    ]
    return out


CASE_NAMES = ["config1", "chain16_k0_p0_z1", "chain16_k8_p1_zm1", "chain14_k3_h7", "chain13_k5_h6",
              "square4_pipi_z1", "square4_k10_h8", "chain12_noh"]


@pytest.fixture(scope="module")
def built_cases(goldens):
    cases = {}
    for name, make in _cases(goldens):
        c = make()
        c.basis.build()
        cases[name] = c
    return cases


@pytest.mark.parametrize("name", CASE_NAMES)
def test_enumeration_bit_exact(built_cases, name):
    c = built_cases[name]
    got = c.basis.states
    expected = c.oracle_states()
    assert got.dtype == np.uint64
    assert np.array_equal(got, expected)


@pytest.mark.parametrize("name", CASE_NAMES)
def test_state_info_bit_exact(built_cases, name):
    c = built_cases[name]
    if c.group is None:
        pytest.skip("no permutation group")
    rng = np.random.default_rng(7)
    n = c.nbits
    xs = rng.integers(0, 1 << n, size=4000, dtype=np.uint64)
    xs = np.concatenate([xs, c.basis.states[:2000]])
    reps, chars, norms = c.basis.state_info(xs)
    oreps, ochars, onorms = O.state_info(c.group, xs, lane_width=8)
    _, ocnt = O.orbit_exact(c.group, xs)
    assert np.array_equal(reps, oreps)
    # characters follow the reference's Halide lane order everywhere
    assert np.array_equal(chars, ochars)
    # norms are exact: sqrt(|Stab|/|G|) when the character is trivial on the stabiliser, else 0
    denom = c.group.order * (2 if c.inv else 1)
    assert np.array_equal(norms, np.sqrt(ocnt / denom))
    # and equal to the reference's floating norm wherever that sum is exact
    exact = onorms ** 2 * denom
    ok = np.abs(exact - np.round(exact)) < 1e-9
    assert np.array_equal(norms[ok], onorms[ok])


@pytest.mark.parametrize("name", CASE_NAMES)
def test_is_representative_bit_exact(built_cases, name):
    c = built_cases[name]
    if c.group is None:
        pytest.skip("no permutation group")
    rng = np.random.default_rng(8)
    xs = rng.integers(0, 1 << c.nbits, size=4000, dtype=np.uint64)
    xs = np.concatenate([xs, c.basis.states[:1000]])
    flags, norms = c.basis.is_representative(xs)
    oflags, onorms = O.is_representative(c.group, xs, lane_width=4)
    assert np.array_equal(flags, oflags)
    assert np.array_equal(norms, onorms)


@pytest.mark.parametrize("name", CASE_NAMES)
def test_state_index_bit_exact(built_cases, name):
    c = built_cases[name]
    states = c.basis.states
    idx = c.basis.index(states)
    assert np.array_equal(idx, np.arange(len(states)))
    rng = np.random.default_rng(9)
    probe = rng.integers(0, 1 << c.nbits, size=5000, dtype=np.uint64)
    got = c.basis.index(probe)
    pos = np.searchsorted(states, probe)
    expected = np.where((pos < len(states)) & (states[np.minimum(pos, len(states) - 1)] == probe), pos, -1)
    assert np.array_equal(got, expected)


@pytest.mark.parametrize("name", CASE_NAMES)
def test_matvec_real_matches_reference_semantics(built_cases, name):
    """ls_chpl_matrix_vector_product: real x, real y, real part of the coefficients."""
    c = built_cases[name]
    states = c.basis.states
    rng = np.random.default_rng(1)
    x = rng.normal(size=len(states))
    y = c.op.apply_to_state_vector(x)
    yo = c.oracle_matvec(states, x)
    assert rel_l2(y, yo) <= RTOL


@pytest.mark.parametrize("name", CASE_NAMES)
def test_matvec_complex_matches_oracle(built_cases, name):
    import torch
    c = built_cases[name]
    states = c.basis.states
    rng = np.random.default_rng(2)
    x = rng.normal(size=len(states)) + 1j * rng.normal(size=len(states))
    y = c.op.apply_device(torch.from_numpy(x).cuda()).cpu().numpy()
    yo = c.oracle_matvec(states, x, complex_=True)
    assert rel_l2(y, yo) <= RTOL


@pytest.mark.parametrize("name", ["config1", "chain14_k3_h7", "square4_pipi_z1"])
@pytest.mark.parametrize("k", [2, 4, 8, 16, 21])
def test_block_matvec_equals_columns(built_cases, name, k):
    import torch
    c = built_cases[name]
    D = c.basis.number_states
    rng = np.random.default_rng(k)
    X = torch.from_numpy(rng.normal(size=(D, k)) + 1j * rng.normal(size=(D, k))).cuda()
    Y = c.op.apply_device(X)
    for j in range(k):
        yj = c.op.apply_device(X[:, j].contiguous())
        assert torch.allclose(Y[:, j], yj, rtol=0, atol=1e-12 * float(yj.abs().max()) + 1e-300)


@pytest.mark.parametrize("name", ["chain14_k3_h7", "square4_k10_h8", "chain13_k5_h6"])
def test_adjoint_matvec(built_cases, name):
    """<u, H x> = <H^dagger u, x> for a non-Hermitian operator (sigma^+ sigma^- on one bond
    direction plus a complex DM-like part)."""
    import torch
    c = built_cases[name]
    n = c.nbits
    # the operator must commute with the basis' symmetries: use the lattice's own bonds
    bonds = LAT.square_bonds(4) if name.startswith("square4") else LAT.chain_bonds(n)
    expr = ls.Expr("2 σ⁺₀ σ⁻₁ + (0.5 + 0.25im) σᶻ₀ σᶻ₁", sites=[list(b) for b in bonds])
    op = ls.Operator(c.basis, expr)
    D = c.basis.number_states
    rng = np.random.default_rng(4)
    x = torch.from_numpy(rng.normal(size=D) + 1j * rng.normal(size=D)).cuda()
    u = torch.from_numpy(rng.normal(size=D) + 1j * rng.normal(size=D)).cuda()
    Hx = op.apply_device(x)
    Hdu = op.apply_device(u, adjoint=True)
    lhs = torch.vdot(u, Hx).item()
    rhs = torch.vdot(Hdu, x).item()
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), 1.0)
    # and against the oracle with the adjoint expression
    Hd_op = ls.Operator(c.basis, expr.adjoint())
    case = Case(c.basis, expr.adjoint())
    yo = case.oracle_matvec(c.basis.states, u.cpu().numpy(), complex_=True)
    assert rel_l2(Hdu.cpu().numpy(), yo) <= RTOL
    assert rel_l2(Hd_op.apply_device(u).cpu().numpy(), yo) <= RTOL


def test_n10_chain_eigsh(goldens):
    """python/example/getting_started.py verbatim through scipy's eigsh on the GPU operator."""
    import scipy.sparse.linalg
    g = goldens["n10_chain"]
    sites = np.arange(10)
    T = ls.Symmetry((sites + 1) % 10, sector=5)
    P = ls.Symmetry(sites[::-1], sector=1)
    basis = ls.SpinBasis(number_spins=10, spin_inversion=-1, symmetries=ls.Symmetries([T, P]))
    basis.build()
    expr = ls.Expr(g["expression"], sites=g["sites"])
    H = ls.Operator(basis, expr)
    e, _ = scipy.sparse.linalg.eigsh(H, k=1, which="SA")
    assert np.isclose(e[0], g["energy"])


@pytest.mark.parametrize("idx", range(5))
def test_hphi_energies_on_gpu(goldens, idx):
    import scipy.sparse.linalg
    from test_oracle_pins import _hphi_case
    entry = goldens["hphi"][idx]
    case = _hphi_case(entry)
    case.basis.build()
    assert np.array_equal(case.basis.states, case.oracle_states())
    e, _ = scipy.sparse.linalg.eigsh(case.op, k=1, which="SA", tol=1e-12)
    assert abs(e[0] - entry["energy"]) < 1e-8


def test_spinful_hubbard_goldens(goldens):
    from test_oracle_pins import _hubbard_2site
    h = goldens["hubbard_2site"]
    for name, args in h["bases"].items():
        basis = ls.SpinfulFermionBasis(*args) if len(args) == 1 else ls.SpinfulFermionBasis(args[0], args[1])
        basis.build()
        op = ls.Operator(basis, _hubbard_2site(h["t"], h["U"]))
        D = basis.number_states
        H = np.stack([op.apply_to_state_vector(np.eye(D)[:, j].copy()) for j in range(D)], axis=1)
        assert np.array_equal(H, np.array(h["matrices"][name], dtype=float))


def test_operator_breaking_the_basis_raises(built_cases):
    c = built_cases["chain16_k0_p0_z1"]
    op = ls.Operator(c.basis, ls.Expr("σ⁺₀"))
    with pytest.raises(RuntimeError):
        op.apply_to_state_vector(np.ones(c.basis.number_states))
    # the library stays usable afterwards
    y = c.op.apply_to_state_vector(np.ones(c.basis.number_states))
    assert np.isfinite(y).all()


def test_empty_sector():
    """A sector with no representatives: N=4 chain, Sz=0, momentum 1, inversion -1."""
    basis = ls.SpinBasis(4, spin_inversion=-1, symmetries=ls.Symmetries(LAT.chain_symmetries(4, 1, None)))
    basis.build()
    case = Case(basis, LAT.heisenberg(LAT.chain_bonds(4)))
    assert np.array_equal(basis.states, case.oracle_states())
    y = case.op.apply_to_state_vector(np.zeros(basis.number_states))
    assert y.shape == (basis.number_states,)
