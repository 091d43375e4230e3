"""Host logic of ParametrizedOperator (coupling tags and re-parametrisation), checked with the
oracle on CPU: H(theta) assembled from tagged unit terms equals the merged sum_c theta_c H_c."""

import importlib

import numpy as np
import pytest

from ls_helpers import LAT, Case, ls

ag = importlib.import_module("lattice-symmetries_gb300.autograd")


def ladder_parts(n_rungs):
    legs, rungs = LAT.ladder(n_rungs)
    return [LAT.heisenberg(legs, 0.25), LAT.heisenberg(rungs, 0.25), LAT.dm_z(legs, 1.0)]


def test_coupling_tags_and_scaling():
    n = 4
    basis = ls.SpinBasis(2 * n, n, None, ls.Symmetries(LAT.ladder_symmetries(n, 0, 0)))
    parts = ladder_parts(n)
    pop = ag.ParametrizedOperator(basis, parts, theta=[1.0, 0.7, 0.2])
    n_off = pop.operator.number_off_diag_terms
    n_diag = pop.operator.number_diag_terms
    assert len(pop.term_coupling) == n_off + n_diag
    assert set(pop.term_coupling.tolist()) == {0, 1, 2}
    per = [ls.Operator(basis, e) for e in parts]
    assert n_off == sum(o.number_off_diag_terms for o in per)
    assert n_diag == sum(o.number_diag_terms for o in per)
    v_unit = pop.generator._off_arrays[0]
    v = pop.operator._off_arrays[0]
    theta = np.array([1.0, 0.7, 0.2])
    assert np.allclose(v, v_unit * theta[pop.term_coupling[:n_off]])
    pop.set_theta([2.0, 0.0, -1.0])
    assert np.allclose(v, v_unit * np.array([2.0, 0.0, -1.0])[pop.term_coupling[:n_off]])


@pytest.mark.parametrize("theta", [[1.0, 0.7, 0.2], [0.3, -1.1, 2.5]])
def test_tagged_terms_equal_merged_expression(theta):
    n = 4
    basis = ls.SpinBasis(2 * n, n, None, ls.Symmetries(LAT.ladder_symmetries(n, 1, 0)))
    parts = ladder_parts(n)
    pop = ag.ParametrizedOperator(basis, parts, theta=theta)
    merged = parts[0].scale(theta[0]) + parts[1].scale(theta[1]) + parts[2].scale(theta[2])
    ref = Case(basis, merged)
    states = ref.oracle_states()
    tagged = Case(basis, merged)
    from ls_helpers import oracle_terms
    tagged.off, tagged.diag = oracle_terms(pop.operator)
    rng = np.random.default_rng(1)
    x = rng.normal(size=len(states)) + 1j * rng.normal(size=len(states))
    y1 = ref.oracle_matvec(states, x, complex_=True)
    y2 = tagged.oracle_matvec(states, x, complex_=True)
    assert np.linalg.norm(y1 - y2) <= 1e-13 * np.linalg.norm(y1)


def test_theta_must_be_double_precision():
    torch = pytest.importorskip("torch")
    n = 4
    basis = ls.SpinBasis(2 * n, n, None, ls.Symmetries(LAT.ladder_symmetries(n, 0, 0)))
    pop = ag.ParametrizedOperator(basis, ladder_parts(n))
    with pytest.raises(TypeError):
        pop.apply(torch.tensor([1.0, 0.7, 0.2]), None)  # float32: 1e-6 steps would be lost to rounding
