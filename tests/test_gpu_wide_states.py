"""States that use all 64 bits (and 63): the packed tables need spare low bits, so these bases
run the fallback orbit-scan kernel; results must still equal the oracle bit for bit / to 1e-12."""

import numpy as np
import pytest

from ls_helpers import LAT, Case, ls

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,h,k", [(64, 2, 0), (64, 2, 5), (63, 2, 1), (64, 3, 0)])
def test_wide_chain_sectors_match_oracle(n, h, k):
    import torch
    basis = ls.SpinBasis(n, h, None, ls.Symmetries(LAT.chain_symmetries(n, k)))
    case = Case(basis, LAT.heisenberg(LAT.chain_bonds(n)))
    basis.build()
    states = np.asarray(basis.states)
    ref = case.oracle_states()
    assert np.array_equal(states, ref)
    assert np.array_equal(basis.index(states), np.arange(len(states)))
    rng = np.random.default_rng(n + h + k)
    x = rng.normal(size=len(states)) + 1j * rng.normal(size=len(states))
    y = case.op.apply_device(torch.from_numpy(x).cuda()).cpu().numpy()
    yo = case.oracle_matvec(states, x, complex_=True)
    assert np.linalg.norm(y - yo) <= 1e-12 * np.linalg.norm(yo)
