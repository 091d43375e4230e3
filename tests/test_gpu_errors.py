"""Error paths of the additive entry points: they report through status codes and messages and
leave the library usable (no device trap)."""

import importlib

import numpy as np
import pytest

from ls_helpers import LAT, ls

pytestmark = pytest.mark.gpu
ag = importlib.import_module("lattice-symmetries_gb300.autograd")


def chain_op(n, k, J=1.0):
    b = ls.SpinBasis(n, n // 2, None, ls.Symmetries(LAT.chain_symmetries(n, k)))
    b.build()
    return ls.Operator(b, LAT.heisenberg(LAT.chain_bonds(n), J))


def test_plan_rejects_a_changed_operator():
    ops = [chain_op(12, k) for k in (0, 1, 2)]
    batch = ls.SectorBatch(ops, k=4)
    batch.run(check=True)
    ops[1]._off_arrays[0][:] *= 2.0  # terms changed after the plan was made
    with pytest.raises(RuntimeError, match="changed after the plan was created"):
        batch.run()


def test_invalid_launch_settings_are_rejected():
    lib = ls._native.lib()
    assert lib.ls_gpu_set_matvec_rhs_tile(3) != 0
    assert "1, 4, 8 or 16" in lib.ls_gpu_last_error().decode()
    assert lib.ls_gpu_set_matvec_rhs_tile(16) == 0


def test_particle_number_breaking_term_in_batched_and_coupling_kernels():
    import torch
    n = 12
    b = ls.SpinBasis(n, n // 2, None, ls.Symmetries(LAT.chain_symmetries(n, 0)))
    b.build()
    bad = LAT.heisenberg(LAT.chain_bonds(n)) + ls.Expr("σˣ₀", sites=[[i] for i in range(n)])
    op = ls.Operator(b, bad)
    batch = ls.SectorBatch([op], k=1)
    batch.X[0, : b.number_states] = 1.0
    with pytest.raises(RuntimeError, match="particle numbers"):
        batch.run(check=True)
    pop = ag.ParametrizedOperator(b, [LAT.heisenberg(LAT.chain_bonds(n)),
                                      ls.Expr("σˣ₀", sites=[[i] for i in range(n)])])
    x = torch.ones(b.number_states, dtype=torch.complex128, device="cuda")
    with pytest.raises(RuntimeError, match="particle numbers"):
        pop.coupling_products(x, x)
    # the library is still usable afterwards
    good = chain_op(n, 0)
    y = good.apply_device(x)
    assert torch.isfinite(y).all()


def test_released_operator_is_reuploaded():
    import torch
    op = chain_op(14, 2)
    x = torch.from_numpy(np.random.default_rng(0).normal(size=op.basis.number_states) + 0j).cuda()
    y1 = op.apply_device(x)
    ls._native.lib().ls_gpu_release_operator(op._payload)
    y2 = op.apply_device(x)
    assert torch.equal(y1, y2)
