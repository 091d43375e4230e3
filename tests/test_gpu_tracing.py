"""Per-stage timing (ls_gpu_set_tracing / ls_gpu_trace_report): the stages of a basis build and
a matvec are reported with their launch counts and positive times while tracing is on, and
nothing is recorded while it is off (the default)."""

import numpy as np
import pytest

from ls_helpers import LAT, ls

pytestmark = pytest.mark.gpu


def test_stages_of_build_and_matvec():
    import torch
    ls.stage_times(reset=True)
    ls.set_tracing(True)
    try:
        basis = ls.SpinBasis(24, 12, 1, ls.Symmetries(LAT.chain_symmetries(24, 0, 0)))
        basis.build()
        op = ls.Operator(basis, LAT.heisenberg(LAT.chain_bonds(24)))
        x = torch.from_numpy(np.random.default_rng(0).normal(size=basis.number_states) + 0j).cuda()
        op.apply_device(x)
        op.apply_device(x)
        t = ls.stage_times(reset=True)
    finally:
        ls.set_tracing(False)
    for stage in ("basis.enumerate", "basis.enumerate_compact", "basis.index", "basis.orbit_norms",
                  "matvec.prescale", "matvec.kernel"):
        assert stage in t, stage
        count, ms = t[stage]
        assert count >= 1 and ms > 0.0, stage
    assert t["matvec.kernel"][0] == 2
    # off: nothing recorded
    op.apply_device(x)
    assert ls.stage_times(reset=True) == {}
