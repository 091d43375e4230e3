"""ls_gpu_enumerate_noalloc: the basis enumeration for callers that cannot allocate device memory
(code under a framework that owns every device allocation, or between stream captures).

It must produce exactly the representatives of the allocating entry point
(ls_hs_build_representatives), call after call, although every call reuses the same static
scratch array.  This file is collected last so that a failure here leaves every other test run.
"""

import ctypes

import numpy as np
import pytest

from ls_helpers import LAT, ls

pytestmark = pytest.mark.gpu

LS_GPU_ERR_INVALID = -1


def _noalloc_states(basis, capacity=None):
    import torch
    lib = ls._native.lib()
    n_ref = basis.number_states
    cap = n_ref if capacity is None else capacity
    out = torch.full((max(cap, 1),), -1, dtype=torch.int64, device="cuda")
    count = ctypes.c_int64(-7)
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.ls_gpu_enumerate_noalloc(basis._payload, out.data_ptr(), cap, ctypes.byref(count), stream)
    msg = lib.ls_gpu_last_error().decode()
    return rc, count.value, out.cpu().numpy().view(np.uint64)[:cap], msg


BASES = {
    "square4_pipi": lambda: ls.SpinBasis(16, 8, 1, ls.Symmetries(LAT.square_symmetries(4, 2, 2))),
    "chain20_k3": lambda: ls.SpinBasis(20, 10, None, ls.Symmetries(LAT.chain_symmetries(20, 3))),
    "chain24_k0_p0_z1": lambda: ls.SpinBasis(24, 12, 1, ls.Symmetries(LAT.chain_symmetries(24, 0, 0))),
    "hubbard8_4_4": lambda: ls.SpinfulFermionBasis(8, (4, 4)),
    "chain14_free": lambda: ls.SpinBasis(14),
}


@pytest.mark.parametrize("name", sorted(BASES))
def test_noalloc_enumeration_matches_allocating_path_twice(name):
    basis = BASES[name]()
    basis.build()
    expected = np.asarray(basis.states)
    for call in range(2):  # the second call sees the previous call's scratch contents
        rc, count, got, msg = _noalloc_states(basis)
        assert rc == 0, msg
        assert count == len(expected)
        assert np.array_equal(got, expected), "call {} differs".format(call)


def test_noalloc_rejects_small_capacity():
    basis = ls.SpinBasis(16, 8, 1, ls.Symmetries(LAT.square_symmetries(4, 2, 2)))
    basis.build()
    n = basis.number_states
    rc, count, got, msg = _noalloc_states(basis, capacity=n - 1)
    assert rc == LS_GPU_ERR_INVALID
    assert count == n
    assert "capacity" in msg
    # nothing beyond the capacity was touched, and the entry point still works afterwards
    rc, count, got, msg = _noalloc_states(basis)
    assert rc == 0 and count == n and np.array_equal(got, basis.states)
