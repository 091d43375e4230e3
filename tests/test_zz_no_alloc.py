"""ls_gpu_enumerate_noalloc: the basis enumeration for callers that cannot allocate device memory
(code under a framework that owns every device allocation, or between stream captures).

It must produce exactly the representatives of the allocating entry point
(ls_hs_build_representatives), call after call, although every call reuses the same static
scratch array.  This file is collected last so that a failure here leaves every other test run.
"""

import ctypes
import json
import os
import subprocess
import sys

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
    # spinful fermions with lattice symmetries (fermionic permutation signs in the scratch tables)
    "hubbard3x3_gamma_3_2": lambda: ls.SpinfulFermionBasis(
        9, (3, 2), symmetries=ls.Symmetries(LAT.square_symmetries(3, 0, 0, True))),
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


def test_noalloc_rejects_too_many_candidates():
    """A projected basis whose candidate range needs more tiles than the static array holds is
    rejected before any launch, with a message, and the entry point keeps working."""
    import torch
    big = ls.SpinBasis(40, 20, None, ls.Symmetries(LAT.chain_symmetries(40, 0)))
    lib = ls._native.lib()
    out = torch.zeros(1, dtype=torch.int64, device="cuda")
    count = ctypes.c_int64(-7)
    rc = lib.ls_gpu_enumerate_noalloc(big._payload, out.data_ptr(), 1, ctypes.byref(count),
                                      torch.cuda.current_stream().cuda_stream)
    assert rc == LS_GPU_ERR_INVALID
    assert "too large" in lib.ls_gpu_last_error().decode()
    basis = BASES["square4_pipi"]()
    basis.build()
    rc, count, got, msg = _noalloc_states(basis)
    assert rc == 0 and np.array_equal(got, basis.states)


# Run in a fresh process: the allocation-free entry point is the library's first call on the
# device that reaches the CUDA runtime past module loading, and the free device memory reported
# by cudaMemGetInfo is the same before and after it.  Modules load eagerly, and a first call that
# is rejected on its size loads this library's module (with its static array) before the
# measurement starts.
_FRESH = r"""
import ctypes, importlib, json, sys
import numpy as np
import torch
sys.path.insert(0, sys.argv[1])
ls = importlib.import_module("lattice-symmetries_gb300")
lat = importlib.import_module("lattice-symmetries_gb300.lattices")
lib = ls._native.lib()
torch.cuda.init()
stream = torch.cuda.current_stream().cuda_stream
out = torch.full((4096,), -1, dtype=torch.int64, device="cuda")
big = ls.SpinBasis(40, 20, None, ls.Symmetries(lat.chain_symmetries(40, 0)))
count = ctypes.c_int64(0)
rc_big = lib.ls_gpu_enumerate_noalloc(big._payload, out.data_ptr(), 1, ctypes.byref(count), stream)
basis = ls.SpinBasis(16, 8, 1, ls.Symmetries(lat.square_symmetries(4, 2, 2)))
torch.cuda.synchronize()
free0 = torch.cuda.mem_get_info()[0]
results = []
for _ in range(2):
    rc = lib.ls_gpu_enumerate_noalloc(basis._payload, out.data_ptr(), out.numel(), ctypes.byref(count), stream)
    torch.cuda.synchronize()
    results.append((rc, count.value, torch.cuda.mem_get_info()[0]))
got = out.cpu().numpy().view(np.uint64)[:count.value].tolist()
basis.build()
print(json.dumps({"rc_big": rc_big, "free0": free0, "calls": results,
                  "equal": got == np.asarray(basis.states).tolist(), "n": basis.number_states}))
"""


def test_noalloc_first_call_allocates_nothing():
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, CUDA_MODULE_LOADING="EAGER")
    res = subprocess.run([sys.executable, "-c", _FRESH, repo], capture_output=True, text=True, env=env,
                         timeout=600)
    assert res.returncode == 0, res.stderr[-2000:]
    d = json.loads(res.stdout.strip().splitlines()[-1])
    assert d["rc_big"] == LS_GPU_ERR_INVALID
    for rc, count, free in d["calls"]:
        assert rc == 0 and count == d["n"]
        assert free == d["free0"], "free device memory changed by {} bytes".format(d["free0"] - free)
    assert d["equal"]
