"""ctypes view of libls_gb300.so (include/ls_gb300.h).

The struct layouts restate kernels/lattice_symmetries_types.h of the reference.  The library is
loaded from ``_lib/libls_gb300.so`` next to this file; importing this module never falls back
to anything else: a missing library raises ImportError.
"""

from __future__ import annotations

import ctypes
import os
import threading
from ctypes import (CFUNCTYPE, POINTER, Structure, c_bool, c_char_p, c_double, c_int, c_int32,
                    c_int64, c_size_t, c_ssize_t, c_uint8, c_uint64, c_void_p)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libls_gb300.so")


class chpl_external_array(Structure):
    _fields_ = [("elts", c_void_p), ("num_elts", c_uint64), ("freer", c_void_p)]


class ls_hs_basis_kernels(Structure):
    _fields_ = [
        ("state_info_kernel", c_void_p),
        ("state_info_data", c_void_p),
        ("is_representative_kernel", c_void_p),
        ("is_representative_data", c_void_p),
        ("state_index_kernel", c_void_p),
        ("state_index_data", c_void_p),
    ]


class ls_hs_permutation_group(Structure):
    _fields_ = [
        ("refcount", c_int),
        ("number_bits", c_int),
        ("number_shifts", c_int),
        ("number_masks", c_int),
        ("masks", POINTER(c_uint64)),
        ("shifts", POINTER(c_uint64)),
        ("eigvals_re", POINTER(c_double)),
        ("eigvals_im", POINTER(c_double)),
        ("haskell_payload", c_void_p),
    ]


LS_HS_SPIN, LS_HS_SPINFUL_FERMION, LS_HS_SPINLESS_FERMION = 0, 1, 2


class ls_hs_basis(Structure):
    _fields_ = [
        ("refcount", c_int),
        ("number_sites", c_int),
        ("number_particles", c_int),
        ("number_up", c_int),
        ("particle_type", c_int),
        ("spin_inversion", c_int),
        ("state_index_is_identity", c_bool),
        ("requires_projection", c_bool),
        ("kernels", POINTER(ls_hs_basis_kernels)),
        ("representatives", chpl_external_array),
        ("haskell_payload", c_void_p),
    ]


class ls_hs_nonbranching_terms(Structure):
    _fields_ = [
        ("number_terms", c_int),
        ("number_bits", c_int),
        ("v", POINTER(c_double)),
        ("m", POINTER(c_uint64)),
        ("l", POINTER(c_uint64)),
        ("r", POINTER(c_uint64)),
        ("x", POINTER(c_uint64)),
        ("s", POINTER(c_uint64)),
    ]


class ls_hs_operator(Structure):
    _fields_ = [
        ("refcount", c_int),
        ("basis", POINTER(ls_hs_basis)),
        ("off_diag_terms", POINTER(ls_hs_nonbranching_terms)),
        ("diag_terms", POINTER(ls_hs_nonbranching_terms)),
        ("haskell_payload", c_void_p),
    ]


class ls_chpl_kernels(Structure):
    _fields_ = [
        ("enumerate_states", c_void_p),
        ("operator_apply_off_diag", c_void_p),
        ("operator_apply_diag", c_void_p),
        ("matrix_vector_product", c_void_p),
    ]


ERROR_HANDLER = CFUNCTYPE(None, c_char_p)

_errors = threading.local()


def _record_error(message):
    lst = getattr(_errors, "messages", None)
    if lst is None:
        lst = []
        _errors.messages = lst
    lst.append(message.decode("utf-8", "replace") if message else "unknown error")


_handler = ERROR_HANDLER(_record_error)

# (name, restype, argtypes) of every function this module binds.
_SIGNATURES = [
    ("ls_hs_set_exception_handler", None, [c_void_p]),
    ("ls_hs_error", None, [c_char_p]),
    ("ls_hs_internal_destroy_external_array", None, [POINTER(chpl_external_array)]),
    ("ls_hs_internal_get_chpl_kernels", POINTER(ls_chpl_kernels), []),
    ("ls_hs_internal_set_chpl_kernels", None, [POINTER(ls_chpl_kernels)]),
    ("ls_chpl_init", None, []),
    ("ls_chpl_finalize", None, []),
    ("ls_internal_create_halide_kernel_data", c_void_p, [POINTER(ls_hs_permutation_group), c_int]),
    ("ls_internal_destroy_halide_kernel_data", None, [c_void_p]),
    ("ls_gpu_create_fermionic_kernel_data", c_void_p, [POINTER(ls_hs_permutation_group), c_int]),
    ("ls_hs_state_info", None, [POINTER(ls_hs_basis), c_ssize_t, POINTER(c_uint64), c_ssize_t,
                                POINTER(c_uint64), c_ssize_t, POINTER(c_double), POINTER(c_double)]),
    ("ls_hs_is_representative", None, [POINTER(ls_hs_basis), c_ssize_t, POINTER(c_uint64), c_ssize_t,
                                       POINTER(c_uint8), POINTER(c_double)]),
    ("ls_hs_state_index", None, [POINTER(ls_hs_basis), c_ssize_t, POINTER(c_uint64), c_ssize_t,
                                 POINTER(c_int64), c_ssize_t]),
    ("ls_hs_build_representatives", None, [POINTER(ls_hs_basis), c_uint64, c_uint64]),
    ("ls_hs_unchecked_set_representatives", None, [POINTER(ls_hs_basis), POINTER(chpl_external_array), c_int]),
    ("ls_hs_create_state_index_binary_search_kernel_data", c_void_p, [POINTER(chpl_external_array), c_int, c_int]),
    ("ls_hs_destroy_state_index_binary_search_kernel_data", None, [c_void_p]),
    ("ls_hs_fixed_hamming_state_to_index", c_ssize_t, [c_uint64]),
    ("ls_hs_fixed_hamming_index_to_state", c_uint64, [c_ssize_t, c_int]),
    ("ls_internal_operator_apply_diag_x1", None, [POINTER(ls_hs_operator), c_ssize_t, POINTER(c_uint64),
                                                  POINTER(c_double), POINTER(c_double)]),
    ("ls_internal_operator_apply_off_diag_x1", None, [POINTER(ls_hs_operator), c_ssize_t, POINTER(c_uint64),
                                                      POINTER(c_uint64), POINTER(c_double), POINTER(c_ssize_t),
                                                      POINTER(c_double)]),
    ("ls_chpl_enumerate_representatives", None, [POINTER(ls_hs_basis), c_uint64, c_uint64,
                                                 POINTER(chpl_external_array)]),
    ("ls_chpl_operator_apply_diag", None, [POINTER(ls_hs_operator), c_int64, POINTER(c_uint64),
                                           POINTER(chpl_external_array), c_int64]),
    ("ls_chpl_operator_apply_off_diag", None, [POINTER(ls_hs_operator), c_int64, POINTER(c_uint64),
                                               POINTER(chpl_external_array), POINTER(chpl_external_array),
                                               POINTER(chpl_external_array), c_int64]),
    ("ls_chpl_matrix_vector_product", None, [POINTER(ls_hs_operator), c_int, POINTER(c_double),
                                             POINTER(c_double)]),
    ("ls_gpu_last_error", c_char_p, []),
    ("ls_gpu_device_synchronize", c_int, []),
    ("ls_gpu_basis_info", c_int, [POINTER(ls_hs_basis), POINTER(c_int64), POINTER(c_void_p), POINTER(c_void_p)]),
    ("ls_gpu_matvec_c128", c_int, [POINTER(ls_hs_operator), c_int, c_void_p, c_int64, c_void_p, c_int64,
                                   c_int, c_void_p]),
    ("ls_gpu_matvec_f64", c_int, [POINTER(ls_hs_operator), c_int, c_void_p, c_int64, c_void_p, c_int64,
                                  c_int, c_void_p]),
    ("ls_gpu_coupling_inner_products", c_int, [POINTER(ls_hs_operator), c_int, POINTER(c_int32), c_void_p,
                                               c_void_p, c_void_p, c_void_p]),
    ("ls_gpu_matvec_multi_sector_c128", c_int, [c_int, POINTER(POINTER(ls_hs_operator)), c_int,
                                                POINTER(c_void_p), POINTER(c_void_p), c_int, c_void_p]),
    ("ls_gpu_sector_plan_create", c_int, [c_int, POINTER(POINTER(ls_hs_operator)), c_int, POINTER(c_void_p),
                                          c_int64, POINTER(c_void_p), c_int64, c_int, POINTER(c_void_p)]),
    ("ls_gpu_sector_plan_run", c_int, [c_void_p, c_void_p]),
    ("ls_gpu_set_enumeration_rule", c_int, [c_int]),
    ("ls_gpu_release_operator", None, [POINTER(ls_hs_operator)]),
    ("ls_gpu_operator_apply_diag", c_int, [POINTER(ls_hs_operator), c_int64, c_void_p, c_void_p, c_void_p]),
    ("ls_gpu_operator_apply_off_diag", c_int, [POINTER(ls_hs_operator), c_int64, c_void_p, c_void_p, c_void_p,
                                               c_void_p, c_void_p]),
    ("ls_gpu_sector_plan_is_batched", c_int, [c_void_p]),
    ("ls_gpu_sector_plan_destroy", c_int, [c_void_p]),
    ("ls_gpu_state_info", c_int, [POINTER(ls_hs_basis), c_int64, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    ("ls_gpu_is_representative", c_int, [POINTER(ls_hs_basis), c_int64, c_void_p, c_void_p, c_void_p, c_void_p]),
    ("ls_gpu_state_index", c_int, [POINTER(ls_hs_basis), c_int64, c_void_p, c_void_p, c_void_p]),
    ("ls_gpu_set_matvec_config", c_int, [c_int, c_int]),
    ("ls_gpu_set_matvec_rhs_tile", c_int, [c_int]),
    ("ls_gpu_get_matvec_config", c_int, [POINTER(c_int), POINTER(c_int), POINTER(c_int)]),
    ("ls_gpu_check_errors", c_int, [c_void_p]),
    ("ls_gpu_enumerate_noalloc", c_int, [POINTER(ls_hs_basis), c_void_p, c_int64, POINTER(c_int64), c_void_p]),
    ("ls_gpu_autotune_matvec", c_int, [POINTER(ls_hs_operator), c_int, POINTER(c_int), POINTER(c_int),
                                       POINTER(c_double)]),
    ("ls_gpu_count_nonzeros", c_int, [POINTER(ls_hs_operator), POINTER(c_int64)]),
    ("ls_gpu_matvec_kernel_info", c_int, [POINTER(ls_hs_operator), POINTER(c_int), POINTER(c_int)]),
    ("ls_gpu_set_tracing", c_int, [c_int]),
    ("ls_gpu_trace_report", c_int, [c_void_p, c_size_t, c_int]),
    ("ls_gpu_sector_plan_set_batched", c_int, [c_void_p, c_int]),
    ("ls_gpu_sector_plan_autotune", c_int, [c_void_p, c_void_p, POINTER(c_int), POINTER(c_double),
                                            POINTER(c_double)]),
    ("ls_gpu_set_block_arithmetic", c_int, [c_int]),
    ("ls_gpu_get_block_arithmetic", c_int, []),
    ("ls_gpu_block_gram", c_int, [c_int64, c_int64, c_int, c_void_p, c_void_p, c_void_p, c_void_p]),
    ("ls_gpu_block_update", c_int, [c_int64, c_int64, c_int, c_double, c_void_p, c_void_p, c_void_p, c_void_p,
                                    c_void_p, c_void_p, c_void_p]),
    ("ls_gpu_block_gram_tc", c_int, [c_int64, c_int64, c_int, c_void_p, c_void_p, c_void_p, c_void_p]),
    ("ls_gpu_block_update_tc", c_int, [c_int64, c_int64, c_int, c_double, c_void_p, c_void_p, c_void_p,
                                       c_void_p, c_void_p, c_void_p, c_void_p]),
]

_lib = None
_lock = threading.Lock()


def load(path: str = LIB_PATH):
    """Loads libls_gb300.so and installs the Python error handler (raises ImportError if absent)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise ImportError(
                "libls_gb300.so not found at {}; build it with "
                "`python lattice-symmetries_gb300/build_native.py`".format(path))
        lib = ctypes.CDLL(path, mode=ctypes.RTLD_GLOBAL)
        for name, res, args in _SIGNATURES:
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        lib.ls_hs_set_exception_handler(ctypes.cast(_handler, c_void_p))
        _lib = lib
        return lib


def lib():
    return load()


def take_errors():
    lst = getattr(_errors, "messages", None)
    if not lst:
        return []
    out = list(lst)
    lst.clear()
    return out


def check(rc=None, what="call"):
    """Raises RuntimeError if the library reported an error through the handler or a status code."""
    msgs = take_errors()
    if msgs:
        raise RuntimeError("; ".join(msgs))
    if rc is not None and rc != 0:
        raise RuntimeError("{} failed ({}): {}".format(what, rc, lib().ls_gpu_last_error().decode()))


def fn_address(name: str) -> int:
    return ctypes.cast(getattr(lib(), name), c_void_p).value


def as_ptr(arr, ctype):
    return arr.ctypes.data_as(POINTER(ctype))
