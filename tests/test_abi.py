"""The C ABI: every symbol of include/ls_gb300.h is exported, struct layouts match the reference's
(kernels/lattice_symmetries_types.h), and host-only entry points behave without a GPU."""

import ctypes
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import REPO
from ls_helpers import ls

N = ls._native
HEADER = os.path.join(REPO, "include", "ls_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"typedef[^;]*;", "", text)
    names = set(re.findall(r"\b((?:ls|chpl__init)_[A-Za-z0-9_]+)\s*\(", text))
    return sorted(n for n in names if not n.endswith("_type"))


def test_every_declared_symbol_is_exported():
    lib = ctypes.CDLL(N.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert missing == []
    assert len(declared_functions()) >= 40


# Started and stopped by the Haskell host library, which stays the host (haskell/cbits/init.c).
HASKELL_RUNTIME = {"ls_hs_init", "ls_hs_exit"}


def test_reference_headers_resolve(goldens):
    """A host linked against the reference's two C headers (kernels/lattice_symmetries_types.h,
    chapel/lib/lattice_symmetries_chapel.h) finds every function it declares in libls_gb300.so,
    apart from the Haskell runtime's start and stop."""
    lib = ctypes.CDLL(N.LIB_PATH)
    declared = goldens["declared_functions"]
    assert set(declared) == {"kernels/lattice_symmetries_types.h", "chapel/lib/lattice_symmetries_chapel.h"}
    names = sorted(set(sum(declared.values(), [])) - HASKELL_RUNTIME)
    assert "ls_chpl_init_kernels" in names and len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert missing == []
    ours = set(declared_functions())
    assert [n for n in names if n not in ours] == []


def test_init_kernels_reinstalls_the_drivers():
    """ls_chpl_init_kernels (LatticeSymmetries.chpl:28-30) puts the library's drivers back into the
    plugin table after a host replaced them; chpl__init_LatticeSymmetries does the same."""
    lib = N.lib()
    lib.ls_chpl_init_kernels.restype = None
    lib.chpl__init_LatticeSymmetries.restype = None
    lib.chpl__init_LatticeSymmetries.argtypes = [ctypes.c_int64, ctypes.c_int32]
    empty = N.ls_chpl_kernels()
    for reinstall in (lambda: lib.ls_chpl_init_kernels(), lambda: lib.chpl__init_LatticeSymmetries(1, 2)):
        lib.ls_hs_internal_set_chpl_kernels(ctypes.byref(empty))
        assert lib.ls_hs_internal_get_chpl_kernels().contents.matrix_vector_product is None
        reinstall()
        k = lib.ls_hs_internal_get_chpl_kernels().contents
        assert k.enumerate_states == N.fn_address("ls_chpl_enumerate_representatives")
        assert k.operator_apply_off_diag == N.fn_address("ls_chpl_operator_apply_off_diag")
        assert k.operator_apply_diag == N.fn_address("ls_chpl_operator_apply_diag")
        assert k.matrix_vector_product == N.fn_address("ls_chpl_matrix_vector_product")


def test_struct_layouts_match_reference(goldens):
    lay = goldens["struct_layouts"]
    prog = r"""
#include <stdio.h>
#include <stddef.h>
#include "ls_gb300.h"
#define F(T, f) printf("%s.%s %zu\n", #T, #f, offsetof(T, f))
#define S(T) printf("sizeof.%s %zu\n", #T, sizeof(T))
int main(void) {
  S(chpl_external_array); S(ls_hs_basis_kernels); S(ls_hs_permutation_group); S(ls_hs_basis);
  S(ls_hs_nonbranching_terms); S(ls_hs_operator); S(ls_chpl_kernels); S(ls_hs_scalar);
  F(ls_hs_permutation_group, masks); F(ls_hs_permutation_group, eigvals_im);
  F(ls_hs_permutation_group, haskell_payload);
  F(ls_hs_basis, particle_type); F(ls_hs_basis, spin_inversion); F(ls_hs_basis, state_index_is_identity);
  F(ls_hs_basis, requires_projection); F(ls_hs_basis, kernels); F(ls_hs_basis, representatives);
  F(ls_hs_basis, haskell_payload);
  F(ls_hs_nonbranching_terms, v); F(ls_hs_nonbranching_terms, s);
  F(ls_hs_operator, basis); F(ls_hs_operator, diag_terms); F(ls_hs_operator, haskell_payload);
  F(ls_chpl_kernels, matrix_vector_product);
  return 0;
}
"""
    with tempfile.TemporaryDirectory() as td:
        src = os.path.join(td, "l.c")
        exe = os.path.join(td, "l")
        open(src, "w").write(prog)
        subprocess.run(["gcc", "-std=c11", "-I", os.path.join(REPO, "include"), src, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    got = {k: int(v) for k, v in (line.split() for line in out.strip().splitlines())}
    for k, v in got.items():
        assert lay[k] == v, k
    # the ctypes mirror used by the Python binding
    assert ctypes.sizeof(N.ls_hs_basis) == lay["sizeof.ls_hs_basis"]
    assert N.ls_hs_basis.representatives.offset == lay["ls_hs_basis.representatives"]
    assert N.ls_hs_basis.kernels.offset == lay["ls_hs_basis.kernels"]
    assert ctypes.sizeof(N.ls_hs_permutation_group) == lay["sizeof.ls_hs_permutation_group"]
    assert ctypes.sizeof(N.ls_hs_operator) == lay["sizeof.ls_hs_operator"]
    assert ctypes.sizeof(N.ls_hs_nonbranching_terms) == lay["sizeof.ls_hs_nonbranching_terms"]


def test_combinadics_match_oracle(oracle):
    lib = N.lib()
    rng = np.random.default_rng(5)
    for _ in range(200):
        h = int(rng.integers(1, 20))
        n = int(rng.integers(h, 40))
        idx = int(rng.integers(0, 1 << 20)) % max(1, int(__import__("math").comb(n, h)))
        s = lib.ls_hs_fixed_hamming_index_to_state(idx, h)
        assert s == oracle.unrank(idx, h)
        assert lib.ls_hs_fixed_hamming_state_to_index(s) == idx


def test_host_term_generation_matches_reference(ref_kernels):
    """ls_internal_operator_apply_{off_diag,diag}_x1 (host) against outputs of reference.c."""
    r = ref_kernels
    n = int(r["apply_n"][0])
    basis = ls.SpinBasis(n)
    expr = ls.Expr("σᶻ₀")  # placeholder; the tables below are written directly
    op = ls.Operator(basis, expr)
    keep = []
    off = ls._api._terms_struct((r["apply_off_v"], r["apply_off_m"], r["apply_off_l"], r["apply_off_r"],
                                 r["apply_off_x"], r["apply_off_s"]), n, keep)
    z = np.zeros(len(r["apply_diag_v"]), dtype=np.uint64)
    diag = ls._api._terms_struct((r["apply_diag_v"], r["apply_diag_m"], r["apply_diag_r"], r["apply_diag_r"],
                                  z, r["apply_diag_s"]), n, keep)
    op._c.off_diag_terms = ctypes.pointer(off)
    op._c.diag_terms = ctypes.pointer(diag)
    alphas = np.ascontiguousarray(r["apply_alphas"])
    xs = np.ascontiguousarray(r["apply_xs"])
    cnt = len(alphas)
    T = len(r["apply_off_v"])
    betas = np.zeros(cnt * T, dtype=np.uint64)
    coeffs = np.zeros(cnt * T, dtype=np.complex128)
    offsets = np.zeros(cnt + 1, dtype=np.int64)
    lib = N.lib()
    lib.ls_internal_operator_apply_off_diag_x1(op._payload, cnt, N.as_ptr(alphas, ctypes.c_uint64),
                                               N.as_ptr(betas, ctypes.c_uint64),
                                               coeffs.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                               offsets.ctypes.data_as(ctypes.POINTER(ctypes.c_ssize_t)),
                                               N.as_ptr(xs, ctypes.c_double))
    k = offsets[-1]
    assert np.array_equal(offsets, r["apply_offsets"])
    assert np.array_equal(betas[:k], r["apply_betas"])
    assert np.array_equal(coeffs[:k], r["apply_coeffs"])
    ys = np.zeros(cnt)
    lib.ls_internal_operator_apply_diag_x1(op._payload, cnt, N.as_ptr(alphas, ctypes.c_uint64),
                                           N.as_ptr(ys, ctypes.c_double), N.as_ptr(xs, ctypes.c_double))
    assert np.array_equal(ys, r["apply_diag_ys"])


def test_plugin_table_installed_at_load():
    lib = N.lib()
    k = lib.ls_hs_internal_get_chpl_kernels().contents
    assert k.enumerate_states == N.fn_address("ls_chpl_enumerate_representatives")
    assert k.matrix_vector_product == N.fn_address("ls_chpl_matrix_vector_product")


def test_error_handler_routes_to_python():
    lib = N.lib()
    lib.ls_hs_error(b"boom")
    with pytest.raises(RuntimeError, match="boom"):
        N.check()


def test_operator_apply_to_basis_state_host_paths():
    """apply_{diag,off_diag}_to_basis_state (BatchedOperator.chpl:298-357) run on the host."""
    basis = ls.SpinBasis(2)
    op = ls.Operator(basis, ls.Expr("1.0 σᶻ₀ σᶻ₁ + 2.0 σ⁺₀ σ⁻₁ + 2.0 σ⁻₀ σ⁺₁"))
    # python/test/test_api.py:64-69: state 1 = |01> has one off-diagonal neighbour
    out = op.apply_off_diag_to_basis_state(1)
    assert len(out) == 1 and out[0] == (2 + 0j, 2)
    assert op.apply_diag_to_basis_state(1) == -1.0
    assert op.apply_diag_to_basis_state(3) == 1.0


def test_host_side_settings_without_a_gpu():
    """Settings that touch no device: block arithmetic modes, launch-shape validation, invalid
    dense-product shapes and NULL plans are rejected with LS_GPU_ERR_INVALID and a message."""
    lib = N.lib()
    ls_ = __import__("importlib").import_module("lattice-symmetries_gb300")
    assert ls_.Operator.block_arithmetic() == "fp64"
    for mode in ("pairs", "auto", "fp64"):
        assert ls_.Operator.block_arithmetic(mode) == mode
    assert lib.ls_gpu_set_block_arithmetic(-1) == -1
    assert lib.ls_gpu_set_block_arithmetic(3) == -1
    assert ls_.Operator.block_arithmetic() == "fp64"
    assert lib.ls_gpu_set_matvec_config(33, 0) == -1
    assert lib.ls_gpu_set_matvec_config(1056, 0) == -1
    assert lib.ls_gpu_set_matvec_config(0, 65) == -1
    assert lib.ls_gpu_block_gram(1, 10, 17, None, None, None, None) == -1
    assert b"k <= 16" in lib.ls_gpu_last_error()
    assert lib.ls_gpu_block_gram(0, 10, 4, None, None, None, None) == -1
    assert lib.ls_gpu_block_update(1, 10, 4, 1.0, None, None, None, None, None, None, None) == -1
    assert lib.ls_gpu_sector_plan_set_batched(None, 1) == -1
    assert b"not a sector plan" in lib.ls_gpu_last_error()
    # the allocation-free enumeration rejects a NULL output with a non-zero capacity before it
    # touches the device
    basis = ls_.SpinBasis(8, 4)
    count = ctypes.c_int64(-1)
    assert lib.ls_gpu_enumerate_noalloc(basis._payload, None, 70, ctypes.byref(count), None) == -1
    assert b"NULL" in lib.ls_gpu_last_error()
    # per-stage timing: nothing traced, an empty report, on and off again
    assert ls_.stage_times() == {}
    ls_.set_tracing(True)
    assert ls_.stage_times() == {}
    ls_.set_tracing(False)
    N.take_errors()


def test_missing_library_fails_loudly(tmp_path):
    """Without the compiled library the binding raises instead of falling back to a CPU path."""
    import subprocess
    import sys
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    # the binding module alone (the package's __init__ would load the built library first)
    code = ("import importlib.util as u; "
            "s = u.spec_from_file_location('lsg_native', 'lattice-symmetries_gb300/_native.py'); "
            "N = u.module_from_spec(s); s.loader.exec_module(N); "
            "N.load({!r})".format(str(tmp_path / "absent" / "libls_gb300.so")))
    res = subprocess.run([sys.executable, "-c", code], cwd=repo, capture_output=True, text=True)
    assert res.returncode != 0
    assert "ImportError" in res.stderr and "build_native.py" in res.stderr
