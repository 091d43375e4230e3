"""Generates the golden fixtures under tests/golden/ from the reference source tree.

Run in a container where the reference is present:

    LS_REFERENCE_DIR=<reference source tree> python tests/golden/make_golden.py
    python tests/golden/make_golden.py --reference <reference source tree>

Outputs (all committed, small):
  reference_goldens.json  known answers extracted from the reference's own tests and data:
      * Benes known-answer tests      haskell/test/LatticeSymmetries/BenesSpec.hs:33-41
      * N=10 chain ground state       python/example/getting_started.py:9-51
      * 2-site Hubbard matrices       python/run_tests.py:128-175
      * HPhi ground-state energies    test/0[1-5]_*/hamiltonian.yaml + HPhi/output/zvo_energy.dat
      * lattice configs               chapel/data/heisenberg_chain_24_symm.yaml,
                                      chapel/data/heisenberg_square_6x6.yaml
      * C struct layouts              kernels/lattice_symmetries_types.h (compiled with gcc)
      * declared functions            kernels/lattice_symmetries_types.h,
                                      chapel/lib/lattice_symmetries_chapel.h
  reference_kernels.npz   outputs of the reference's own kernels/indexing.c and kernels/reference.c
                          (built by oracle/Makefile into oracle/_ref) on seeded inputs.
"""

from __future__ import annotations

import argparse
import ast
import ctypes
import json
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


# ------------------------------------------------------------------------------------------------
# A minimal YAML reader for the reference's config files (mappings, "- " lists, flow lists,
# quoted strings, comments, &anchors / *aliases).  PyYAML is not available here.
# ------------------------------------------------------------------------------------------------
def _strip_comment(line: str) -> str:
    out, q = [], None
    for ch in line:
        if q:
            out.append(ch)
            if ch == q:
                q = None
        elif ch in "\"'":
            q = ch
            out.append(ch)
        elif ch == "#":
            break
        else:
            out.append(ch)
    return "".join(out).rstrip()


def _scalar(tok: str, anchors):
    tok = tok.strip()
    if tok.startswith("*"):
        return anchors[tok[1:]]
    if tok.startswith('"') and tok.endswith('"'):
        return tok[1:-1]
    if tok in ("null", "~", ""):
        return None
    if tok in ("true", "false"):
        return tok == "true"
    try:
        return int(tok)
    except ValueError:
        pass
    try:
        return float(tok)
    except ValueError:
        return tok


def _flow(text: str, anchors):
    text = text.strip()
    anchor = None
    if text.startswith("&"):
        anchor, text = text[1:].split(None, 1)
    if text.startswith("*"):
        return anchors[text[1:].strip()]
    if text.startswith("["):
        val = json.loads(text)
    else:
        val = _scalar(text, anchors)
    if anchor:
        anchors[anchor] = val
    return val


def parse_yaml(path: str):
    lines = []
    for raw in open(path, encoding="utf-8").read().splitlines():
        s = _strip_comment(raw)
        if s.strip():
            lines.append(s)
    # join flow sequences that span lines
    joined = []
    buf = None
    depth = 0
    for s in lines:
        if buf is None:
            buf = s
        else:
            buf += " " + s.strip()
        depth = buf.count("[") - buf.count("]")
        if depth <= 0:
            joined.append(buf)
            buf = None
    anchors = {}

    def block(i, indent):
        # returns (value, next_index)
        if i < len(joined) and joined[i].lstrip().startswith("- ") and \
                len(joined[i]) - len(joined[i].lstrip()) == indent:
            items = []
            while i < len(joined) and len(joined[i]) - len(joined[i].lstrip()) == indent and \
                    joined[i].lstrip().startswith("- "):
                content = joined[i].lstrip()[2:]
                sub_indent = indent + 2
                if ":" in content and not content.startswith("["):
                    # mapping inside a list item: rewrite the first key at sub_indent
                    joined[i] = " " * sub_indent + content
                    val, i = mapping(i, sub_indent)
                else:
                    val = _flow(content, anchors)
                    i += 1
                items.append(val)
            return items, i
        return mapping(i, indent)

    def mapping(i, indent):
        out = {}
        while i < len(joined):
            line = joined[i]
            ind = len(line) - len(line.lstrip())
            if ind < indent:
                break
            if ind > indent:
                raise ValueError("bad indentation: " + line)
            key, _, rest = line.strip().partition(":")
            rest = rest.strip()
            if rest == "" or (rest.startswith("&") and len(rest.split()) == 1):
                anchor = rest[1:] if rest.startswith("&") else None
                i += 1
                if i < len(joined):
                    nind = len(joined[i]) - len(joined[i].lstrip())
                    val, i = block(i, nind) if nind > indent or joined[i].lstrip().startswith("- ") else (None, i)
                else:
                    val = None
                if anchor:
                    anchors[anchor] = val
                out[key] = val
            else:
                out[key] = _flow(rest, anchors)
                i += 1
        return out, i

    val, _ = mapping(0, 0)
    return val


# ------------------------------------------------------------------------------------------------
def benes_kats(ref):
    text = open(os.path.join(ref, "haskell/test/LatticeSymmetries/BenesSpec.hs"), encoding="utf-8").read()
    perms = {}
    for name, body in re.findall(r"let (p\S*) = toBenesNetwork \(mkPermutation \[([0-9, ]+)\]\)", text):
        perms[name] = [int(v) for v in body.split(",")]
    for name, body in re.findall(r"(v\S*) = mkPermutation \[([0-9, ]+)\]", text):
        perms["p" + name[1:]] = [int(v) for v in body.split(",")]
    kats = []
    for name, x, y in re.findall(r"permuteBits (p\S*) (0b[01]+) `shouldBe` (0b[01]+)", text):
        kats.append({"permutation": perms[name], "x": int(x, 2), "y": int(y, 2),
                     "source": "haskell/test/LatticeSymmetries/BenesSpec.hs"})
    return kats


def n10_chain(ref):
    path = os.path.join(ref, "python/example/getting_started.py")
    text = open(path, encoding="utf-8").read()
    e0 = float(re.search(r"np\.isclose\(eigenvalues\[0\], (-?[0-9.]+)\)", text).group(1))
    return {"number_spins": 10, "hamming_weight": 5, "spin_inversion": -1,
            "symmetries": [{"permutation": [(i + 1) % 10 for i in range(10)], "sector": 5},
                           {"permutation": list(range(10))[::-1], "sector": 1}],
            "expression": re.search(r'ls\.Expr\("([^"]+)", sites=edges\)', text).group(1),
            "sites": [[i, (i + 1) % 10] for i in range(10)], "energy": e0,
            "source": "python/example/getting_started.py:9-51"}


def hubbard_matrices(ref):
    path = os.path.join(ref, "python/run_tests.py")
    tree = ast.parse(open(path, encoding="utf-8").read())
    out = {}
    for node in ast.walk(tree):
        if isinstance(node, ast.FunctionDef) and node.name.startswith("test_hubbard_hamiltonian_matrix"):
            for sub in ast.walk(node):
                if isinstance(sub, ast.Assign) and getattr(sub.targets[0], "id", "") == "valid_matrix":
                    out[node.name] = ast.literal_eval(sub.value.args[0])
                if isinstance(sub, ast.Call) and getattr(sub.func, "attr", "") == "SpinfulFermionBasis":
                    args = [ast.literal_eval(a) for a in sub.args]
                    out[node.name + ":basis"] = args
    return {"t": 1, "U": 2, "matrices": {k: v for k, v in out.items() if ":" not in k},
            "bases": {k.split(":")[0]: v for k, v in out.items() if ":" in k},
            "hopping": ["c†↑₀ c↑₁", "c†↑₁ c↑₀", "c†↓₁ c↓₀", "c†↓₀ c↓₁"],
            "source": "python/run_tests.py:128-175"}


def hphi(ref):
    out = []
    base = os.path.join(ref, "test")
    for d in sorted(os.listdir(base)):
        y = parse_yaml(os.path.join(base, d, "hamiltonian.yaml"))
        energy = None
        for line in open(os.path.join(base, d, "HPhi/output/zvo_energy.dat")):
            if line.startswith("Energy"):
                energy = float(line.split()[-1])
        out.append({"name": d, "basis": y["basis"], "terms": y["hamiltonian"]["terms"], "energy": energy,
                    "source": "test/{}/hamiltonian.yaml, HPhi/output/zvo_energy.dat".format(d)})
    return out


def chapel_configs(ref):
    out = {}
    for name in ("heisenberg_chain_24_symm", "heisenberg_square_6x6"):
        y = parse_yaml(os.path.join(ref, "chapel/data", name + ".yaml"))
        out[name] = {"basis": y["basis"], "terms": y["hamiltonian"]["terms"],
                     "source": "chapel/data/{}.yaml".format(name)}
    return out


def struct_layouts(ref):
    prog = r"""
#include <stdio.h>
#include <stddef.h>
#include "lattice_symmetries_types.h"
#define F(T, f) printf("\"%s.%s\": %zu,\n", #T, #f, offsetof(T, f))
#define S(T) printf("\"sizeof.%s\": %zu,\n", #T, sizeof(T))
int main(void) {
  printf("{\n");
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
  printf("\"end\": 0}\n");
  return 0;
}
"""
    with tempfile.TemporaryDirectory() as td:
        src = os.path.join(td, "layout.c")
        exe = os.path.join(td, "layout")
        open(src, "w").write(prog)
        subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ref, "kernels"), src, "-o", exe], check=True)
        res = subprocess.run([exe], capture_output=True, text=True, check=True)
    d = json.loads(res.stdout)
    d.pop("end")
    d["source"] = "kernels/lattice_symmetries_types.h compiled with gcc (x86-64 LP64)"
    return d


def reference_kernel_outputs(ref, out_path):
    """Runs the reference's compiled indexing.c / reference.c on seeded inputs."""
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "ref", "REFERENCE=" + ref], check=True)
    L = ctypes.CDLL(os.path.join(REPO, "oracle", "_ref", "libls_ref.so"))

    class ext(ctypes.Structure):
        _fields_ = [("elts", ctypes.c_void_p), ("num_elts", ctypes.c_uint64), ("freer", ctypes.c_void_p)]

    L.ls_hs_create_state_index_binary_search_kernel_data.restype = ctypes.c_void_p
    L.ls_hs_create_state_index_binary_search_kernel_data.argtypes = [ctypes.POINTER(ext), ctypes.c_int, ctypes.c_int]
    L.ls_hs_state_index_binary_search_kernel.argtypes = [ctypes.c_ssize_t, ctypes.c_void_p, ctypes.c_ssize_t,
                                                         ctypes.c_void_p, ctypes.c_ssize_t, ctypes.c_void_p]
    rng = np.random.default_rng(seed=11)
    results = {}
    # index: sorted random states of 30 bits, needles half present half absent
    for name, nbits, n, prefix in (("idx_a", 30, 50000, 22), ("idx_b", 36, 20000, 22), ("idx_c", 12, 300, 22)):
        states = np.unique(rng.integers(0, 1 << nbits, size=n, dtype=np.uint64))
        present = rng.choice(states, size=2000)
        absent = rng.integers(0, 1 << nbits, size=2000, dtype=np.uint64)
        needles = np.concatenate([present, absent]).astype(np.uint64)
        arr = ext(states.ctypes.data, states.size, None)
        data = L.ls_hs_create_state_index_binary_search_kernel_data(ctypes.byref(arr), nbits, prefix)
        idx = np.zeros(needles.size, dtype=np.int64)
        L.ls_hs_state_index_binary_search_kernel(needles.size, needles.ctypes.data, 1, idx.ctypes.data, 1, data)
        results[name + "_states"] = states
        results[name + "_needles"] = needles
        results[name + "_indices"] = idx
        results[name + "_meta"] = np.array([nbits, prefix])
    # term generation: Heisenberg chain N=12 terms (m, l, r, x, s, v) built here, applied by reference.c
    n = 12
    offm, offl, offr, offx, offs, offv = [], [], [], [], [], []
    dm, dr, ds, dv = [], [], [], []
    for i in range(n):
        j = (i + 1) % n
        bi, bj = 1 << i, 1 << j
        # 2 s+_i s-_j : requires bit i = 0, bit j = 1 on the ket
        offm += [bi | bj, bi | bj]
        offl += [bi, bj]
        offr += [bj, bi]
        offx += [bi | bj, bi | bj]
        offs += [0, 0]
        offv += [2.0 + 0.5j, 2.0 - 0.5j]
        dm.append(0)
        dr.append(0)
        ds.append(bi | bj)
        dv.append(1.0 + 0j)

    class terms(ctypes.Structure):
        _fields_ = [("number_terms", ctypes.c_int), ("number_bits", ctypes.c_int), ("v", ctypes.c_void_p),
                    ("m", ctypes.c_void_p), ("l", ctypes.c_void_p), ("r", ctypes.c_void_p),
                    ("x", ctypes.c_void_p), ("s", ctypes.c_void_p)]

    class op(ctypes.Structure):
        _fields_ = [("refcount", ctypes.c_int), ("basis", ctypes.c_void_p), ("off", ctypes.POINTER(terms)),
                    ("diag", ctypes.POINTER(terms)), ("payload", ctypes.c_void_p)]

    A = {k: np.array(v, dtype=np.uint64) for k, v in (("m", offm), ("l", offl), ("r", offr), ("x", offx), ("s", offs))}
    Av = np.array(offv, dtype=np.complex128)
    D = {k: np.array(v, dtype=np.uint64) for k, v in (("m", dm), ("r", dr), ("s", ds))}
    Dv = np.array(dv, dtype=np.complex128)
    toff = terms(len(offv), n, Av.ctypes.data, A["m"].ctypes.data, A["l"].ctypes.data, A["r"].ctypes.data,
                 A["x"].ctypes.data, A["s"].ctypes.data)
    tdiag = terms(len(dv), n, Dv.ctypes.data, D["m"].ctypes.data, D["r"].ctypes.data, D["r"].ctypes.data,
                  np.zeros(len(dv), dtype=np.uint64).ctypes.data, D["s"].ctypes.data)
    zeros_keep = np.zeros(len(dv), dtype=np.uint64)
    tdiag.x = zeros_keep.ctypes.data
    o = op(1, None, ctypes.pointer(toff), ctypes.pointer(tdiag), None)
    alphas = rng.integers(0, 1 << n, size=500, dtype=np.uint64)
    xs = rng.normal(size=500)
    betas = np.zeros(500 * len(offv), dtype=np.uint64)
    coeffs = np.zeros(500 * len(offv), dtype=np.complex128)
    offsets = np.zeros(501, dtype=np.int64)
    L.ls_internal_operator_apply_off_diag_x1(ctypes.byref(o), ctypes.c_ssize_t(500), alphas.ctypes.data_as(ctypes.c_void_p),
                                             betas.ctypes.data_as(ctypes.c_void_p), coeffs.ctypes.data_as(ctypes.c_void_p),
                                             offsets.ctypes.data_as(ctypes.c_void_p), xs.ctypes.data_as(ctypes.c_void_p))
    ys = np.zeros(500)
    L.ls_internal_operator_apply_diag_x1(ctypes.byref(o), ctypes.c_ssize_t(500), alphas.ctypes.data_as(ctypes.c_void_p),
                                         ys.ctypes.data_as(ctypes.c_void_p), xs.ctypes.data_as(ctypes.c_void_p))
    k = int(offsets[-1])
    results.update({"apply_n": np.array([n]), "apply_alphas": alphas, "apply_xs": xs,
                    "apply_off_m": A["m"], "apply_off_l": A["l"], "apply_off_r": A["r"], "apply_off_x": A["x"],
                    "apply_off_s": A["s"], "apply_off_v": Av, "apply_diag_m": D["m"], "apply_diag_r": D["r"],
                    "apply_diag_s": D["s"], "apply_diag_v": Dv,
                    "apply_betas": betas[:k], "apply_coeffs": coeffs[:k], "apply_offsets": offsets,
                    "apply_diag_ys": ys})
    np.savez_compressed(out_path, **results)


def declared_functions(ref):
    """Names of the functions the reference's two C headers declare (a host linked against them
    resolves these symbols)."""
    out = {}
    for rel in ("kernels/lattice_symmetries_types.h", "chapel/lib/lattice_symmetries_chapel.h"):
        text = open(os.path.join(ref, rel), encoding="utf-8").read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        text = re.sub(r"#[^\n]*", "", text)
        text = re.sub(r"typedef[^;]*;", "", text)
        names = re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", text)
        out[rel] = sorted({n for n in names if n.startswith(("ls_", "chpl__init_")) and not n.endswith("_type")})
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("LS_REFERENCE_DIR", "/root/reference"))
    args = ap.parse_args()
    ref = args.reference
    if not ref or not os.path.isdir(ref):
        sys.exit("reference tree not found: pass --reference or set LS_REFERENCE_DIR")
    data = {
        "benes_kats": benes_kats(ref),
        "n10_chain": n10_chain(ref),
        "hubbard_2site": hubbard_matrices(ref),
        "hphi": hphi(ref),
        "chapel_configs": chapel_configs(ref),
        "struct_layouts": struct_layouts(ref),
        "declared_functions": declared_functions(ref),
    }
    with open(os.path.join(HERE, "reference_goldens.json"), "w", encoding="utf-8") as f:
        json.dump(data, f, ensure_ascii=False, indent=1)
    reference_kernel_outputs(ref, os.path.join(HERE, "reference_kernels.npz"))
    print("wrote", os.path.join(HERE, "reference_goldens.json"), os.path.join(HERE, "reference_kernels.npz"))


if __name__ == "__main__":
    main()
