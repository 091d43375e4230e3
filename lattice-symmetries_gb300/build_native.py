"""Builds libls_gb300.so (sm_103a) from csrc/ with nvcc, one translation unit per process.

Usage: ``python lattice-symmetries_gb300/build_native.py`` or ``build_native.build()``.
The library is written to ``lattice-symmetries_gb300/_lib/libls_gb300.so``.
"""

from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(OUT_DIR, "libls_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-Xptxas", "-warn-spills"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(REPO, "include", "ls_gb300.h"))
    return hs


def _compile(src: str, verbose_ptxas: bool) -> str:
    obj = os.path.join(OBJ_DIR, os.path.basename(src) + ".o")
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + ["-I", os.path.join(REPO, "include"), "-I", CSRC,
                                         "-c", src, "-o", obj]
    if verbose_ptxas:
        cmd[cmd.index("-warn-spills")] = "-v"
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("nvcc failed for {}:\n{}\n{}".format(src, res.stdout, res.stderr))
    if verbose_ptxas:
        sys.stderr.write(res.stderr)
    elif res.stderr.strip():
        sys.stderr.write(res.stderr)
    return obj


def _stale(obj: str, deps) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose_ptxas: bool = False, jobs: int = 0) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    srcs = sources()
    hdrs = headers()
    todo = []
    objs = []
    for s in srcs:
        obj = os.path.join(OBJ_DIR, os.path.basename(s) + ".o")
        objs.append(obj)
        if force or verbose_ptxas or _stale(obj, [s] + hdrs):
            todo.append(s)
    if todo:
        jobs = jobs or min(len(todo), max(1, os.cpu_count() or 1))
        with concurrent.futures.ThreadPoolExecutor(max_workers=jobs) as ex:
            for f in [ex.submit(_compile, s, verbose_ptxas) for s in todo]:
                f.result()
    # relink when an object is newer than the library (also after a link that failed)
    if todo or not os.path.exists(LIB_PATH) or _stale(LIB_PATH, objs):
        tmp = LIB_PATH + ".tmp"
        cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "shared", "-o", tmp] + objs
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("link failed:\n{}\n{}".format(res.stdout, res.stderr))
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    force = "--force" in sys.argv
    print(build(force=force, verbose_ptxas="--ptxas" in sys.argv))
