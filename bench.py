"""H*x throughput of the exact-diagonalization hot path on one GB300 (and N replicas).

Workload (default, `--config j1j2_6x6`): J1-J2 Heisenberg model on the 6x6 square torus,
J1 = 1, J2 = 0.5 (sigma.sigma form of chapel/data/heisenberg_square_6x6.yaml plus the diagonal
bonds), Sz = 0, group = translations (36) x C4v (8) x spin inversion, momentum (pi, pi) sector,
about 1.6e7 representatives, x complex128 with re/im ~ N(0, 1) from numpy seed 2.

A step is one plain single-vector H*x (complex128) over the whole sector.

    metric  = matrix elements / s = (D + NNZ) / t     (NNZ: off-diagonal elements of H)
    value   = device-resident x, CUDA events around K steps on the launching stream
    e2e     = the same metric through the reference-facing C-ABI call ls_chpl_matrix_vector_product
              with host buffers (one call with num_vectors = 2: Re x and Im x, which the real
              Hamiltonian of this sector maps separately), copies inside the timed region
    extra   = block H*X with 16 right-hand sides and the adjoint H^dagger x, per vector

`--impl reference` times the CPU restatement of the reference's algorithm (Benes orbit scan,
scatter with atomics, prefix-table index; oracle/ls_oracle.c) with all host threads, on seeded
random column samples of a basis that the restatement enumerates itself (the setup, also
reported); it loads nothing of the product (oracle/workloads.py restates the workload).
"""

from __future__ import annotations

import argparse
import importlib
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

# DRAM bytes (read + write) of one matvec launch from an ncu capture of the same workload, with the
# integer (ALU) pipe utilisation of that capture; summaries and commands in profiles/.
NCU_CAPTURES = {
    "j1j2_6x6": {"traffic": 34.214e9 + 0.265e9, "alu_pipe_pct": 68.7,
                 "source": "profiles/k_matvec_packed_j1j2_6x6.md"},
    "xxz24_sectors": {"traffic": 2.749e9 + 0.681e9, "alu_pipe_pct": 26.0, "fp64_pipe_pct": 80.4,
                      "source": "profiles/k_matvec_sectors_xxz24.md"},
}

CONFIGS = {
    "j1j2_6x6": dict(L=6, kx=3, ky=3, J2=0.5, inversion=1, seed=2,
                     description="J1-J2 Heisenberg 6x6 torus, J2=0.5, Sz=0, T(36)xC4v(8)xZ2, (pi,pi) sector"),
    "chain24": dict(chain=24, seed=1,
                    description="Heisenberg chain N=24 PBC, Sz=0, T x P x Z2, k=0 p=+1 z=+1"),
    "hubbard16": dict(L=4, up=7, down=7, t=1.0, U=8.0, rhs=8, lanczos_steps=60, seed=5,
                      description="Hubbard 4x4 torus, t=1, U=8, 7 up + 7 down, translations x C4v with "
                                  "fermionic signs, Gamma sector; 8 complex RHS, block Lanczos ground state and "
                                  "dE0/d(t, U) by Hellmann-Feynman vs finite differences"),
    "ladder28_grad": dict(rungs=14, theta=(1.0, 0.7, 0.2), seed=4,
                          description="2-leg spin-1/2 ladder, 14 rungs PBC along legs, couplings J_leg, J_rung, "
                                      "D (z.(S_i x S_j) along legs), theta=(1.0, 0.7, 0.2), leg translations x leg "
                                      "exchange, Sz=0, k=0; loss Re<v, H(theta) x>, backward = adjoint matvec + "
                                      "per-coupling products, checked against central differences (h=1e-6)"),
    "xxz24_sectors": dict(n=24, delta=1.5, rhs=16, lanczos_steps=100, seed=3,
                          description="XXZ chain N=24 PBC, Delta=1.5, Sz=0, 24 momenta x z=+-1 (48 sectors), "
                                      "16 RHS: the batched workload at a size for kernel profiles"),
    "xxz28_sectors": dict(n=28, delta=1.5, rhs=16, lanczos_steps=100, lanczos_compare_steps=30, seed=3,
                          description="XXZ chain N=28 PBC, Jxy=1, Delta=1.5, Sz=0, all 28 momenta x z=+-1 "
                                      "(56 sectors), 16 complex RHS per sector, one batched launch in a CUDA "
                                      "graph, 100 block-Lanczos steps"),
}


# ------------------------------------------------------------------------------------------------
def build_workload(ls, lat, name):
    c = CONFIGS[name]
    if "chain" in c:
        n = c["chain"]
        syms = ls.Symmetries(lat.chain_symmetries(n, 0, 0))
        basis = ls.SpinBasis(n, n // 2, 1, syms)
        expr = lat.heisenberg(lat.chain_bonds(n))
    else:
        L = c["L"]
        syms = ls.Symmetries(lat.square_symmetries(L, c["kx"], c["ky"]))
        basis = ls.SpinBasis(L * L, L * L // 2, c["inversion"], syms)
        expr = lat.heisenberg(lat.square_bonds(L)) + lat.heisenberg(lat.square_bonds(L, diagonal=True), c["J2"])
    return basis, expr


def load_peaks():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index=0):
        self.device_index = device_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device_index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        return False

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def _oracle():
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O

    O.build()
    return O


def random_columns(rng, D, n):
    """A seeded random sample of about n distinct column indices of [0, D), sorted."""
    n = int(min(n, D))
    if n >= D // 2:
        return np.sort(rng.choice(D, size=n, replace=False)).astype(np.int64)
    return np.unique(rng.integers(0, D, size=n)).astype(np.int64)


class ColumnSampler:
    """The CPU restatement of the reference's matvec (oracle/ls_oracle.c lso_matvec_sample: Benes
    orbit scan in the reference's chunk order, prefix-table index of kernels/indexing.c, scatter
    with relaxed atomic adds as DistributedMatrixVector.chpl:91-143) over seeded random samples of
    columns, on `threads` host threads.  A step processes one sample: the orbit norms of its
    column states (state_info, as BatchedOperator.chpl:232-238 does per batch) and the scatter."""

    def __init__(self, O, group, inv, nbits, reps, off, diag, x, threads, seed):
        self.O = O
        O.set_threads(threads)
        self.group, self.inv, self.nbits = group, inv, nbits
        self.reps = np.ascontiguousarray(reps, dtype=np.uint64)
        self.D = len(self.reps)
        self.off, self.diag = off, diag
        self.x = np.ascontiguousarray(x, dtype=np.complex128)
        self.index = O.Index(self.reps, nbits, 22)
        self.y = np.zeros(self.D, dtype=np.complex128)
        self.rng = np.random.default_rng(seed)
        self.threads = threads

    def run(self, cols):
        t0 = time.perf_counter()
        norms = self.O.state_info(self.group, self.reps[cols], lane_width=8, use_benes=True)[2]
        nnz = self.O.matvec_sample(self.group, 2, self.inv, self.nbits, self.reps, cols, norms, self.off, self.diag,
                                   self.x[cols], self.y, self.index)
        return time.perf_counter() - t0, nnz

    def calibrate(self, seconds):
        """Columns per sample so that one sample takes about `seconds`."""
        n = 256
        while True:
            t, _ = self.run(random_columns(self.rng, self.D, n))
            if t >= 0.25 or n >= self.D:
                break
            n = min(self.D, n * 4)
        return int(min(self.D, max(n, seconds / max(t / n, 1e-12))))

    def timed(self, n_cols, warmup, steps):
        """Elements per second over `steps` fresh samples (after `warmup` untimed ones):
        (sampled columns + their off-diagonal elements) / time."""
        for _ in range(warmup):
            self.run(random_columns(self.rng, self.D, n_cols))
        tot_t, tot_e, cols_done = 0.0, 0, 0
        for _ in range(steps):
            cols = random_columns(self.rng, self.D, n_cols)
            t, nnz = self.run(cols)
            tot_t += t
            tot_e += len(cols) + nnz
            cols_done += len(cols)
        return tot_e / tot_t, tot_t / steps, cols_done // max(1, steps)

    def column_products(self, cols, coef):
        """y = H[:, cols] coef (the oracle's scatter of those columns alone)."""
        self.y[:] = 0
        norms = self.O.state_info(self.group, self.reps[cols], lane_width=8, use_benes=True)[2]
        self.O.matvec_sample(self.group, 2, self.inv, self.nbits, self.reps, cols, norms, self.off, self.diag, coef,
                             self.y, self.index)
        return self.y.copy()


def oracle_inputs(O, basis, op):
    """The oracle's group and term tables for a product basis and operator (our arm's CPU leg)."""
    gens = [(sym.permutation, sym.sector) for sym in basis.symmetries.generators]
    el = O.close_group(gens)
    re, im = O.characters(el)
    masks, shifts = basis.symmetries.network()
    g = O.Group(np.array([e[0] for e in el]), re, im, basis._c.spin_inversion, basis.number_bits, masks, shifts)
    return g, O.Terms(*op._off_arrays), O.Terms(*op._diag_arrays)


def bench_config(name, D):
    """The `config` object of both arms (identical for the same workload)."""
    return {"workload": name, "description": CONFIGS[name]["description"], "number_states": D, "rhs": 1,
            "parallelism": "replicas",
            "l2": "inputs larger than L2 (x 16 B/state, representatives + norms + index)"}


def enumeration_pin(name):
    path = os.path.join(REPO, "tests", "golden", "enumeration_pins.json")
    key = {"j1j2_6x6": "square6_pipi_z1"}.get(name)
    if key is None or not os.path.exists(path):
        return None
    with open(path) as f:
        return json.load(f).get(key)


def check_parity(sampler, op, D, x_host, name, states):
    """The GPU's H x_s against the oracle's scatter of the same sampled columns (x_s = x on 64
    seeded random columns, zero elsewhere), outside every timed region; plus the enumeration
    against the oracle's full-sector pin where one exists."""
    import hashlib

    import torch
    cols = random_columns(np.random.default_rng(11), D, 64)
    y_ref = sampler.column_products(cols, x_host[cols])
    xs = torch.zeros(D, dtype=torch.complex128, device="cuda")
    xs[torch.from_numpy(cols).cuda()] = torch.from_numpy(np.ascontiguousarray(x_host[cols])).cuda()
    y = op.apply_device(xs).cpu().numpy()
    tol = 1e-12 * np.abs(y_ref).max()
    rows_equal = bool(np.array_equal(np.nonzero(np.abs(y) > tol)[0], np.nonzero(np.abs(y_ref) > tol)[0]))
    out = {"columns": int(len(cols)), "rel_l2": float(np.linalg.norm(y - y_ref) / np.linalg.norm(y_ref)),
           "nonzero_rows_equal": rows_equal, "tolerance": 1e-12,
           "oracle": "oracle/ls_oracle.c lso_matvec_sample (scatter of the same columns)"}
    pin = enumeration_pin(name)
    if pin is not None:
        out["enumeration_matches_oracle_pin"] = bool(
            len(states) == pin["count"] and
            hashlib.sha256(np.ascontiguousarray(states).astype("<u8").tobytes()).hexdigest() == pin["sha256"])
    return out


# ------------------------------------------------------------------------------------------------
def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def _cuda_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def run_reference(args):
    """--impl reference: the CPU restatement of the reference's algorithm on the host cores, built
    from the oracle alone (oracle/workloads.py); nothing of the product is loaded."""
    import hashlib

    world, rank, local = dist_setup()
    if rank != 0:
        return 0
    if args.config not in ("j1j2_6x6", "chain24"):
        print(json.dumps({"impl": "reference", "unavailable": "the CPU reference arm covers the single-sector "
                          "workloads j1j2_6x6 and chain24; run it with one of them"}))
        return 0
    O = _oracle()
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import workloads as WL

    threads = os.cpu_count() or 1
    O.set_threads(threads)
    w = WL.workload(args.config)
    lo, hi = w.estimates()
    # Setup (untimed for the matvec metric, reported on its own): the reference's enumeration,
    # StatesEnumeration.chpl:242-268, over every candidate of the sector on all host threads.
    t0 = time.perf_counter()
    reps = O.enumerate_projected_par(w.group, lo, hi, lane_width=8, use_benes=True)
    t_enum = time.perf_counter() - t0
    candidates = O.rank(hi) - O.rank(lo) + 1
    D = len(reps)
    rng = np.random.default_rng(CONFIGS[args.config]["seed"])
    x = rng.normal(size=D) + 1j * rng.normal(size=D)
    sampler = ColumnSampler(O, w.group, w.inv, w.n, reps, w.off, w.diag, x, threads, seed=7)
    per_step = max(0.2, args.cpu_seconds / max(1, args.steps + args.warmup))
    n_cols = sampler.calibrate(per_step)
    value, t_step, cols = sampler.timed(n_cols, args.warmup, args.steps)
    line = {
        "impl": "reference", "metric": "H*x matrix elements/s", "value": value, "unit": "elements/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_step * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
        "data": "synthetic", "config": bench_config(args.config, D),
        "cpu_baseline": {"value": value, "unit": "elements/s", "cores": threads, "kind": "port",
                         "sample": "per step a fresh seeded random sample of {} of {} columns (oracle/ls_oracle.c "
                                   "lso_matvec_sample: Benes orbit scan, prefix index, atomic scatter); basis from the "
                                   "oracle's own enumeration".format(cols, D)},
        "e2e": {"value": value, "unit": "elements/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "enumeration": {"candidates": candidates, "states": D, "seconds": t_enum,
                        "candidates_per_s": candidates / t_enum, "cores": threads,
                        "sha256": hashlib.sha256(reps.astype("<u8").tobytes()).hexdigest()},
    }
    print(json.dumps(line))
    return 0


def run_ladder(args):
    """Differentiation workload: forward y = H(theta) x and the hand-written backward (adjoint
    matvec for dL/dx, fused per-coupling products for dL/dtheta), with a central-difference check."""
    import torch

    ls = importlib.import_module("lattice-symmetries_gb300")
    lat = importlib.import_module("lattice-symmetries_gb300.lattices")
    ag = importlib.import_module("lattice-symmetries_gb300.autograd")
    c = CONFIGS[args.config]
    R = c["rungs"]
    torch.cuda.set_device(0)
    legs, rungs = lat.ladder(R)
    basis = ls.SpinBasis(2 * R, R, None, ls.Symmetries(lat.ladder_symmetries(R, 0, 0)))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    basis.build()
    t_build = time.perf_counter() - t0
    parts = [lat.heisenberg(legs, 0.25), lat.heisenberg(rungs, 0.25), lat.dm_z(legs, 1.0)]
    theta0 = list(c["theta"])
    pop = ag.ParametrizedOperator(basis, parts, theta=theta0)
    D = basis.number_states
    nnz = pop.operator.count_nonzeros()
    elements = D + nnz
    rng = np.random.default_rng(c["seed"])
    v = torch.from_numpy(rng.normal(size=D) + 1j * rng.normal(size=D)).cuda()
    x0 = torch.from_numpy(rng.normal(size=D) + 1j * rng.normal(size=D)).cuda()
    stream = torch.cuda.current_stream()

    def forward_backward():
        theta = torch.tensor(theta0, dtype=torch.float64, requires_grad=True)
        x = x0.clone().requires_grad_(True)
        loss = torch.real(torch.vdot(v, pop.apply(theta, x)))
        loss.backward()
        return loss, theta.grad, x.grad

    for _ in range(args.warmup):
        forward_backward()
    torch.cuda.synchronize()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clocks:
        start.record(stream)
        for _ in range(args.steps):
            loss, gtheta, gx = forward_backward()
        end.record(stream)
        torch.cuda.synchronize()
    t_ms = start.elapsed_time(end) / args.steps
    # a forward + backward step touches every matrix element three times: H x, H^dagger v and the
    # per-coupling products <v, H_c x>
    value = 3 * elements / (t_ms * 1e-3)
    # parts of the step
    start.record(stream)
    y = pop.operator.apply_device(x0, check=False)
    end.record(stream)
    torch.cuda.synchronize()
    t_fwd = start.elapsed_time(end)
    start.record(stream)
    pop.operator.apply_device(v, adjoint=True, check=False)
    end.record(stream)
    torch.cuda.synchronize()
    t_adj = start.elapsed_time(end)
    start.record(stream)
    cp = pop.coupling_products(v, x0)
    end.record(stream)
    torch.cuda.synchronize()
    t_cp = start.elapsed_time(end)
    # central differences of L(theta) = Re <v, H(theta) x>, h = 1e-6
    h = 1e-6
    fd = []
    for i in range(3):
        tp, tm = list(theta0), list(theta0)
        tp[i] += h
        tm[i] -= h
        lp = float(torch.real(torch.vdot(v, pop.apply(torch.tensor(tp, dtype=torch.float64), x0))))
        lm = float(torch.real(torch.vdot(v, pop.apply(torch.tensor(tm, dtype=torch.float64), x0))))
        fd.append((lp - lm) / (2 * h))
    g = gtheta.numpy().tolist()
    line = {
        "metric": "H*x matrix elements/s", "value": value, "unit": "elements/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
        "config": {"workload": args.config, "description": c["description"], "number_states": D, "nnz": nnz,
                   "rhs": 1, "parallelism": "replicas", "l2": "inputs larger than L2 (x, v 16 B/state)"},
        "cpu_baseline": None, "gpu_launches": 6 * args.steps, "clocks": clocks.summary(), "basis_build_s": t_build,
        "extra": {"forward_ms": t_fwd, "adjoint_ms": t_adj, "coupling_products_ms": t_cp,
                  "grad_theta": g, "grad_theta_central_fd": fd,
                  "max_rel_diff_grad_vs_fd": max(abs(a - b) / max(1.0, abs(b)) for a, b in zip(g, fd)),
                  "loss": loss.item()},
    }
    print(json.dumps(line))
    return 0


def run_hubbard(args):
    """Symmetric Hubbard sector: 8-RHS matvec throughput, block-Lanczos ground state, and the
    Hellmann-Feynman gradient of E0 with respect to (t, U) against central differences."""
    import torch

    ls = importlib.import_module("lattice-symmetries_gb300")
    lat = importlib.import_module("lattice-symmetries_gb300.lattices")
    ag = importlib.import_module("lattice-symmetries_gb300.autograd")
    lanczos = importlib.import_module("lattice-symmetries_gb300.lanczos")
    c = CONFIGS[args.config]
    L, k = c["L"], c["rhs"]
    n = L * L
    torch.cuda.set_device(0)
    syms = ls.Symmetries(lat.square_symmetries(L, 0, 0, True))
    basis = ls.SpinfulFermionBasis(n, (c["up"], c["down"]), symmetries=syms)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    basis.build()
    t_build = time.perf_counter() - t0
    theta0 = [c["t"], c["U"]]
    pop = ag.ParametrizedOperator(basis, list(lat.hubbard_parts(lat.square_bonds(L), n)), theta=theta0)
    op = pop.operator
    D = basis.number_states
    nnz = op.count_nonzeros()
    elements = D + nnz
    rng = np.random.default_rng(c["seed"])
    X = torch.from_numpy(rng.normal(size=(D, k)) + 1j * rng.normal(size=(D, k))).cuda()
    Y = torch.empty_like(X)
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    for _ in range(args.warmup):
        op.apply_device(X, out=Y, stream=sptr, check=False)
    op.check_errors(sptr)
    torch.cuda.synchronize()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clocks:
        start.record(stream)
        for _ in range(args.steps):
            op.apply_device(X, out=Y, stream=sptr, check=False)
        end.record(stream)
        torch.cuda.synchronize()
    op.check_errors(sptr)
    t_ms = start.elapsed_time(end) / args.steps
    value = elements * k / (t_ms * 1e-3)
    if args.no_extras:
        print(json.dumps({"metric": "H*x matrix elements/s", "value": value, "unit": "elements/s", "n_gpus": 1,
                          "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_ms,
                          "config": {"workload": args.config, "number_states": D, "nnz": nnz, "rhs": k},
                          "gpu_launches": 2 * args.steps}))
        return 0
    # one vector per launch, for the per-vector comparison
    x1 = X[:, 0].contiguous()
    y1 = torch.empty_like(x1)
    start.record(stream)
    for _ in range(args.steps):
        op.apply_device(x1, out=y1, stream=sptr, check=False)
    end.record(stream)
    torch.cuda.synchronize()
    t_plain = start.elapsed_time(end) / args.steps

    hx = torch.empty(X.shape, dtype=X.dtype, pin_memory=True)
    hy = torch.empty_like(hx, pin_memory=True)
    hx.copy_(X)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ne = max(1, min(args.steps, 3))
    for _ in range(ne):
        X.copy_(hx, non_blocking=True)
        op.apply_device(X, out=Y, stream=sptr, check=False)
        hy.copy_(Y, non_blocking=True)
    torch.cuda.synchronize()
    te = (time.perf_counter() - t0) / ne
    e2e = {"value": elements * k / te, "unit": "elements/s", "h2d_bytes_per_step": hx.numel() * 16,
           "d2h_bytes_per_step": hy.numel() * 16, "path": "Operator.apply_device with pinned host X/Y copies"}

    theta = torch.tensor(theta0, dtype=torch.float64, requires_grad=True)
    # a short untimed run first: the first factorisations and eigensolves of the process load
    # the dense linear-algebra libraries (seconds)
    lanczos.ground_state_energy(pop, list(theta0), k=k, steps=3, seed=c["seed"], graph=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e0 = lanczos.ground_state_energy(pop, theta, k=k, steps=c["lanczos_steps"], seed=c["seed"], graph=True)
    torch.cuda.synchronize()
    t_lanczos = time.perf_counter() - t0
    e0.backward()
    hf = theta.grad.numpy().tolist()
    h = 1e-4
    fd = []
    for i in range(2):
        tp, tm = list(theta0), list(theta0)
        tp[i] += h
        tm[i] -= h
        ep = float(lanczos.ground_state_energy(pop, tp, k=k, steps=c["lanczos_steps"], seed=c["seed"]))
        em = float(lanczos.ground_state_energy(pop, tm, k=k, steps=c["lanczos_steps"], seed=c["seed"]))
        fd.append((ep - em) / (2 * h))
    # the same Lanczos run with torch FP64 GEMMs for the dense products
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e0_fp64 = float(lanczos.ground_state_energy(pop, list(theta0), k=k, steps=c["lanczos_steps"], seed=c["seed"],
                                                dense="fp64"))
    torch.cuda.synchronize()
    t_fp64 = time.perf_counter() - t0

    bytes_per_launch = D * (16 + 32 * k) + nnz * (16 + 16 * k)
    achieved = bytes_per_launch / (t_ms * 1e-3) / 1e9
    peak, peak_kind = load_peaks()
    # the reference has no fermionic bases with lattice symmetries, so it has no CPU path to time
    cpu = None
    line = {
        "metric": "H*x matrix elements/s", "value": value, "unit": "elements/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
        "config": {"workload": args.config, "description": c["description"], "number_states": D, "nnz": nnz,
                   "rhs": k, "parallelism": "replicas", "l2": "inputs larger than L2 (X, Y 8 columns)"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": None, "peak_source": peak_kind, "bytes_per_launch": bytes_per_launch},
        "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": 2 * args.steps, "clocks": clocks.summary(),
        "basis_build_s": t_build,
        "extra": {"plain_one_vector_ms": t_plain, "speedup_per_vector_vs_plain": t_plain * k / t_ms,
                  "ground_state": {"E0": e0.item(), "lanczos_steps": c["lanczos_steps"], "seconds": t_lanczos,
                                   "dE0_dtheta_hellmann_feynman": hf, "dE0_dtheta_central_fd": fd,
                                   "fd_step": h, "theta": theta0,
                                   "dense": "tensor-core Gram / update kernels (ls_gpu_block_gram_tc, "
                                            "ls_gpu_block_update_tc)",
                                   "E0_fp64_dense": e0_fp64, "seconds_fp64_dense": t_fp64}},
    }
    print(json.dumps(line))
    return 0


def run_sectors(args):
    """The batched workload: 56 sectors x 16 RHS through one persistent launch per step (CUDA
    graph replay), compared with per-sector launches, then 100 block-Lanczos steps."""
    import torch

    ls = importlib.import_module("lattice-symmetries_gb300")
    lat = importlib.import_module("lattice-symmetries_gb300.lattices")
    lanczos = importlib.import_module("lattice-symmetries_gb300.lanczos")
    rep = importlib.import_module("lattice-symmetries_gb300.replicas")
    c = CONFIGS[args.config]
    n, k = c["n"], c["rhs"]
    expr = lat.xxz(lat.chain_bonds(n), 1.0, c["delta"])
    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    # the sectors (momentum, z): under torchrun each rank takes its share (largest first to the
    # least loaded rank; the 2n sectors hold about C(n, n/2) / 2n states each, so unit weights)
    sectors = [(mom, z) for mom in range(n) for z in (1, -1)]
    mine = rep.my_units([1.0] * len(sectors))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ops = []
    for si in mine:
        mom, z = sectors[si]
        basis = ls.SpinBasis(n, n // 2, z, ls.Symmetries(lat.chain_symmetries(n, mom)))
        basis.build(exact_norms=True)
        ops.append(ls.Operator(basis, expr))
    t_build = time.perf_counter() - t0
    sizes = [op.basis.number_states for op in ops]
    nnzs = [op.count_nonzeros() for op in ops]
    elements = sum(sizes) + sum(nnzs)  # per right-hand side, this rank's sectors
    batch = ls.SectorBatch(ops, k=k)
    for s, d in enumerate(sizes):
        rng = np.random.default_rng([c["seed"], mine[s]])  # per-sector stream: same X for any split
        xs = rng.normal(size=(d, k)) + 1j * rng.normal(size=(d, k))
        batch.X[s, :d].copy_(torch.from_numpy(xs))
    # the plan's autotuner: one persistent launch over all sectors, or one launch per sector
    tune = batch.autotune()
    batch.capture()
    # kernels per run: batched, the prescaled pair copy of X (pair arithmetic; the n translations
    # are at most 64 group elements) + the matvec; per sector, a prescaled copy + the matvec each
    pairs_in_use = args.block_arithmetic == "pairs" or (args.block_arithmetic == "auto" and n <= 64)
    launches_per_run = (1 + int(pairs_in_use)) if tune["batched"] else 2 * len(ops)
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        batch.replay()
    torch.cuda.synchronize()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    rep.barrier()
    with ClockSampler(local) as clocks:
        start.record(stream)
        for _ in range(args.steps):
            batch.replay()
        end.record(stream)
        torch.cuda.synchronize()
    rep.barrier()
    batch.check_errors()
    t_ms = rep.max_over_ranks(start.elapsed_time(end) / args.steps)  # the slowest rank
    elements_all = rep.sum_over_ranks(elements)
    value = elements_all * k / (t_ms * 1e-3)

    if world > 1:
        # every rank's sector ground states (block Lanczos on its own batch), merged
        e0 = lanczos.sector_ground_states(batch, steps=c["lanczos_steps"], seed=c["seed"], graph=True)
        merged = rep.gather_results({si: float(e) for si, e in zip(mine, e0)})
        states_all = int(rep.sum_over_ranks(sum(sizes)))
        if rank == 0:
            g = min(merged, key=merged.get)
            print(json.dumps({
                "metric": "H*x matrix elements/s", "value": value, "unit": "elements/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_ms, "higher_is_better": True,
                "scaling": "strong", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
                "config": {"workload": args.config, "description": c["description"], "sectors": len(sectors),
                           "states": states_all, "rhs": k, "parallelism": "sectors split over {} ranks".format(world),
                           "block_arithmetic": args.block_arithmetic},
                "gpu_launches": None, "clocks": clocks.summary(),
                "extra": {"ground_state_energy": merged[g], "sector_of_ground_state": list(sectors[g]),
                          "sectors_per_rank": len(mine)}}))
        torch.distributed.destroy_process_group()
        return 0

    if args.no_extras:
        print(json.dumps({"metric": "H*x matrix elements/s", "value": value, "unit": "elements/s", "n_gpus": 1,
                          "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_ms,
                          "config": {"workload": args.config, "sectors": len(ops), "states": sum(sizes),
                                     "nnz": sum(nnzs), "rhs": k, "form": "batched" if tune["batched"] else
                                     "per-sector launches"}, "gpu_launches": launches_per_run * args.steps}))
        return 0
    # the same launch in the other block arithmetic (FP32 pairs when the headline is FP64, else
    # FP64), and the difference it makes; the headline number is the --block-arithmetic one
    other = "auto" if args.block_arithmetic == "fp64" else "fp64"
    batch.run(check=True)
    y_head = batch.Y.clone()
    ls.Operator.block_arithmetic(other)
    batch.run()
    torch.cuda.synchronize()
    start.record(stream)
    for _ in range(2):
        batch.run()
    end.record(stream)
    torch.cuda.synchronize()
    t_other_block = start.elapsed_time(end) / 2
    other_rel_l2 = float(torch.linalg.vector_norm(batch.Y - y_head) / torch.linalg.vector_norm(y_head))
    ls.Operator.block_arithmetic(args.block_arithmetic)
    batch.run(check=True)
    del y_head
    # the same work as one launch per sector (no batching across sectors, no graph)
    start.record(stream)
    for s, op in enumerate(ops):
        op.apply_device(batch.x(s), out=batch.y(s), check=False)
    end.record(stream)
    torch.cuda.synchronize()
    t_loop = start.elapsed_time(end)
    # plain: one vector per launch, one sector after the other (per-vector cost)
    x1 = [batch.x(s)[:, 0].contiguous() for s in range(len(ops))]
    y1 = [torch.empty_like(v) for v in x1]
    start.record(stream)
    for s, op in enumerate(ops):
        op.apply_device(x1[s], out=y1[s], check=False)
    end.record(stream)
    torch.cuda.synchronize()
    t_plain = start.elapsed_time(end)

    # end to end: pinned host X in, host Y out, around every batched step
    hx = torch.empty(batch.X.shape, dtype=batch.X.dtype, pin_memory=True)
    hy = torch.empty_like(hx, pin_memory=True)
    hx.copy_(batch.X)
    ne = max(1, min(args.steps, 3))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(ne):
        batch.X.copy_(hx, non_blocking=True)
        batch.replay()
        hy.copy_(batch.Y, non_blocking=True)
    torch.cuda.synchronize()
    te = (time.perf_counter() - t0) / ne
    e2e = {"value": elements * k / te, "unit": "elements/s", "h2d_bytes_per_step": hx.numel() * 16,
           "d2h_bytes_per_step": hy.numel() * 16, "path": "SectorBatch.replay with pinned host X/Y copies"}

    # dense products on the tensor cores (the default): the full recurrence and the lean one (one
    # Cholesky-QR pass, no local re-orthogonalisation)
    timer = {}
    e0 = lanczos.sector_ground_states(batch, steps=c["lanczos_steps"], seed=c["seed"], graph=True, timer=timer,
                                      dense="tensor")
    timer_lean = {}
    e0_lean = lanczos.sector_ground_states(batch, steps=c["lanczos_steps"], seed=c["seed"], graph=True,
                                           timer=timer_lean, lean=True, dense="tensor")
    # the same recurrence with the FP32-pair kernels and with torch FP64 GEMMs for the dense products
    # (fewer steps on the large workload: FP64 GEMMs are slow on GB300)
    cmp_steps = c.get("lanczos_compare_steps", c["lanczos_steps"])
    timer_tc = timer
    e0_tc = e0
    if cmp_steps != c["lanczos_steps"]:
        timer_tc = {}
        e0_tc = lanczos.sector_ground_states(batch, steps=cmp_steps, seed=c["seed"], graph=True, timer=timer_tc,
                                             dense="tensor")
    timer_pc = {}
    e0_pc = lanczos.sector_ground_states(batch, steps=cmp_steps, seed=c["seed"], graph=True, timer=timer_pc,
                                         dense="paired")
    timer_f = {}
    e0_f = lanczos.sector_ground_states(batch, steps=cmp_steps, seed=c["seed"], graph=True, timer=timer_f,
                                        dense="fp64")

    bytes_per_launch = sum(sizes) * (16 + 32 * k) + sum(nnzs) * (16 + 16 * k)
    achieved = bytes_per_launch / (t_ms * 1e-3) / 1e9
    peak, peak_kind = load_peaks()
    cpu = None
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        O = _oracle()
        b0 = ops[0].basis
        g0, off0, diag0 = oracle_inputs(O, b0, ops[0])
        sampler = ColumnSampler(O, g0, b0._c.spin_inversion, b0.number_bits, b0.states, off0, diag0,
                                batch.x(0)[:, 0].cpu().numpy(), threads, seed=7)
        n_cols = sampler.calibrate(args.cpu_seconds / 4)
        rate, t_s, cols = sampler.timed(n_cols, 1, 3)
        cpu = {"value": rate, "unit": "elements/s", "cores": threads, "kind": "port",
               "sample": "sector k=0 z=+1, one vector, 3 seeded random samples of {} of {} columns "
                         "(oracle/ls_oracle.c lso_matvec_sample), {:.2f} s each".format(cols, sizes[0], t_s)}
    line = {
        "metric": "H*x matrix elements/s", "value": value, "unit": "elements/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
        "config": {"workload": args.config, "description": c["description"], "sectors": len(ops),
                   "states": sum(sizes), "nnz": sum(nnzs), "rhs": k, "parallelism": "replicas",
                   "l2": "inputs larger than L2 (X, Y {:.2f} GB each)".format(batch.X.numel() * 16 / 1e9)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": NCU_CAPTURES.get(args.config, {}).get("traffic"),
                     "alu_pipe_pct": NCU_CAPTURES.get(args.config, {}).get("alu_pipe_pct"),
                     "fp64_pipe_pct": NCU_CAPTURES.get(args.config, {}).get("fp64_pipe_pct"),
                     "peak_source": peak_kind, "bytes_per_launch": bytes_per_launch,
                     "note": "FP64-pipe-bound gather kernel with 16 columns (FP32-pair multiply-adds are "
                             "opt-in); frac is of algorithmic bytes with every gather counted from DRAM; "
                             "traffic and pipe figures are from the ncu capture named in traffic_source "
                             "(batched FP64 launch, N = 24), not measured by this run",
                     "traffic_source": NCU_CAPTURES.get(args.config, {}).get("source")},
        "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches_per_run * args.steps, "clocks": clocks.summary(),
        "basis_build_s": t_build,
        "extra": {"form": "one persistent launch over all sectors" if tune["batched"] else
                  "one launch per sector (in the CUDA graph)",
                  "autotune_ms": {"batched": tune["ms_batched"], "per_sector": tune["ms_per_sector"]},
                  "block_arithmetic": args.block_arithmetic,
                  "other_block_arithmetic": {
                      "arithmetic": other, "ms_per_step": t_other_block, "rel_l2_vs_headline": other_rel_l2,
                      "note": "auto = FP32-pair multiply-adds for groups of at most 64 elements (each product "
                              "below 2^-45 relative, each output within ~2^-45 of the sum of its terms' "
                              "magnitudes); fp64 = FP64 multiply-adds"},
                  "per_sector_launches_ms": t_loop, "batched_speedup_vs_per_sector": t_loop / t_ms,
                  "plain_one_vector_all_sectors_ms": t_plain,
                  "speedup_per_vector_vs_plain": t_plain * k / t_ms,
                  "lanczos": {"steps": c["lanczos_steps"], "ms_per_step": timer["ms"] / timer["steps"],
                              "step_over_matvec": timer["ms"] / timer["steps"] / t_ms,
                              "ground_state_energy": float(np.min(e0)),
                              "sector_of_ground_state": int(np.argmin(e0)),
                              "dense": "tensor-core Gram / update kernels (ls_gpu_block_gram_tc, "
                                       "ls_gpu_block_update_tc: fixed-point bf16 digits, exact FP32 group "
                                       "sums, FP64 results)",
                              "lean_ms_per_step": timer_lean["ms"] / timer_lean["steps"],
                              "lean_step_over_matvec": timer_lean["ms"] / timer_lean["steps"] / t_ms,
                              "lean_max_abs_diff_sector_e0": float(np.max(np.abs(e0_lean - e0))),
                              "compare": {"steps": cmp_steps,
                                          "tensor_ms_per_step": timer_tc["ms"] / timer_tc["steps"],
                                          "paired_ms_per_step": timer_pc["ms"] / timer_pc["steps"],
                                          "fp64_ms_per_step": timer_f["ms"] / timer_f["steps"],
                                          "max_abs_diff_sector_e0_tensor_vs_fp64":
                                              float(np.max(np.abs(e0_tc - e0_f))),
                                          "max_abs_diff_sector_e0_paired_vs_fp64":
                                              float(np.max(np.abs(e0_pc - e0_f)))}}},
    }
    print(json.dumps(line))
    return 0


def block_and_adjoint(op, rng, D, elements, ms_per_step, steps, x, y, sptr):
    """Adjoint H^dagger x, then block H*X and H^dagger*X with 16 right-hand sides (after tuning
    the launch shape and right-hand-side tile for 16 columns), timed per vector."""
    import torch
    stream = torch.cuda.current_stream()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    nb = max(1, steps // 2)

    def timed(fn):
        for _ in range(2):
            fn()
        torch.cuda.synchronize()
        start.record(stream)
        for _ in range(nb):
            fn()
        end.record(stream)
        torch.cuda.synchronize()
        return start.elapsed_time(end) / nb

    extra = {}
    ta = timed(lambda: op.apply_device(x, out=y, adjoint=True, stream=sptr, check=False))
    extra["adjoint"] = {"ms_per_step": ta, "value": elements / (ta * 1e-3)}
    K16 = 16
    X16 = torch.from_numpy(rng.normal(size=(D, K16)) + 1j * rng.normal(size=(D, K16))).cuda()
    Y16 = torch.empty_like(X16)
    saved = op.launch_config()
    op.autotune(K16)
    t16 = timed(lambda: op.apply_device(X16, out=Y16, stream=sptr, check=False))
    extra["block16"] = {"ms_per_block": t16, "value_per_vector": elements * K16 / (t16 * 1e-3),
                        "speedup_per_vector_vs_plain": ms_per_step * K16 / t16,
                        "launch": dict(zip(("threads", "waves", "rhs_tile"), op.launch_config()))}
    t16a = timed(lambda: op.apply_device(X16, out=Y16, adjoint=True, stream=sptr, check=False))
    extra["adjoint_block16"] = {"ms_per_block": t16a, "value_per_vector": elements * K16 / (t16a * 1e-3),
                                "speedup_per_vector_vs_plain": ms_per_step * K16 / t16a}
    op.check_errors(sptr)
    lib = importlib.import_module("lattice-symmetries_gb300")._native.lib()
    lib.ls_gpu_set_matvec_config(saved[0], saved[1])  # back to the one-vector launch shape
    lib.ls_gpu_set_matvec_rhs_tile(saved[2])
    return extra


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="j1j2_6x6", choices=sorted(CONFIGS))
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the block-16 and adjoint lines")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shape")
    ap.add_argument("--block-arithmetic", default="fp64", choices=["fp64", "auto", "pairs"],
                    help="multiply-adds of complex blocks of 8/16 columns (fp64, the default; auto: FP32 "
                         "pairs for groups of at most 64 elements; pairs: FP32 pairs for every group)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    importlib.import_module("lattice-symmetries_gb300").Operator.block_arithmetic(args.block_arithmetic)
    if args.config in ("xxz24_sectors", "xxz28_sectors"):
        return run_sectors(args)  # under torchrun the sectors are split over the ranks
    if args.config in ("hubbard16", "ladder28_grad"):
        world, rank, _ = dist_setup()
        if rank != 0:
            return 0  # single-sector workloads: under torchrun only rank 0 runs them
        if args.config == "hubbard16":
            return run_hubbard(args)
        return run_ladder(args)

    import torch

    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    ls = importlib.import_module("lattice-symmetries_gb300")
    lat = importlib.import_module("lattice-symmetries_gb300.lattices")
    rep = importlib.import_module("lattice-symmetries_gb300.replicas")
    basis, expr = build_workload(ls, lat, args.config)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    basis.build()
    t_build = time.perf_counter() - t0
    op = ls.Operator(basis, expr)
    # per-stage times of a second, traced build of the same basis (outside every timed region)
    ls.stage_times(reset=True)
    ls.set_tracing(True)
    build_workload(ls, lat, args.config)[0].build()
    ls.set_tracing(False)
    stages_build = ls.stage_times(reset=True)
    D = basis.number_states
    nnz = op.count_nonzeros()
    elements = D + nnz
    tuned = (None, None, None) if args.no_autotune else op.autotune(1)
    rng = np.random.default_rng(CONFIGS[args.config]["seed"])
    x_host = rng.normal(size=D) + 1j * rng.normal(size=D)
    x = torch.from_numpy(x_host).cuda()
    y = torch.empty_like(x)
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream

    def step():
        op.apply_device(x, out=y, stream=sptr, check=False)

    for _ in range(args.warmup):
        step()
    op.check_errors(sptr)
    rep.barrier()
    torch.cuda.synchronize()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clocks:
        start.record(stream)
        for _ in range(args.steps):
            step()
        end.record(stream)
        torch.cuda.synchronize()
    op.check_errors(sptr)
    t_ms = start.elapsed_time(end)
    t_ms = rep.max_over_ranks(t_ms)  # replicas: the slowest rank's time
    # per-stage times of one traced step (outside the timed region)
    ls.set_tracing(True)
    step()
    ls.set_tracing(False)
    stages_step = ls.stage_times(reset=True)
    ms_per_step = t_ms / args.steps
    value = world * elements * args.steps / (t_ms * 1e-3)

    # roofline of the matvec kernel (one launch per step): algorithmic bytes
    bytes_per_launch = 8 * D + 8 * D + 16 * D + 16 * D + nnz * (16 + 8 + 8)
    achieved_gbs = bytes_per_launch / (ms_per_step * 1e-3) / 1e9
    peak, peak_kind = load_peaks()


    # end to end through the reference-facing C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        # the Hamiltonian is real in this sector, so H x = H Re(x) + i H Im(x): both parts go
        # through one reference-facing call with num_vectors = 2 (host buffers, copies inside)
        xs = np.ascontiguousarray(np.stack([x_host.real, x_host.imag]))
        op.apply_to_state_vectors(xs)
        torch.cuda.synchronize()
        ne = max(1, min(args.steps, 3))
        t_calls = []
        for _ in range(ne):
            t0 = time.perf_counter()
            ys = op.apply_to_state_vectors(xs)
            t_calls.append(time.perf_counter() - t0)
        te = sum(t_calls) / ne
        # the same through two one-vector calls, as the reference's interface allows
        t0 = time.perf_counter()
        yr = op.apply_to_state_vector(np.ascontiguousarray(x_host.real))
        yi = op.apply_to_state_vector(np.ascontiguousarray(x_host.imag))
        t_two = time.perf_counter() - t0
        # stages of one more (traced, untimed) call
        ls.set_tracing(True)
        t0 = time.perf_counter()
        op.apply_to_state_vectors(xs)
        t_traced = time.perf_counter() - t0
        ls.set_tracing(False)
        stages_e2e = ls.stage_times(reset=False)
        stages_e2e_host = ls.stage_times(reset=True, host=True)
        e2e = {"value": world * elements / te, "unit": "elements/s", "h2d_bytes_per_step": 2 * 8 * D,
               "d2h_bytes_per_step": 2 * 8 * D,
               "path": "ls_chpl_matrix_vector_product(num_vectors=2: Re x, Im x), host buffers",
               "two_single_vector_calls": {"value": world * elements / t_two},
               "stages_ms": {k: v[1] for k, v in stages_e2e.items()},
               "stages_host_ms": {k: v[1] for k, v in stages_e2e_host.items()},
               "traced_call_ms": t_traced * 1e3, "calls_ms": [t * 1e3 for t in t_calls]}

    # block matvec (16 right-hand sides) and adjoint, per vector
    extra = {} if args.no_extras else block_and_adjoint(op, rng, D, elements, ms_per_step, args.steps, x, y, sptr)

    cpu, parity, cpu_enum = None, None, None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        O = _oracle()
        g, off, diag = oracle_inputs(O, basis, op)
        states = basis.states
        sampler = ColumnSampler(O, g, basis._c.spin_inversion, basis.number_bits, states, off, diag, x_host,
                                threads, seed=7)
        per_step = max(0.2, args.cpu_seconds / 6)
        n_cols = sampler.calibrate(per_step)
        rate, t_s, cols = sampler.timed(n_cols, 1, 5)
        cpu = {"value": rate, "unit": "elements/s", "cores": threads, "kind": "port",
               "sample": "5 seeded random samples of {} of {} columns (oracle/ls_oracle.c lso_matvec_sample: "
                         "Benes orbit scan, prefix index, atomic scatter), {:.2f} s each".format(cols, D, t_s)}
        parity = check_parity(sampler, op, D, x_host, args.config, states)
        # the reference's enumeration (StatesEnumeration.chpl:242-268) restated on the host cores,
        # over the whole sector, against the GPU build
        lo, hi = basis._estimates()
        t0 = time.perf_counter()
        cpu_reps = O.enumerate_projected_par(g, lo, hi, lane_width=8, use_benes=True)
        t_cpu_enum = time.perf_counter() - t0
        n_cand = O.rank(hi) - O.rank(lo) + 1
        cpu_enum = {"candidates": n_cand, "seconds": t_cpu_enum, "candidates_per_s": n_cand / t_cpu_enum,
                    "cores": threads, "gpu_seconds": t_build, "gpu_speedup": t_cpu_enum / t_build,
                    "how": "oracle/ls_oracle.c lso_enumerate_projected_par (Benes orbit scan, chunk order "
                           "with early exit), all host threads"}
        parity["enumeration_equals_cpu"] = bool(np.array_equal(cpu_reps, states))
        del cpu_reps

    if rank == 0:
        line = {
            "metric": "H*x matrix elements/s", "value": value, "unit": "elements/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
            "config": bench_config(args.config, D),
            "roofline": {"bound": "hbm", "achieved": achieved_gbs, "peak": peak, "unit": "GB/s",
                         "frac": achieved_gbs / peak, "peak_source": peak_kind,
                         "traffic": NCU_CAPTURES.get(args.config, {}).get("traffic"),
                         "alu_pipe_pct": NCU_CAPTURES.get(args.config, {}).get("alu_pipe_pct"),
                         "traffic_source": NCU_CAPTURES.get(args.config, {}).get("source"),
                         "bytes_per_launch": bytes_per_launch,
                         "note": "integer-ALU bound orbit scan; frac is of algorithmic bytes; traffic (DRAM bytes "
                                 "per launch) and alu_pipe_pct are from the ncu capture named in traffic_source, "
                                 "not measured by this run"},
            "nnz": nnz,
            "cpu_baseline": cpu, "parity": parity, "e2e": e2e, "gpu_launches": 2 * args.steps,
            "clocks": clocks.summary(), "basis_build_s": t_build, "cpu_enumeration": cpu_enum, "extra": extra,
            "stages_ms": {"basis_build": {k: v[1] for k, v in stages_build.items()},
                          "matvec_step": {k: v[1] for k, v in stages_step.items()},
                          "how": "CUDA events per stage (ls_gpu_set_tracing), untimed passes"},
            "autotune": {"threads": tuned[0], "waves": tuned[1], "ms": tuned[2]},
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
