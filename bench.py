#!/usr/bin/env python3
"""Benchmark of the Cyclix CheFSI step on one GB300: mixed precision vs plain FP64.

A step is one eigSolver call (src/eigSolver.m:26-125, past the first-SCF bound estimation):
Chebyshev filter of degree 24 over all states, H*psi for the projection, Rayleigh-Ritz
(Gram, Cholesky, projected Hamiltonian, general FP64 eigensolver, sort, rotation,
W-normalisation) on the cyclic 96 x 24 x 64 grid, FD order 12, one Bloch wavenumber,
Ns = 256 states, 77 atoms with 4 KB projectors each (seeded synthetic inputs).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  ``value`` is the device-timed mixed-precision step time
(inputs resident in HBM; psi = 302 MB complex64 > L2 so no flush is needed); ``e2e`` is the
same step through the host-buffer C-ABI entry (cx_eigsolver_host, complex128 psi copied in
and out every step from page-locked memory).  ``--impl reference`` times the CPU restatement
of the reference (the reference itself is MATLAB and cannot run here) on all host cores.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOAD = "cyclic-96x24x64-ns256-m24"
METRIC = "SCF-step time & H*psi HBM GB/s: mixed vs FP64 on GB300 at 1e-6 Ha/atom"


def env_int(k, d):
    try:
        return int(os.environ.get(k, d))
    except ValueError:
        return d


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits", "-lms", "200",
                                          "-i", str(self.index)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), float(d.get("bf16_tflops", 1933.1)), "measured"
    return 6800.0, 1900.0, "fallback"


# ----------------------------------------------------------------------------- CPU baseline (oracle)
def _cpu_hpsi_chunk(args):
    seed, n, kvec, spin, S = args
    from oracle import cychel_ops as O
    H = O.Hamiltonian(S, np.asarray(kvec), S.Veff[:, spin])
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((S.N, n)) + 1j * rng.standard_normal((S.N, n))
    H(X[:, :1])                       # warm the operator
    t = time.perf_counter()
    H(X)
    return time.perf_counter() - t


def cpu_baseline(S, ns_total, npl, sample_states=None, workers=None):
    """Oracle CheFSI step on a bounded sample, scaled to the full step (ms).

    H*psi: ``sample_states`` states on ``workers`` spawned processes (one chunk each), scaled
    by (npl + 1) applications and Ns/sample (linear in Ns).  Rayleigh-Ritz (orth by SVD,
    projection, general eig, rotation, W-normalisation): timed on ``sample_states`` columns and
    scaled by (Ns/sample)^2 for the N x Ns x Ns products and ^3 for the dense eig.
    """
    import multiprocessing as mp
    import scipy.linalg as sla
    workers = workers or os.cpu_count() or 1
    sample_states = sample_states or max(2 * workers, 32)
    per = max(1, sample_states // workers)
    sample_states = per * workers
    k = S.kptgrid[0]
    ctx = mp.get_context("spawn")
    # one BLAS thread per worker process: the workers already cover every core, and many
    # small products per H*psi make oversubscribed BLAS threads spin against one another
    saved = {v: os.environ.get(v) for v in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")}
    for v in saved:
        os.environ[v] = "1"
    try:
        with ctx.Pool(workers) as pool:
            ts = pool.map(_cpu_hpsi_chunk, [(i, per, tuple(k), 0, S) for i in range(workers)])
    finally:
        for v, old_v in saved.items():
            if old_v is None:
                os.environ.pop(v, None)
            else:
                os.environ[v] = old_v
    t_h = max(ts)                                    # wall time of one parallel H*psi over the sample
    t_filter = t_h * (npl + 1) * (ns_total / sample_states)
    ncols = min(64, ns_total)
    rng = np.random.default_rng(0)
    X = rng.standard_normal((S.N, ncols)) + 1j * rng.standard_normal((S.N, ncols))
    HX = rng.standard_normal((S.N, ncols)) + 1j * rng.standard_normal((S.N, ncols))
    t0 = time.perf_counter()
    Q = sla.orth(X)
    t1 = time.perf_counter()
    Hs = Q.conj().T @ HX
    t2 = time.perf_counter()
    A = rng.standard_normal((ns_total, ns_total)) + 1j * rng.standard_normal((ns_total, ns_total))
    t3 = time.perf_counter()
    D, V = sla.eig(A)
    t4 = time.perf_counter()
    P = Q @ V[:ncols, :ncols]
    sc = 1.0 / np.sqrt(np.sum(S.W[:, None] * (P * P.conj()).real, axis=0))
    P *= sc
    t5 = time.perf_counter()
    q2 = (ns_total / ncols) ** 2
    t_rr = (t1 - t0) * q2 + (t2 - t1) * q2 + (t4 - t3) + (t5 - t4) * q2
    total_ms = (t_filter + t_rr) * 1e3
    sample = (f"H*psi of {sample_states} of {ns_total} states on {workers} spawned processes, x{npl + 1} applications "
              f"x{ns_total / sample_states:g} (linear in Ns); orth/projection/rotation on {ncols} columns x{q2:g} "
              f"(quadratic in Ns); dense general eig at the full {ns_total} x {ns_total}")
    return total_ms, workers, sample


# ----------------------------------------------------------------------------- replicas
def max_over_ranks(value: float, dist=None) -> float:
    """Slowest rank's per-step time (the whole job finishes with it); identity on one process."""
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ----------------------------------------------------------------------------- GPU arms
def gpu_step_times(S, blocks, prec, steps, warmup, npl, profile_stencil=False, ramp=6):
    from cyclix_msparc_gb300.msparc import CyclixGPU
    from cyclix_msparc_gb300.workloads import initial_psi
    g = CyclixGPU(S, blocks, prec)
    for b, (_, _, n) in enumerate(g.blocks):
        g.set_psi(b, initial_psi(S.N, n, 10 + b))
    nblk = len(g.blocks)
    EV = np.zeros(int(sum(g.Ns)))
    a0, bup, lc = np.zeros(nblk), np.zeros(nblk), np.zeros(nblk)
    count = 1
    # ramp-up: the first SCF cycles (bound estimation, rhoTrigger cycles) bring psi near the
    # steady state of an SCF run; then the warm-up steps, then the timed steps
    for _ in range(ramp + max(warmup, 1)):
        g.eigsolve(count, npl, EV, a0, bup, lc)
        count += 1
    g.sync()
    g.launch_count(reset=True)
    fb0 = g.eig_fallbacks()
    g.timer_start()
    for _ in range(steps):
        g.eigsolve(count, npl, EV, a0, bup, lc)
        count += 1
    ms = g.timer_stop()
    launches = g.launch_count(reset=True)
    fallbacks = g.eig_fallbacks() - fb0
    prof = None
    if profile_stencil:
        g.profile(True)
        g.eigsolve(count, npl, EV, a0, bup, lc)
        count += 1
        n, kms, by = g.profile_read()
        prof = (n, kms, by, g.profile_read_apply())
        g.profile(False)
    return g, ms / steps, launches / steps, EV.copy(), prof, count, (a0, bup, lc), fallbacks


def e2e_host(g, count, npl, steps, bounds):
    """Same step through cx_eigsolver_host with page-locked complex128 psi (copies in the timed region)."""
    import ctypes as C
    N = g.N
    tot = int(sum(g.Ns))
    psi = np.empty(N * tot, dtype=np.complex128)
    off = 0
    for b in range(len(g.blocks)):
        psi[off * N:(off + g.Ns[b]) * N] = g.get_psi(b).reshape(-1, order="F")
        off += g.Ns[b]
    nbytes = psi.nbytes
    reg = g.lib.cx_host_register(psi.ctypes.data_as(C.c_void_p), nbytes) == 0
    EV = np.zeros(tot)
    a0, bup, lc = (np.ascontiguousarray(v.copy()) for v in bounds)
    g.sync()
    t = time.perf_counter()
    for _ in range(steps):
        g.eigsolve_host(count, npl, psi, EV, a0, bup, lc)
        count += 1
    dt = (time.perf_counter() - t) / steps
    if reg:
        g.lib.cx_host_unregister(psi.ctypes.data_as(C.c_void_p))
    return dt * 1e3, nbytes, nbytes


# ----------------------------------------------------------------------------- all configurations
CONFIGS = [
    ("cyclic-40x12x20-ns48-m20", True),
    ("cyclic-96x24x64-ns256-m24", True),
    ("cyclic-batched-16nu-64x16x48-ns96to320-m24", True),
    ("helical-80x32x40-96k2s-ns192-m24", True),
    ("scf-128x48x96-384at-8k-ns1024", False),   # FP64 Rayleigh-Ritz of 8 x ~1000 states: minutes per step
]


def config_lines(only=None, max_scf=40, skip_steps=False):
    """One eigSolver step per configuration (mixed and, where it fits the run, FP64), plus the full
    mixed-precision SCF of the 384-atom cell.  One JSON line per configuration on stdout."""
    from cyclix_msparc_gb300.msparc import CyclixGPU
    from cyclix_msparc_gb300.workloads import WORKLOADS, block_layout, initial_psi, make_system
    for name, with_fp64 in CONFIGS:
        if only and name != only:
            continue
        wl = WORKLOADS[name]
        t0 = time.perf_counter()
        S = make_system(wl)
        setup_s = time.perf_counter() - t0
        scf_cell = S.Veff is None
        if scf_cell:
            S.Veff = np.repeat((-S.rho_at)[:, None], S.nspin, axis=1)
        blocks = block_layout(wl, S)
        nblk = len(blocks)
        res = {"workload": name, "N": S.N, "blocks": nblk, "states": int(sum(n for (_, _, n) in blocks)), "npl": wl.npl,
               "setup_s": round(setup_s, 1)}
        evs = {}
        for prec in (() if skip_steps else (("mixed", "fp64") if with_fp64 else ("mixed",))):
            g = CyclixGPU(S, blocks, prec)
            try:
                for b, (_, _, n) in enumerate(blocks):
                    g.set_psi(b, initial_psi(S.N, n, 900 + b))
                EV = np.zeros(res["states"])
                a0, bup, lc = np.zeros(nblk), np.zeros(nblk), np.zeros(nblk)
                g.eigsolve(1, wl.npl, EV, a0, bup, lc)           # bounds (Lanczos) and first filter
                g.sync()
                if prec == "mixed":
                    g.profile(True)
                g.timer_start()
                g.eigsolve(2, wl.npl, EV, a0, bup, lc)
                ms = g.timer_stop()
                res[f"{prec}_ms_per_step"] = round(ms, 2)
                if prec == "mixed":
                    n_l, kms, by = g.profile_read()
                    g.profile(False)
                    res["stencil_gbs"] = round(by / (kms * 1e-3) / 1e9, 1) if kms > 0 else None
                evs[prec] = EV.copy()
            finally:
                g.close()
        if skip_steps:
            pass
        elif "fp64" in evs:
            off, err = 0, 0.0
            for (_, _, n) in blocks:
                err = max(err, float(np.max(np.abs(evs["mixed"][off:off + n // 2] - evs["fp64"][off:off + n // 2]))))
                off += n
            res["eig_err_lowest_half_ha"] = err
            res["speedup_mixed_vs_fp64"] = round(res["fp64_ms_per_step"] / res["mixed_ms_per_step"], 2)
        else:
            res["fp64_ms_per_step"] = None
            res["fp64_note"] = "not run: FP64 Rayleigh-Ritz of 8 x ~1000 states takes minutes per step on GB300 FP64"
        if scf_cell:
            # the full mixed-precision SCF to 1e-6 (src/scf.m) on this cell, from the atomic density
            S.Veff = None
            g = CyclixGPU(S, blocks, "mixed")
            try:
                for b, (_, _, n) in enumerate(blocks):
                    g.set_psi(b, initial_psi(S.N, n, 900 + b))
                t0 = time.perf_counter()
                r, EV, rho, V, hist = g.scf(S, scf_tol=1e-6, max_scf=max_scf)
                res["scf_mixed"] = {"n_scf": r.n_scf, "converged": bool(r.converged), "E_per_atom_ha": r.Etotal / S.n_atm,
                                    "err": r.err,
                                    "wall_s": round(time.perf_counter() - t0, 1), "general_eig_solves": g.eig_fallbacks(),
                                    "history_E_per_atom": [round(float(e), 10) for (e, _) in hist]}
            finally:
                g.close()
        print(json.dumps(res), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--only-mixed", action="store_true",
                    help="profiling mode: time only the mixed-precision device-resident steps (no CPU baseline, FP64 arm or e2e)")
    ap.add_argument("--workload", default=WORKLOAD, help="workload name (profiling mode)")
    ap.add_argument("--ramp", type=int, default=6, help="untimed SCF ramp-up steps before the warm-up steps")
    ap.add_argument("--max-scf", type=int, default=40, help="SCF step limit of the full-SCF configuration (--configs)")
    ap.add_argument("--scf-only", action="store_true", help="--configs: only the full SCF of the SCF cell")
    ap.add_argument("--configs", action="store_true",
                    help="one eigSolver step of every workload (mixed and FP64) and the full mixed SCF of the 384-atom cell")
    args = ap.parse_args()
    warmup = max(3, args.warmup)
    rank = env_int("RANK", 0)
    world = env_int("WORLD_SIZE", 1)

    from cyclix_msparc_gb300.workloads import WORKLOADS, make_system, block_layout
    wl = WORKLOADS[WORKLOAD]
    config = {"workload": WORKLOAD, "grid": [wl.Nr, wl.Nt, wl.Nz], "fd_order": 12, "Ns": list(wl.Ns), "filter_degree": wl.npl,
              "n_atoms": wl.n_atm, "bloch": "nu=1", "step": "eigSolver: Chebyshev filter + H*psi + Rayleigh-Ritz, steady state (after 6 untimed SCF ramp-up steps)",
              "l2": "inputs larger than L2 (psi complex64 302 MB)", "parallelism": f"replicas x{args.gpus}"}

    if args.impl == "reference":
        if rank != 0:
            return 0
        S = make_system(wl)
        vals = []
        info = None
        for i in range(warmup + args.steps):
            ms, cores, sample = cpu_baseline(S, wl.Ns[0], wl.npl)
            info = (cores, sample)
            if i >= warmup:
                vals.append(ms)
        v = statistics.mean(vals)
        line = {"impl": "reference", "metric": METRIC, "value": round(v, 3), "unit": "ms", "n_gpus": args.gpus, "steps": args.steps,
                "warmup": warmup, "ms_per_step": round(v, 3), "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
                "dtype": "c128", "data": "synthetic (seeded)", "config": config,
                "cpu_baseline": {"value": round(v, 3), "unit": "ms", "cores": info[0], "kind": "port", "sample": info[1]},
                "e2e": {"value": round(v, 3), "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                "note": "the reference is MATLAB (not installable here); this arm times the NumPy/SciPy restatement of it"}
        print(json.dumps(line), flush=True)
        return 0

    if args.configs:
        config_lines(None if args.workload == WORKLOAD else args.workload, args.max_scf, args.scf_only)
        return 0

    if args.only_mixed:
        wlp = WORKLOADS[args.workload]
        S = make_system(wlp)
        g, ms, launches, _, prof, _, _, fb = gpu_step_times(S, block_layout(wlp, S), "mixed", args.steps, warmup, wlp.npl,
                                                            profile_stencil=True, ramp=args.ramp)
        g.close()
        n_launch, stencil_ms, stencil_bytes, apply_ms = prof
        print(json.dumps({"mode": "only-mixed", "workload": args.workload, "ms_per_step": round(ms, 3),
                          "stencil_avg_ms": round(stencil_ms / max(n_launch, 1), 4),
                          "stencil_gbs": round(stencil_bytes / (stencil_ms * 1e-3) / 1e9, 1) if stencil_ms > 0 else None,
                          "nl_apply_avg_ms": round(apply_ms / max(n_launch, 1), 4), "eig_fallbacks": fb,
                          "launches_per_step": launches}), flush=True)
        return 0

    dist = None
    if world > 1:
        # replicas: every rank runs the whole workload on its own GPU; no data-path collective
        import torch.distributed as dist_mod
        dist_mod.init_process_group("gloo")
        dist = dist_mod
        from cyclix_msparc_gb300.msparc import select_device
        select_device(env_int("LOCAL_RANK", 0))
    S = make_system(wl)
    blocks = block_layout(wl, S)
    hbm_peak, _, peak_kind = measured_peaks()

    # CPU baseline first (spawned processes; before any GPU work in this process)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        ms, cores, sample = cpu_baseline(S, wl.Ns[0], wl.npl)
        cpu = {"value": round(ms, 1), "unit": "ms", "cores": cores, "kind": "port", "sample": sample}

    if dist:
        dist.barrier()
    clocks = ClockSampler(env_int("LOCAL_RANK", 0))
    clocks.start()
    g, ms_mixed, launches, ev_mixed, prof, count, bounds, fb_mixed = gpu_step_times(S, blocks, "mixed", args.steps, warmup, wl.npl,
                                                                                     profile_stencil=True, ramp=args.ramp)
    clk = clocks.stop()
    ms_mixed = max_over_ranks(ms_mixed, dist)
    e2e_ms, h2d, d2h = e2e_host(g, count + 1, wl.npl, max(2, min(args.steps, 3)), bounds)
    g.close()
    # plain FP64 arm (same steps, fewer repetitions: it is ~5x slower)
    g64, ms_fp64, _, ev_fp64, _, _, _, _ = gpu_step_times(S, blocks, "fp64", max(1, min(args.steps, 3)), warmup, wl.npl,
                                                          ramp=args.ramp)
    g64.close()
    nlow = wl.Ns[0] // 2
    ev_err = float(np.max(np.abs(ev_mixed[:nlow] - ev_fp64[:nlow])))

    n_launch, stencil_ms, stencil_bytes, apply_ms = prof
    achieved = stencil_bytes / (stencil_ms * 1e-3) / 1e9 if stencil_ms > 0 else 0.0
    per_launch_bytes = stencil_bytes / max(n_launch, 1)
    # DRAM bytes of one three-array launch from the committed ncu summary of this kernel and workload
    traffic = None
    tf = ROOT / "profiles" / "cheb_tma_kernel_cyclic-96x24x64-ns256.md"
    if tf.exists():
        for ln in tf.read_text().splitlines():
            if ln.startswith("| dram_bytes_per_launch"):
                try:
                    traffic = int(ln.split("|")[2].strip())
                except ValueError:
                    traffic = None
    if rank != 0:
        return 0
    line = {
        "metric": METRIC, "value": round(ms_mixed, 3), "unit": "ms", "n_gpus": args.gpus, "steps": args.steps, "warmup": warmup,
        "ms_per_step": round(ms_mixed, 3), "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "c64 filter / bf16x9 GEMM / f64 eig", "data": "synthetic (seeded)", "config": config,
        "fp64_ms_per_step": round(ms_fp64, 3), "speedup_mixed_vs_fp64": round(ms_fp64 / ms_mixed, 3),
        "eig_err_mixed_vs_fp64_ha": ev_err,
        "stencil_gbs": round(achieved, 1),
        "nl_apply_avg_ms": round(apply_ms / max(n_launch, 1), 4),
        "eig_general_solver_steps": fb_mixed,
        "roofline": {"bound": "hbm", "kernel": "cheb_tma_kernel (fused H*psi local part + Chebyshev step, complex64)", "achieved": round(achieved, 1),
                     "peak": hbm_peak, "peak_kind": peak_kind, "unit": "GB/s", "frac": round(achieved / hbm_peak, 4),
                     "traffic": traffic, "traffic_launch_algorithmic_bytes": 3 * S.N * wl.Ns[0] * 8 + 4 * S.N,
                     "algorithmic_bytes_per_launch": per_launch_bytes,
                     "avg_launch_ms": round(stencil_ms / max(n_launch, 1), 4)},
        "cpu_baseline": cpu,
        "e2e": {"value": round(e2e_ms, 3), "unit": "ms", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": int(round(launches * args.steps)),
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
