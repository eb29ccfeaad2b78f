#!/usr/bin/env python3
"""Benchmark of the Cyclix SCF step on one GB300: mixed precision vs plain FP64.

A step is one pass of the SCF loop of src/scf.m:111-306 as cx_scf_step runs it: the eigSolver
step over all Bloch blocks (Chebyshev filter of degree 24, H*psi, Rayleigh-Ritz: Gram, Cholesky,
projected Hamiltonian, subspace eigensolver, sort, rotation, W-normalisation), occupations,
density, the AAR Poisson solve, LDA_PW potential, energy, error and Pulay mixing.  Workload: the
batched cyclic cell, 16 Bloch wavenumbers nu = 0..15 on a 64 x 16 x 48 grid (FD order 12) with
uneven block sizes drawn in [96, 320] (3,345 states), 96 atoms with 4 KB projectors and Gaussian
pseudocharges (seeded synthetic inputs).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  ``value`` is the device-timed mixed-precision SCF step (inputs
resident in HBM; psi = 1.3 GB complex64 > L2, so no flush is needed); ``e2e`` is the same step
through the C-ABI with S.psi on the host (cx_scf_step with psi copied in and out every step from
page-locked memory).  Both arms run on to SCF convergence, and the line states the energy-per-atom
and occupied-eigenvalue differences of mixed against FP64.  ``--impl reference`` times the CPU
restatement of the reference (the reference itself is MATLAB and cannot run here) on all host
cores, on a bounded sample of each step scaled to the whole step (the scale factors are in the line).
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

WORKLOAD = "scf-batched-16nu-64x16x48-96at-ns96to320-m24"
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


class CpuScfStep:
    """The oracle's SCF step (oracle/cychel_ops.py, oracle/scf.py) on a bounded sample, scaled to
    the whole step.

    Sample of step i: block b = i mod nblk.  Measured: one whole H*psi over all Ns_b columns of
    block b on ``workers`` spawned processes; the Rayleigh-Ritz of block b at full size (orth by
    SVD, projected matrix, general eig, rotation, W-normalisation); the density contribution of
    block b; and, in full, the occupations, the AAR Poisson solve with its ILU preconditioner,
    LDA_PW and Pulay mixing.  Scaled: H*psi by (npl + 1) applications and sum(Ns)/Ns_b (linear
    in the states), the Rayleigh-Ritz by sum(Ns^2)/Ns_b^2 (its N x Ns x Ns products dominate),
    the density by sum(Ns)/Ns_b.  The scale factors are reported with each sample.
    """

    def __init__(self, S, blocks, npl, workers=None):
        import multiprocessing as mp
        from oracle import scf as OS
        self.S, self.blocks, self.npl = S, blocks, npl
        self.workers = workers or os.cpu_count() or 1
        self.ns = np.array([n for (_, _, n) in blocks], dtype=float)
        self.poisson = OS.PoissonOperator(S)         # ILU set-up: initialisation, not the step
        self.Veff = S.Veff if S.Veff is not None else None
        rho = S.rho_at.copy()
        self.phi, _, _ = self.poisson.solve(-4 * np.pi * (rho + S.b), None, 1e-8)
        if self.Veff is None:
            self.S.Veff = (self.phi + OS.lda_pw_potential(rho))[:, None]
        self.mixer = OS.PeriodicPulay(S.N)
        self.vin = self.S.Veff[:, 0].copy()
        self.it = 1
        self.ctx = mp.get_context("spawn")
        self.pool = None

    def __enter__(self):
        saved = {v: os.environ.get(v) for v in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")}
        # one BLAS thread per worker process: the workers cover every core
        for v in saved:
            os.environ[v] = "1"
        try:
            self.pool = self.ctx.Pool(self.workers)
        finally:
            for v, old_v in saved.items():
                if old_v is None:
                    os.environ.pop(v, None)
                else:
                    os.environ[v] = old_v
        return self

    def __exit__(self, *a):
        self.pool.close()
        self.pool.join()

    def step(self, i):
        import scipy.linalg as sla
        from oracle import scf as OS
        S = self.S
        b = i % len(self.blocks)
        k, spin, n = self.blocks[b]
        per = [n // self.workers + (1 if w < n % self.workers else 0) for w in range(self.workers)]
        t0 = time.perf_counter()
        ts = self.pool.map(_cpu_hpsi_chunk, [(100 * i + w, per[w], tuple(k), 0, S) for w in range(self.workers) if per[w] > 0])
        t_h = time.perf_counter() - t0
        rng = np.random.default_rng(i)
        X = rng.standard_normal((S.N, n)) + 1j * rng.standard_normal((S.N, n))
        HX = rng.standard_normal((S.N, n)) + 1j * rng.standard_normal((S.N, n))
        t1 = time.perf_counter()
        Q = sla.orth(X)
        Hs = Q.conj().T @ HX
        D, V = sla.eig(Hs)
        ind = np.argsort(D.real, kind="stable")
        P = Q @ V[:, ind]
        P *= 1.0 / np.sqrt(np.sum(S.W[:, None] * (P * P.conj()).real, axis=0))
        t2 = time.perf_counter()
        lam_f, occ = OS.occupations([np.sort(D.real)] * len(self.blocks), S.wkpt, S.bet, S.occfac, S.NegCharge, S.elec_T_type)
        rho = OS.electron_density([P], [occ[b]], S.wkpt[b:b + 1], S.N)
        t3 = time.perf_counter()
        rho = np.abs(rho) * (abs(S.NegCharge) / max(float(S.W @ np.abs(rho)), 1e-300))
        phi, _, iters = self.poisson.solve(-4 * np.pi * (rho + S.b), self.phi, 1e-8)
        vxc = OS.lda_pw_potential(rho)
        veff = phi + vxc
        OS.total_energy([np.sort(D.real)], [occ[b]], S.wkpt[b:b + 1], S.occfac, S.bet, lam_f, rho, S.b, phi, vxc, S.W, S.Eself,
                        S.E_corr, S.elec_T_type)
        self.vin = self.mixer(veff, self.vin, self.it)
        self.it += 1
        t4 = time.perf_counter()
        sc_h = (self.npl + 1) * self.ns.sum() / n
        sc_rr = float((self.ns ** 2).sum()) / n ** 2
        sc_d = self.ns.sum() / n
        t_occ_dens = (t3 - t2)
        total = t_h * sc_h + (t2 - t1) * sc_rr + t_occ_dens * sc_d + (t4 - t3)
        return total * 1e3, (t4 - t0) * 1e3, dict(block=b, Ns=int(n), hpsi_s=round(t_h, 3), hpsi_scale=round(sc_h, 2),
                                                    rr_s=round(t2 - t1, 3), rr_scale=round(sc_rr, 2),
                                                    density_s=round(t_occ_dens, 3), density_scale=round(sc_d, 2),
                                                    poisson_xc_mix_s=round(t4 - t3, 3), poisson_iters=int(iters))


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
class _NvtxRange:
    """An NVTX range around the timed passes (so that a profiler can be limited to them with
    ``ncu --nvtx --nvtx-include timed_scf_steps/``); a no-op when torch has no CUDA NVTX."""

    def __init__(self, name):
        self.name = name
        self.nv = None

    def __enter__(self):
        try:
            import torch
            torch.cuda.nvtx.range_push(self.name)
            self.nv = torch.cuda.nvtx
        except Exception:
            self.nv = None
        return self

    def __exit__(self, *a):
        if self.nv is not None:
            self.nv.range_pop()


def scf_arm(S, blocks, prec, steps, warmup, ramp, e2e_steps=0, max_passes=80, scf_tol=1e-6, profile=False, clocks=None):
    """SCF of ``S`` on the GPU through cx_scf_init / cx_scf_step / cx_scf_finish.

    ``ramp`` + ``warmup`` untimed passes, then ``steps`` passes timed with CUDA events on the
    handle's stream (device-resident psi), then (``profile``) one pass with per-launch stencil
    timing, then ``e2e_steps`` passes with psi copied in and out from page-locked host memory
    (wall clock), then passes until the SCF converges (or ``max_passes``) and cx_scf_finish
    (mixed: with the FP64 Rayleigh-quotient refinement)."""
    import ctypes as C
    from cyclix_msparc_gb300.msparc import CyclixGPU
    from cyclix_msparc_gb300.workloads import initial_psi
    g = CyclixGPU(S, blocks, prec)
    out = {}
    try:
        for b, (_, _, n) in enumerate(blocks):
            g.set_psi(b, initial_psi(S.N, n, 10 + b))
        g.scf_init(S, scf_tol=scf_tol, max_scf=max(1, max_passes))
        recs = []
        for _ in range(ramp + warmup):
            recs.append(g.scf_step())
        g.sync()
        g.launch_count(reset=True)
        fb0, hm0 = g.eig_fallbacks(), g.eig_hermitian()
        if clocks:
            clocks.start()
        timed = []
        with _NvtxRange("timed_scf_steps"):      # pushed before the timer starts (first use imports torch)
            g.timer_start()
            for _ in range(steps):
                timed.append(g.scf_step())
            ms = g.timer_stop()
        if clocks:
            out["clocks"] = clocks.stop()
        out["ms_per_step"] = ms / max(steps, 1)
        out["launches"] = g.launch_count(reset=True)
        out["general_eig"] = g.eig_fallbacks() - fb0
        out["hermitian_eig"] = g.eig_hermitian() - hm0
        out["timed"] = timed
        out["stencil_config"] = g.stencil_config()
        recs += timed
        if profile:
            g.profile(True)
            recs.append(g.scf_step())
            n_l, kms, by = g.profile_read()
            out["stencil"] = (n_l, kms, by, g.profile_read_apply(), g.profile_read_contract())
            g.profile(False)
        if e2e_steps:
            tot = int(sum(g.Ns))
            psi = np.empty(S.N * tot, dtype=np.complex128)
            off = 0
            for b in range(len(blocks)):
                psi[off * S.N:(off + g.Ns[b]) * S.N] = g.get_psi(b).reshape(-1, order="F")
                off += g.Ns[b]
            reg = g.lib.cx_host_register(psi.ctypes.data_as(C.c_void_p), psi.nbytes) == 0
            EV = np.zeros(tot)
            g.sync()
            t = time.perf_counter()
            for _ in range(e2e_steps):
                recs.append(g.scf_step(psi_host=psi, EigVal=EV))
            out["e2e_ms"] = (time.perf_counter() - t) / e2e_steps * 1e3
            out["e2e_recs"] = recs[-e2e_steps:]
            out["e2e_bytes"] = (psi.nbytes, psi.nbytes + EV.nbytes)
            if reg:
                g.lib.cx_host_unregister(psi.ctypes.data_as(C.c_void_p))
        while (not recs or not recs[-1].converged) and len(recs) < max_passes:
            recs.append(g.scf_step())
        res, EV, rho, V = g.scf_finish()
        out.update(result=res, EigVal=EV, recs=recs, passes=len(recs), converged=bool(recs[-1].converged))
    finally:
        g.close()
    return out


def eigsolver_arm(S, blocks, prec, steps, warmup, npl, ramp=6):
    """Device-resident eigSolver steps of a fixed-potential workload (profiling): ramp + warmup
    untimed steps, ``steps`` timed (CUDA events), then one step with per-launch stencil timing."""
    from cyclix_msparc_gb300.msparc import CyclixGPU
    from cyclix_msparc_gb300.workloads import initial_psi
    g = CyclixGPU(S, blocks, prec)
    try:
        for b, (_, _, n) in enumerate(blocks):
            g.set_psi(b, initial_psi(S.N, n, 10 + b))
        nblk = len(blocks)
        EV = np.zeros(int(sum(g.Ns)))
        a0, bup, lc = np.zeros(nblk), np.zeros(nblk), np.zeros(nblk)
        count = 1
        for _ in range(ramp + warmup):
            g.eigsolve(count, npl, EV, a0, bup, lc)
            count += 1
        g.sync()
        g.launch_count(reset=True)
        fb0, hm0 = g.eig_fallbacks(), g.eig_hermitian()
        g.timer_start()
        for _ in range(steps):
            g.eigsolve(count, npl, EV, a0, bup, lc)
            count += 1
        ms = g.timer_stop() / max(steps, 1)
        launches = g.launch_count(reset=True) / max(steps, 1)
        paths = (g.eig_fallbacks() - fb0, g.eig_hermitian() - hm0, g.stencil_config())
        g.profile(True)
        g.eigsolve(count, npl, EV, a0, bup, lc)
        prof = g.profile_read() + (g.profile_read_apply(), g.profile_read_contract())
        g.profile(False)
    finally:
        g.close()
    return ms, launches, paths, prof


def occupied_eig_error(blocks, ev_a, ev_b, lam_f, bet):
    """max |ev_a - ev_b| over the occupied states of ev_b: below lambda_f + 5 / bet (occupation > 1e-12)."""
    off, err = 0, 0.0
    for (_, _, n) in blocks:
        sel = ev_b[off:off + n] < lam_f + 5.0 / bet
        if sel.any():
            err = max(err, float(np.max(np.abs(ev_a[off:off + n][sel] - ev_b[off:off + n][sel]))))
        off += n
    return err


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
            t0 = time.perf_counter()
            r = scf_arm(S, blocks, "mixed", 0, 0, 0, max_passes=max_scf + 3)
            recs = r["recs"]
            res["scf_mixed"] = {"n_scf": r["result"].n_scf, "passes": r["passes"], "converged": r["converged"],
                                "E_per_atom_ha": r["result"].Etotal / S.n_atm, "err": r["result"].err,
                                "wall_s": round(time.perf_counter() - t0, 1),
                                "ms_per_step_last5": round(float(np.mean([x.step_ms for x in recs[-5:]])), 1),
                                "poisson": poisson_roofline(S, recs[-5:], measured_peaks()[0]),
                                "history_E_per_atom": [round(float(x.Etotal) / S.n_atm, 10) for x in recs if x.density_updated],
                                "history_err": [float(x.err) for x in recs if x.density_updated]}
        print(json.dumps(res), flush=True)


def poisson_roofline(S, recs, hbm_peak):
    """Roofline of the AAR Poisson solve (matrix-free Lap_std, Jacobi preconditioner) over the
    passes' device time, against GB300's FP64 rate (the solve is not HBM-bound; its vectors stay in
    L2, and it mostly waits at grid barriers).  Per point a
    Richardson iteration does about 60 FP64 operations (the 37-point stencil with its radial and
    theta factors, the residual, the preconditioner, the history differences and the update) and
    an Anderson iteration (every p = 6th) about 50 more (the upper triangle of DF'DF and DF'res,
    m = 7, and the update); the bytes (read x and f, write r and x: 4 N 8 per iteration, plus
    2 m N 8 of history every 6th) stay in L2.  peak = GB300's nominal FP64 rate (1.25 TFLOP/s:
    not among the measured peaks)."""
    its = sum(r.poisson_iters for r in recs)
    ms = sum(r.poisson_ms for r in recs)
    if its == 0 or ms <= 0:
        return None
    flops = its * 60.0 * S.N + (its // 6) * 50.0 * S.N
    by = its * 4 * S.N * 8 + (its // 6) * 2 * 7 * S.N * 8
    gfs = flops / (ms * 1e-3) / 1e9
    return {"bound": "latency (grid barriers; FP64 pipe 19 % busy under ncu)", "iters_per_step": round(its / len(recs), 1),
            "ms_per_step": round(ms / len(recs), 3),
            "achieved": round(gfs, 1), "peak": 1250.0, "peak_kind": "nominal", "unit": "GFLOP/s", "frac": round(gfs / 1250.0, 4),
            "bytes_gbs": round(by / (ms * 1e-3) / 1e9, 1), "hbm_peak_gbs": hbm_peak}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--only-mixed", action="store_true",
                    help="profiling mode: time only the mixed-precision device-resident steps (no CPU baseline, FP64 arm or e2e)")
    ap.add_argument("--workload", default=WORKLOAD, help="SCF workload name")
    ap.add_argument("--ramp", type=int, default=6, help="untimed SCF passes before the warm-up passes")
    ap.add_argument("--fp64-steps", type=int, default=5, help="timed passes of the plain FP64 arm")
    ap.add_argument("--max-passes", type=int, default=60, help="SCF pass limit of each arm")
    ap.add_argument("--max-scf", type=int, default=40, help="SCF step limit of the full-SCF configuration (--configs)")
    ap.add_argument("--scf-only", action="store_true", help="--configs: only the full SCF of the SCF cell")
    ap.add_argument("--configs", action="store_true",
                    help="one eigSolver step of every workload (mixed and FP64) and the full mixed SCF of the 384-atom cell")
    args = ap.parse_args()
    warmup = max(3, args.warmup)
    rank = env_int("RANK", 0)
    world = env_int("WORLD_SIZE", 1)

    from cyclix_msparc_gb300.workloads import WORKLOADS, make_system, block_layout
    if args.configs:
        config_lines(None if args.workload == WORKLOAD else args.workload, args.max_scf, args.scf_only)
        return 0
    wl = WORKLOADS[args.workload]
    config = {"workload": wl.name, "grid": [wl.Nr, wl.Nt, wl.Nz], "fd_order": 12, "blocks": len(wl.Ns), "Ns": list(wl.Ns),
              "states": int(sum(wl.Ns)), "filter_degree": wl.npl, "n_atoms": wl.n_atm, "xc": "LDA_PW",
              "bloch": f"nu = 0..{len(wl.kpts) - 1}" if len(wl.kpts) > 1 else "one wavenumber",
              "step": "one SCF pass (src/scf.m:111-306): eigSolver of all blocks + occupations + density + AAR Poisson + LDA_PW + "
                      "energy + Pulay mixing, steady state (after untimed ramp-up passes)",
              "l2": "inputs larger than L2 (psi complex64 {:.2f} GB)".format(wl.N * sum(wl.Ns) * 8 / 1e9),
              "parallelism": f"replicas x{args.gpus}"}

    if args.impl == "reference":
        if rank != 0:
            return 0
        S = make_system(wl)
        blocks = block_layout(wl, S)
        vals, samples, infos = [], [], []
        with CpuScfStep(S, blocks, wl.npl) as cpu:
            for i in range(warmup + args.steps):
                ms, sample_ms, info = cpu.step(i)
                if i >= warmup:
                    vals.append(ms)
                    samples.append(sample_ms)
                    infos.append(info)
            cores = cpu.workers
        v = statistics.mean(vals)
        line = {"impl": "reference", "metric": METRIC, "value": round(v, 3), "unit": "ms", "n_gpus": args.gpus, "steps": args.steps,
                "warmup": warmup, "ms_per_step": round(v, 3), "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
                "dtype": "c128", "data": "synthetic (seeded)", "config": config,
                "cpu_baseline": {"value": round(v, 3), "unit": "ms", "cores": cores, "kind": "port", "extrapolated": True,
                                 "sample_ms_per_step": round(statistics.mean(samples), 1),
                                 "sample": "per step, block i mod 16 measured in full (one whole H*psi over all its states on "
                                           f"{cores} spawned processes, its Rayleigh-Ritz, its density), the occupations, AAR Poisson "
                                           "(ILU), LDA_PW and Pulay mixing measured in full; H*psi scaled by (npl+1) x sum(Ns)/Ns_b, "
                                           "Rayleigh-Ritz by sum(Ns^2)/Ns_b^2, density by sum(Ns)/Ns_b",
                                 "per_step": infos},
                "e2e": {"value": round(v, 3), "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                "note": "the reference is MATLAB (not installable here); this arm times the NumPy/SciPy restatement of it"}
        print(json.dumps(line), flush=True)
        return 0

    if args.only_mixed:
        S = make_system(wl)
        if not wl.scf:
            ms, launches, (gen, herm, cfg), prof = eigsolver_arm(S, block_layout(wl, S), "mixed", args.steps, warmup, wl.npl,
                                                                 args.ramp)
            n_launch, stencil_ms, stencil_bytes, apply_ms, contract_ms = prof
            print(json.dumps({"mode": "only-mixed", "unit": "eigSolver step", "workload": args.workload, "ms_per_step": round(ms, 3),
                              "stencil_avg_ms": round(stencil_ms / max(n_launch, 1), 4),
                              "stencil_gbs": round(stencil_bytes / (stencil_ms * 1e-3) / 1e9, 1) if stencil_ms > 0 else None,
                              "nl_apply_avg_ms": round(apply_ms / max(n_launch, 1), 4),
                              "nl_contract_avg_ms": round(contract_ms / max(n_launch, 1), 4), "general_eig": gen, "hermitian_eig": herm,
                              "launches_per_step": launches, "stencil_config": cfg}), flush=True)
            return 0
        r = scf_arm(S, block_layout(wl, S), "mixed", args.steps, warmup, args.ramp, profile=True, max_passes=0)
        n_launch, stencil_ms, stencil_bytes, apply_ms, contract_ms = r["stencil"]
        print(json.dumps({"mode": "only-mixed", "unit": "SCF step", "workload": args.workload, "ms_per_step": round(r["ms_per_step"], 3),
                          "stencil_avg_ms": round(stencil_ms / max(n_launch, 1), 4),
                          "stencil_gbs": round(stencil_bytes / (stencil_ms * 1e-3) / 1e9, 1) if stencil_ms > 0 else None,
                          "nl_apply_avg_ms": round(apply_ms / max(n_launch, 1), 4),
                          "nl_contract_avg_ms": round(contract_ms / max(n_launch, 1), 4), "general_eig": r["general_eig"],
                          "hermitian_eig": r["hermitian_eig"], "launches_per_step": r["launches"] / max(args.steps, 1),
                          "poisson": poisson_roofline(S, r["timed"], 6793.4)}), flush=True)
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
        vals, samples = [], []
        with CpuScfStep(S, blocks, wl.npl) as c:
            for i in range(3):
                ms, sample_ms, _ = c.step(i)
                vals.append(ms)
                samples.append(sample_ms)
            cores = c.workers
        S.Veff = None
        cpu = {"value": round(statistics.mean(vals), 1), "unit": "ms", "cores": cores, "kind": "port", "extrapolated": True,
               "sample_ms_per_step": round(statistics.mean(samples), 1),
               "sample": "3 steps, each: one block measured in full (whole H*psi over its states, its Rayleigh-Ritz, its "
                         "density), occupations, AAR Poisson, LDA_PW and mixing in full; scaled to all 16 blocks and npl+1 H*psi"}

    if dist:
        dist.barrier()
    clocks = ClockSampler(env_int("LOCAL_RANK", 0))
    mixed = scf_arm(S, blocks, "mixed", args.steps, warmup, args.ramp, e2e_steps=args.steps, max_passes=args.max_passes,
                    profile=True, clocks=clocks)
    ms_mixed = max_over_ranks(mixed["ms_per_step"], dist)
    fp64 = scf_arm(S, blocks, "fp64", args.fp64_steps, warmup, args.ramp, max_passes=args.max_passes)
    res_m, res_d = mixed["result"], fp64["result"]
    e_err = abs(res_m.Etotal - res_d.Etotal) / S.n_atm
    ev_err = occupied_eig_error(blocks, mixed["EigVal"], fp64["EigVal"], res_d.lambda_f, S.bet)

    n_launch, stencil_ms, stencil_bytes, apply_ms, contract_ms = mixed["stencil"]
    achieved = stencil_bytes / (stencil_ms * 1e-3) / 1e9 if stencil_ms > 0 else 0.0
    per_launch_bytes = stencil_bytes / max(n_launch, 1)
    # DRAM bytes of one three-array launch from the committed ncu summary of this kernel and workload
    traffic = None
    tf = ROOT / "profiles" / f"cheb_tma_kernel_{wl.name}.md"
    if tf.exists():
        for ln in tf.read_text().splitlines():
            if ln.startswith("| dram_bytes_per_launch"):
                try:
                    traffic = int(ln.split("|")[2].strip())
                except ValueError:
                    traffic = None
    if rank != 0:
        return 0
    h2d, d2h = mixed["e2e_bytes"]
    line = {
        "metric": METRIC, "value": round(ms_mixed, 3), "unit": "ms", "n_gpus": args.gpus, "steps": args.steps, "warmup": warmup,
        "ms_per_step": round(ms_mixed, 3), "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "c64 filter / 3xTF32 tensor-core GEMM / f64 eig, Poisson, SCF", "data": "synthetic (seeded)", "config": config,
        "fp64_ms_per_step": round(fp64["ms_per_step"], 3), "speedup_mixed_vs_fp64": round(fp64["ms_per_step"] / ms_mixed, 3),
        "error_mixed_vs_fp64": {"energy_ha_per_atom": e_err, "occupied_eigenvalues_ha": ev_err,
                                "mixed": {"E_per_atom": res_m.Etotal / S.n_atm, "passes": mixed["passes"], "converged": mixed["converged"],
                                          "scf_err": res_m.err},
                                "fp64": {"E_per_atom": res_d.Etotal / S.n_atm, "passes": fp64["passes"], "converged": fp64["converged"],
                                         "scf_err": res_d.err}},
        "stencil_gbs": round(achieved, 1),
        "nl_apply_avg_ms": round(apply_ms / max(n_launch, 1), 4),
        "nl_contract_avg_ms": round(contract_ms / max(n_launch, 1), 4),
        "eig_paths_timed": {"general_solver": mixed["general_eig"], "hermitian_part": mixed["hermitian_eig"]},
        "timed_passes": [{"step_ms": round(x.step_ms, 1), "filter_ms": round(x.filter_ms, 1), "rayleigh_ritz_ms": round(x.rr_ms, 1),
                          "poisson_ms": round(x.poisson_ms, 1), "poisson_iters": x.poisson_iters, "scf_err": float(x.err)}
                         for x in mixed["timed"]],
        "e2e_passes_step_ms": [round(x.step_ms, 1) for x in mixed.get("e2e_recs", [])],
        "stencil_config": mixed["stencil_config"],
        "poisson": poisson_roofline(S, mixed["timed"], hbm_peak),
        "roofline": {"bound": "hbm", "kernel": "cheb_tma_kernel (fused H*psi local part + Chebyshev step, complex64)",
                     "achieved": round(achieved, 1), "peak": hbm_peak, "peak_kind": peak_kind, "unit": "GB/s",
                     "frac": round(achieved / hbm_peak, 4), "traffic": traffic,
                     "traffic_launch_algorithmic_bytes": 3 * S.N * int(sum(wl.Ns)) * 8 + 4 * S.N,
                     "algorithmic_bytes_per_launch": per_launch_bytes, "avg_launch_ms": round(stencil_ms / max(n_launch, 1), 4)},
        "cpu_baseline": cpu,
        "e2e": {"value": round(mixed["e2e_ms"], 3), "unit": "ms", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "steps": args.steps},
        "gpu_launches": int(mixed["launches"]),
        "clocks": mixed.get("clocks"),
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
