"""Benchmark: converged least-stable modes per second on one GB300.

Workload (the configuration the metric is quoted on): 4096 temporal
instances, N uniform over {48, 64, 96, 128} (pencils of order 240-640),
alpha ~ U[0.05, 0.4], beta ~ U[0, 0.3], Re ~ log-U[300, 3000],
M ~ U[0, 2] (clamped to >= 1e-3), seeded with PCG64(20261203 + rank).
Mean profiles are synthetic with the stated shapes: U = erf(y/2), V = W = 0,
T by Crocco-Busemann with an adiabatic Tw, rho = 1/T, 2000 rows on [0, 60];
Sutherland viscosity with S/T_inf = 0.3815, Pr = 0.72, Streett map with
ymax = 50 and half the points below y = 2.

One step = one pass of the seeded mixed-precision path over the whole batch
(STAB_MODE_COARSE: a full spectrum at N = 32 in double-word arithmetic for
the candidate shifts; the top candidate polished at full N from its N = 32
eigenvector by complex64 LU shift-invert with FP64 residuals, with a
double-word LU retry where that contracts slowly; instances whose seed
spectrum did not resolve the mode take a second seed level at N = 48, its
four candidates polished side by side and trusted when that level resolved
the mode or both levels agree on it; the rest keep an unverified pair or
take the plain FP64 path).  A mode counts as converged when it agrees with the plain FP64
path (the full GPU spectrum, itself checked against the CPU oracle by the
tests) to |d omega| / |omega| <= 1e-10 and its eigenvector to 1e-8.  The
working set (393 MB of profiles and ~7 GB of matrices) is far larger than
L2, so no flush is needed.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "converged least-stable modes/sec at |d omega|<=1e-10 (seeded+mixed vs plain FP64)"
UNIT = "modes/s"
TOL = 1e-10
T0_SUTH = 110.4 / 0.3815
HBM_FALLBACK_GBS = 6800.0  # used only when MEASURED_PEAKS.json is absent


def bf16_peak():
    """(TFLOP/s, source) of the cuBLAS bf16 burst measured on this machine, or None."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh)["bf16_tflops"]), "MEASURED_PEAKS.json bf16_tflops (measured)"
    except (OSError, KeyError, ValueError):
        return None


def hbm_peak():
    """(GB/s, source) of the HBM copy bandwidth measured on this machine."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh)["hbm_gbs"]), "MEASURED_PEAKS.json hbm_gbs (measured)"
    except (OSError, KeyError, ValueError):
        return HBM_FALLBACK_GBS, "fallback 6.8 TB/s"
# DRAM bytes per instance of the seed eigensolve, ncu at 1024 instances
# (profiles/k_eig_plain_dw_seed_traffic_1024.md: 47.85 GB read + 41.36 GB written)
COARSE_TRAFFIC_PER_INSTANCE = (47.85e9 + 41.36e9) / 1024
# kernel -> (work key of Batch.work(), bound, what the algorithmic count is)
KERNEL_WORK = {
    "k_eig_plain": ("eig_fp64", "fp64", "FP64 flops counted by the kernel (Householder reduction + QR sweeps)"),
    "k_eig_plain_coarse": ("eig_fp64_coarse", "dw", "flops counted by the kernel on the seed batch (N=32 by "
                           "default), run in double-word arithmetic"),
    "k_eig_plain_fallback": ("eig_fp64", "fp64", "FP64 flops counted by the kernel on the fallback instances"),
    "k_lu_c": ("lu_c64", "fp32", "8/3 n^3 real flops per complex64 LU, per factorisation run"),
    "k_lu_tc": ("lu_c64", "hbm", "trailing-matrix traffic of the complex64 LU with 16-column panels: every "
                "panel step reads and writes A22, sum over steps of (n - k)^2 x 16 bytes = n^3 / 3 bytes per LU "
                "(work lu_c64 / 8)"),
    "k_lu_tc_tma": ("lu_c64", "hbm", "as k_lu_tc (n^3 / 3 bytes per LU)"),
    "k_lu_z": ("lu_c128", "fp64", "8/3 n^3 real flops per complex128 LU, per factorisation run"),
    "k_lu_dz": ("lu_c128", "dw", "8/3 n^3 real flops per double-word complex LU, per factorisation run"),
}


def workload(count: int, seed: int):
    """Run parameters (dicts) and one contiguous (count, 2000, 6) profile array."""
    from scipy.special import erf
    rng = np.random.Generator(np.random.PCG64(seed))
    N = rng.choice([48, 64, 96, 128], size=count)
    al = rng.uniform(0.05, 0.4, count)
    be = rng.uniform(0.0, 0.3, count)
    Re = 10.0 ** rng.uniform(math.log10(300.0), math.log10(3000.0), count)
    M = np.maximum(rng.uniform(0.0, 2.0, count), 1e-3)
    y = np.linspace(0.0, 60.0, 2000)
    U = erf(y / 2.0)
    prof = np.empty((count, y.size, 6))
    for k in range(count):
        Tw = 1.0 + 0.2 * math.sqrt(0.72) * M[k] ** 2
        T = Tw + (1.0 - Tw) * U + 0.2 * M[k] ** 2 * U * (1.0 - U)
        prof[k, :, 0] = y
        prof[k, :, 1] = 1.0 / T
        prof[k, :, 2] = U
        prof[k, :, 3] = 0.0
        prof[k, :, 4] = 0.0
        prof[k, :, 5] = T
    params = [dict(itype=1, ny=int(N[k]), Ma=float(M[k]), Re=float(Re[k]), Pr=0.72, mattyp=1, T0=T0_SUTH,
                   yi=1.0 / 23.0, ymax=50.0, alpha=[float(al[k]), 0.0], beta=[float(be[k]), 0.0],
                   omega=[0.0, 0.0], top=0, wallt=0) for k in range(count)]
    return params, prof


VEC_TOL = 1e-8


def vec_diff(a, r):
    """max |a - r| after dividing each vector by its first max-modulus entry."""
    a = np.asarray(a)
    r = np.asarray(r)
    pa, pr = int(np.argmax(np.abs(a))), int(np.argmax(np.abs(r)))
    if a[pa] == 0 or r[pr] == 0 or not (np.all(np.isfinite(a)) and np.all(np.isfinite(r))):
        return np.inf
    return float(np.max(np.abs(a / a[pa] - r / r[pr])))


def surrogate_leg(ctx, stream, args):
    """Surrogate-seeded solve of the network workload: instances at N = 128 with
    (M, Re, alpha, beta, erf width s) drawn over the sweep ranges with s in
    [1.5, 3] (seed 20261204).  The network (6 -> 4 x 256 GELU -> 162, BF16) is
    trained here by the library's kernels on plain FP64 solves at N = 64 of
    the same distribution (a separate draw), then seeds MODE_SURROGATE; the
    coarse-seeded mode on the same batch is the method without it.  Every
    result is checked against the plain FP64 path at N = 128."""
    import torch
    import stab_gb300 as sg
    from stab_gb300 import surrogate as su
    t0 = time.perf_counter()
    ds = su.make_dataset(ctx, args.sur_train, 20261206)
    P = ds["params"]
    v = ds["valid"]
    X = su.features(P["M"], P["Re"], P["alpha"], P["beta"], P["width"])[v]
    sur = su.Surrogate(ctx, max_batch=8192)
    fit = sur.fit(X, ds["omega"][v], P["alpha"][v], ds["coef"][v], steps=8000, batch=1024)
    train = {"samples": int(v.sum()), "label_N": su.TRAIN_NY, "dataset_s": ds["seconds"], "fit_s": fit["seconds"],
             "steps": fit["steps"], "batch": fit["batch"], "final_loss": fit["losses"][-1][1]}
    n = args.sur_count
    Q = su.sample_params(n, 20261204)
    params = [su.stab_params(Q["M"][k], Q["Re"][k], Q["alpha"][k], Q["beta"][k], 128) for k in range(n)]
    profs = [su.erf_profile(Q["M"][k], Q["width"][k]) for k in range(n)]
    Xq = su.features(Q["M"], Q["Re"], Q["alpha"], Q["beta"], Q["width"])
    b = ctx.batch(params, profs)
    b.run(sg.MODE_PLAIN)
    truth, _, _, tst, _ = b.results()
    t_inf = time.perf_counter()
    w_hat = sur.seed_batch(b, Xq, Q["alpha"])
    infer_s = time.perf_counter() - t_inf
    rel = np.abs(w_hat - truth) / np.abs(truth)
    resolved = (np.real(truth / Q["alpha"]) > 0.0) & (np.real(truth / Q["alpha"]) < 3.0)
    out = {"workload": f"{n} temporal instances at N=128 (n=640), s~U[1.5,3], seed 20261204",
           "train": train, "inference_s": infer_s,
           "pred_rel_err_median": float(np.median(rel[resolved])) if np.any(resolved) else None,
           "pred_rel_err_note": "instances whose least-stable phase speed is in (0, 3)"}
    for name, mode in (("coarse_seeded", sg.MODE_COARSE), ("surrogate_seeded", sg.MODE_SURROGATE)):
        b.run(mode)          # warm-up (sizes pools, captures the graph)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(2):
            b.run(mode)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / 2
        eig, err, iters, st, _ = b.results()
        match = (np.abs(eig - truth) / np.abs(truth) <= TOL) & (tst == sg.ST_OK)
        ok = int(np.sum(match & np.isin(st, [sg.ST_OK, sg.ST_FELLBACK])))
        unv = int(np.sum(st == sg.ST_UNVERIFIED))
        unv_ok = int(np.sum(match & (st == sg.ST_UNVERIFIED)))
        out[name] = {"value": (ok + unv_ok) / (ms / 1000.0), "unit": UNIT, "ms_per_step": ms,
                     "converged": ok + unv_ok, "converged_trusted_status": ok,
                     "unverified": unv, "unverified_matching": unv_ok, "of": n, "counts": b.counts()}
    out["total_s"] = time.perf_counter() - t0
    b.close()
    sur.close()
    return out


def single_instance_leg(ctx, stream, cpu: bool):
    """Configs 0 and 1 as single-instance latencies: the plain temporal solve
    (N = 64, Streett map on [0, 50], full spectrum + least-stable
    eigenvector, M = 0.5, Re = 1000, alpha = 0.2) and the spatial solve
    (N = 96 crossflow, omega = 0.05, beta = 0.1, M = 0.8, Re = 2000: full
    spectrum of order 960, then the polish of the least-stable alpha), each
    checked against the CPU oracle on the same inputs when `cpu`."""
    import torch
    import stab_gb300 as sg
    from oracle import stab_oracle as so
    out = {}
    for name, itype, N, M, Re, a, b_, w, cross in (("config0_temporal_n64", 1, 64, 0.5, 1000.0, 0.2, 0.0, 0.0, False),
                                                  ("config1_spatial_n96", 2, 96, 0.8, 2000.0, 0.0, 0.1, 0.05, True)):
        y, vt = so.synthetic_profile(M, 50.0, crossflow=cross)
        prof = np.column_stack([y, vt])
        p = sg.StabParams.make(itype=itype, ny=N, Ma=M, Re=Re, Pr=0.72, mattyp=1, T0=T0_SUTH, yi=1.0 / 23.0,
                               ymax=50.0, alpha=a, beta=b_, omega=w)
        ctx.full_spectrum(p, prof)                       # warm-up: derivative tables, pools
        torch.cuda.synchronize()
        t = time.perf_counter()
        eig, vec, li, st = ctx.full_spectrum(p, prof)
        gpu_s = time.perf_counter() - t
        rec = {"gpu_full_spectrum_ms": 1000.0 * gpu_s, "order": p.m(), "status": int(st),
               "least": [float(eig[li].real), float(eig[li].imag)] if li >= 0 else None}
        if itype == 2 and li >= 0:
            t = time.perf_counter()
            pe, perr, pit, pst, _ = ctx.solve_batch([p], [prof], sg.MODE_SEEDED, seeds=[eig[li]])
            rec["gpu_polish_ms"] = 1000.0 * (time.perf_counter() - t)
            rec["polish_rel_change"] = float(abs(pe[0] - eig[li]) / abs(eig[li]))
        if cpu:
            sp = so.StabParams(mattyp=1, T0=T0_SUTH, Ma=M, Re=Re, Pr=0.72, ny=N, yi=1.0 / 23.0, ymax=50.0, ievec=1,
                               ider=1, top=0, wall=0, wallt=0, curve=0, itype=itype, alpha=complex(a),
                               beta=complex(b_), omega=complex(w))
            vt2 = vt.copy()
            vt2[:, 2] = 0.0
            t = time.perf_counter()
            es = so.solve(sp, y, vt2, want_vectors=(itype == 1))
            rec["cpu_oracle_s"] = time.perf_counter() - t
            if li >= 0:
                j = so.getevec_select(es.eig, eig[li])
                rec["rel_err_vs_oracle"] = float(abs(es.eig[j] - eig[li]) / abs(es.eig[j]))
        out[name] = rec
    return out


def serving_leg(ctx, args):
    """The serving loop (stab_gb300/serve.py): Poisson arrivals at 2000/s for
    args.serve_seconds of temporal and spatial requests with N ~ U{32..192},
    admitted by free device memory and solved in batches through the
    coarse-seeded path.  Reports throughput and latency percentiles."""
    import torch
    import stab_gb300 as sg
    from stab_gb300 import serve as sv
    reqs = sv.make_requests(2000.0, args.serve_seconds, 20261205)
    solve = sv.gpu_solver(ctx, sg.MODE_COARSE)
    solve(sv.make_requests(200.0, 0.05, 20261206))          # warm-up
    st = sv.serve(reqs, solve, lambda: torch.cuda.mem_get_info()[0], 4096)
    out = st.summary()
    out.update({"requests": len(reqs), "rate_per_s": 2000.0, "arrival_window_s": args.serve_seconds,
                "solved_ok_or_fellback": sum(1 for r in reqs if r.status in (sg.ST_OK, sg.ST_FELLBACK)),
                "mix": "50/50 temporal/spatial, N~U{32..192}, seed 20261205"})
    return out


def spatial_workload(count: int, seed: int):
    """Batched spatial sweep around the configuration-1 case: crossflow
    profiles W = 0.08 y exp(1 - y/1.5)/1.5 with U = erf(y/2) and the
    Crocco-Busemann T, N in {64, 96} (companion orders 640 and 960),
    omega ~ U[0.03, 0.07], beta ~ U[0.05, 0.15], log Re ~ U[log 1000, log 3000],
    M ~ U[0.5, 1.0]."""
    from oracle import stab_oracle as so
    rng = np.random.Generator(np.random.PCG64(seed))
    N = rng.choice([64, 96], size=count)
    om = rng.uniform(0.03, 0.07, count)
    be = rng.uniform(0.05, 0.15, count)
    Re = 10.0 ** rng.uniform(3.0, math.log10(3000.0), count)
    M = rng.uniform(0.5, 1.0, count)
    prof = np.empty((count, 2000, 6))
    for k in range(count):
        y, vt = so.synthetic_profile(float(M[k]), 50.0, crossflow=True)
        prof[k, :, 0] = y
        prof[k, :, 1:] = vt
    params = [dict(itype=2, ny=int(N[k]), Ma=float(M[k]), Re=float(Re[k]), Pr=0.72, mattyp=1, T0=T0_SUTH,
                   yi=1.0 / 23.0, ymax=50.0, alpha=[0.0, 0.0], beta=[float(be[k]), 0.0],
                   omega=[float(om[k]), 0.0], top=0, wallt=0) for k in range(count)]
    return params, prof


def spatial_score(w, st, ref, ref_st, ms):
    """modes/s and status counts of a coarse-seeded spatial pass against the plain result"""
    import stab_gb300 as sg
    rel = np.abs(w - ref) / np.maximum(np.abs(ref), 1e-300)
    trusted = np.isin(st, [sg.ST_OK, sg.ST_FELLBACK]) & (ref_st == sg.ST_OK)
    ok = trusted & (rel <= TOL)
    unver = (st == sg.ST_UNVERIFIED) & (ref_st == sg.ST_OK)
    return {"value": float(np.sum(ok)) / (ms / 1000.0), "unit": "modes/s", "ms_per_step": ms,
            "converged": int(np.sum(ok)), "trusted_but_wrong": int(np.sum(trusted & ~(rel <= TOL))),
            "unverified": int(np.sum(unver)), "unverified_matching": int(np.sum(unver & (rel <= TOL))),
            "status_histogram": {int(k): int(v) for k, v in zip(*np.unique(st, return_counts=True))}}


def spatial_leg(ctx, stream, count):
    """The batched spatial sweep: one plain FP64 pass (the reference
    result), then the coarse-seeded pass timed after a warm-up pass; modes/s
    of both and the count matching the plain result to 1e-10 with a trusted
    status."""
    import torch
    import stab_gb300 as sg
    params, prof = spatial_workload(count, 20261206)
    sp = [to_stab(d) for d in params]
    b = ctx.batch(sp, [prof[k] for k in range(count)])
    try:
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        b.run(sg.MODE_PLAIN)
        ev1.record(stream)
        torch.cuda.synchronize()
        plain_ms = ev0.elapsed_time(ev1)
        ref, _, _, ref_st, _ = b.results()
        b.run(sg.MODE_COARSE)
        torch.cuda.synchronize()
        ev0.record(stream)
        b.run(sg.MODE_COARSE)
        ev1.record(stream)
        torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1)
        w, err, iters, st, _ = b.results()
        counts = b.counts()
        # the same pass with another setting: without second-level trust by
        # agreement of the seed levels, and with the second level at N = 48
        def other(setter, reset):
            setter()
            try:
                b.run(sg.MODE_COARSE)
                torch.cuda.synchronize()
                ev0.record(stream)
                b.run(sg.MODE_COARSE)
                ev1.record(stream)
                torch.cuda.synchronize()
                w_o, _, _, st_o, _ = b.results()
                return spatial_score(w_o, st_o, ref, ref_st, ev0.elapsed_time(ev1))
            finally:
                reset()
        no_lc = other(lambda: ctx.set_option(sg.OPT_LEVEL_CONSISTENCY, 0),
                      lambda: ctx.set_option(sg.OPT_LEVEL_CONSISTENCY, 1))
        lev48 = other(lambda: ctx.set_option(sg.OPT_MEDIUM_NY_SPATIAL, 48),
                      lambda: ctx.set_option(sg.OPT_MEDIUM_NY_SPATIAL, 24))
    finally:
        b.close()
    rel = np.abs(w - ref) / np.maximum(np.abs(ref), 1e-300)
    trusted = np.isin(st, [sg.ST_OK, sg.ST_FELLBACK]) & (ref_st == sg.ST_OK)
    ok = trusted & (rel <= TOL)
    unver = (st == sg.ST_UNVERIFIED) & (ref_st == sg.ST_OK)
    return {"workload": f"{count} spatial crossflow instances, N in {{64, 96}} (companion orders 640, 960), "
                        "omega~U[.03,.07], beta~U[.05,.15], Re~logU[1000,3000], M~U[.5,1], seed 20261206",
            "coarse_seeded": {"value": float(np.sum(ok)) / (ms / 1000.0), "unit": "modes/s", "ms_per_step": ms,
                              "converged": int(np.sum(ok)), "of": count,
                              "trusted_but_wrong": int(np.sum(trusted & ~(rel <= TOL))),
                              "unverified": int(np.sum(unver)),
                              "unverified_matching": int(np.sum(unver & (rel <= TOL))),
                              "stages": counts,
                              "status_histogram": {int(k): int(v) for k, v in zip(*np.unique(st, return_counts=True))}},
            "no_level_consistency": no_lc,
            "second_level_n48": lev48,
            "plain_fp64": {"value": float(np.sum(ref_st == sg.ST_OK)) / (plain_ms / 1000.0), "unit": "modes/s",
                           "ms_per_step": plain_ms},
            "speedup_seeded_over_plain": (float(np.sum(ok)) / ms) / max(float(np.sum(ref_st == sg.ST_OK)) / plain_ms,
                                                                        1e-300)}


def to_stab(d):
    import stab_gb300 as sg
    return sg.StabParams.make(itype=d["itype"], ny=d["ny"], Ma=d["Ma"], Re=d["Re"], Pr=d["Pr"],
                              mattyp=d["mattyp"], T0=d["T0"], yi=d["yi"], ymax=d["ymax"],
                              alpha=complex(*d["alpha"]), beta=complex(*d["beta"]), omega=complex(*d["omega"]))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for ln in self.proc.stdout:
            self.rows.append([t.strip() for t in ln.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for q, nm in enumerate(names):
                if len(r) > 5 + q and r[5 + q].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(n_gpus):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def reduce_max(x, world):
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(x, world):
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def cpu_model() -> str:
    try:
        with open("/proc/cpuinfo") as fh:
            for ln in fh:
                if ln.lower().startswith(("model name", "cpu part", "hardware")):
                    return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.processor() or platform.machine()


def cpu_leg(params, prof, sample: int, procs: int, threads: int = 1):
    """The oracle (reference algorithm) on `sample` instances with `procs`
    processes of `threads` BLAS threads each: (modes/s, results, seconds)."""
    from oracle import baseline
    jobs = []
    for k in range(sample):
        d = dict(params[k])
        d["profile"] = prof[k]
        jobs.append(d)
    pool = baseline.pool(procs, threads)
    try:
        t0 = time.perf_counter()
        out = pool.map(baseline.solve_one, jobs, chunksize=1)
        dt = time.perf_counter() - t0
    finally:
        pool.close()
        pool.join()
    eig = np.array([complex(*o[0]) for o in out])
    return sample / dt, eig, dt


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    params, prof = workload(args.count, 20261203)
    procs = os.cpu_count() or 1
    sample = args.ref_sample
    times = []
    for it in range(args.warmup + args.steps):
        lo = (it * sample) % args.count
        sel = list(range(lo, lo + sample))
        rate, _, dt = cpu_leg([params[k] for k in sel], prof[sel], sample, procs)
        if it >= args.warmup:
            times.append(dt)
    ms = 1000.0 * statistics.mean(times)
    value = sample / (ms / 1000.0)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
            "config": {"workload": f"temporal sweep, {sample} of {args.count} instances per step, "
                                   "N in {48,64,96,128}, seed 20261203", "count": sample},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": procs, "kind": "port",
                             "sample": f"{sample} instances per step (ZGESV+ZGEEV('N','V') via scipy LAPACK, "
                                       f"{procs} single-thread processes)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--count", type=int, default=4096)
    ap.add_argument("--cpu-sample", type=int, default=64)
    ap.add_argument("--cpu-sample-threaded", type=int, default=16,
                    help="instances of the one-process multi-threaded CPU mode")
    ap.add_argument("--plain-reps", type=int, default=3, help="timed passes of the plain FP64 path")
    ap.add_argument("--spatial", type=int, default=256, help="instances of the batched spatial sweep leg (0: skip)")
    ap.add_argument("--variants", type=int, default=1, help="1: also time the pass with each stage's other "
                    "implementation (polish LU on CUDA cores, seed QR in shared memory)")
    ap.add_argument("--ref-sample", type=int, default=48)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--surrogate", type=int, default=1, help="1: also run the surrogate-seeded leg")
    ap.add_argument("--sur-train", type=int, default=8192)
    ap.add_argument("--sur-count", type=int, default=1024)
    ap.add_argument("--serve-seconds", type=float, default=1.0, help="arrival window of the serving leg (0: skip)")
    ap.add_argument("--seed-ny", type=int, default=32, help="N of the coarse seed spectrum (stab_set_seed_size)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    rank, world, local = dist_setup(args.gpus)
    if args.impl == "reference":
        return run_reference(args, rank, world)

    params, prof = workload(args.count, 20261203 + rank)
    # CPU baseline first: the spawn pools start before any GPU work.  Two
    # modes: (ii) one single-thread process per core over the instances,
    # (i) one process with one BLAS thread per core; the faster is reported.
    cpu = None
    if rank == 0 and args.cpu_sample > 0:
        procs = os.cpu_count() or 1
        rate, cpu_eig, dt = cpu_leg(params, prof, args.cpu_sample, procs)
        s1 = max(1, min(args.cpu_sample, args.cpu_sample_threaded))
        rate1, _, dt1 = cpu_leg(params, prof, s1, 1, procs)
        modes = {"processes": {"value": rate, "sample": args.cpu_sample, "seconds": dt,
                               "how": f"{procs} single-thread processes"},
                 "threads": {"value": rate1, "sample": s1, "seconds": dt1,
                             "how": f"1 process, OPENBLAS_NUM_THREADS={procs}"}}
        best = max(modes, key=lambda k: modes[k]["value"])
        cpu = {"value": modes[best]["value"], "unit": UNIT, "cores": procs, "kind": "port",
               "cpu_model": cpu_model(), "mode": best, "modes": modes,
               "sample": f"first {modes[best]['sample']} instances of the workload, "
                         f"{modes[best]['seconds']:.1f} s: oracle restatement of ZGESV+ZGEEV('N','V') "
                         f"(scipy LAPACK), {modes[best]['how']}"}

    import torch
    import stab_gb300 as sg
    torch.cuda.set_device(local)
    ctx = sg.Context(local)
    ctx.set_seed_size(args.seed_ny)
    stream = torch.cuda.Stream()          # a real stream: the legacy default would not order with ours
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    sp = [to_stab(d) for d in params]
    # pinned host copy of the inputs for the end-to-end leg
    prof_pinned = torch.from_numpy(prof).pin_memory()
    prof_np = prof_pinned.numpy()
    profiles = [prof_np[k] for k in range(args.count)]
    batch = ctx.batch(sp, profiles)
    # LU panel widths for the orders of this workload and of the N = 32 seeds
    tune = ctx.autotune(sorted({5 * d["ny"] for d in params} | {160}))
    # FP32 / FP64 / double-word multiply-add rates of this GPU, measured now:
    # the denominators of the kernels bound by those pipes
    peaks = ctx.peak_rates()

    # reference result: plain FP64 full spectrum on every instance; one
    # untimed pass (pool growth, first-use costs), then args.plain_reps timed
    batch.run(sg.MODE_PLAIN)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    plain_times = []
    for _ in range(args.plain_reps):
        e0.record(stream)
        batch.run(sg.MODE_PLAIN)
        e1.record(stream)
        torch.cuda.synchronize()
        plain_times.append(e0.elapsed_time(e1))
    plain_ms = statistics.mean(plain_times)
    ref_eig, _, _, ref_st, ref_vec = batch.results(want_vectors=True)
    plain_work = batch.work()

    # warm-up and timed steps of the seeded mixed path
    for _ in range(args.warmup):
        batch.run(sg.MODE_COARSE)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    barrier(world)
    torch.cuda.synchronize()
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for _ in range(args.steps):
        batch.run(sg.MODE_COARSE)
    t1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop()
    ms_local = t0.elapsed_time(t1) / args.steps
    eig, err, iters, status, vecs = batch.results(want_vectors=True)
    work = batch.work()
    rel = np.abs(eig - ref_eig) / np.maximum(np.abs(ref_eig), 1e-300)
    ok_val = (rel <= TOL) & np.isin(status, [sg.ST_OK, sg.ST_FELLBACK]) & (ref_st == sg.ST_OK)
    # eigenvector bar: within 1e-8 of the plain FP64 vector after dividing each
    # by its first max-modulus entry
    vdiff = np.array([vec_diff(a, r) for a, r in zip(vecs, ref_vec)])
    ok = ok_val & (vdiff <= VEC_TOL)
    converged_local = int(np.sum(ok))
    fell = int(np.sum(status == sg.ST_FELLBACK))
    # trusted statuses whose eigenvalue is not the plain path's least-stable one
    wrong_trusted = np.nonzero(np.isin(status, [sg.ST_OK, sg.ST_FELLBACK]) & (ref_st == sg.ST_OK)
                               & ~(rel <= TOL))[0]
    st_hist = {int(k): int(v) for k, v in zip(*np.unique(status, return_counts=True))}
    counts_last = batch.counts()

    # per-kernel breakdown of one extra step (CUDA events on the launch stream)
    ctx.reset_kernel_stats()
    ctx.eig_phases(reset=True)
    ctx.set_profiling(True)
    batch.run(sg.MODE_COARSE)
    stats = ctx.kernel_stats()
    ctx.set_profiling(False)
    phases = ctx.eig_phases(reset=True)
    # "stage:" entries time whole candidate rounds; they are not kernels
    stages = {k[6:]: round(v[1], 3) for k, v in stats.items() if k.startswith("stage:")}
    stats = {k: v for k, v in stats.items() if not k.startswith("stage:")}
    launches_per_step = sum(v[0] for v in stats.values())

    # the same pass with a stage switched to its other implementation (CUDA
    # events, two passes each after one untimed pass), for the design notes;
    # each variant's results are scored like the default pass's
    def score(b):
        e_s, _, _, st_s, v_s = b.results(want_vectors=True)
        rel_s = np.abs(e_s - ref_eig) / np.maximum(np.abs(ref_eig), 1e-300)
        trusted_s = np.isin(st_s, [sg.ST_OK, sg.ST_FELLBACK]) & (ref_st == sg.ST_OK)
        ok_s = trusted_s & (rel_s <= TOL) & (np.array([vec_diff(a, r) for a, r in zip(v_s, ref_vec)]) <= VEC_TOL)
        return {"converged": int(np.sum(ok_s)), "trusted_but_wrong": int(np.sum(trusted_s & ~(rel_s <= TOL))),
                "status_histogram": {int(k): int(v) for k, v in zip(*np.unique(st_s, return_counts=True))}}

    def variant_ms(setter, reset):
        setter()
        try:
            batch.run(sg.MODE_COARSE)
            torch.cuda.synchronize()
            v0, v1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            v0.record(stream)
            for _ in range(2):
                batch.run(sg.MODE_COARSE)
            v1.record(stream)
            torch.cuda.synchronize()
            return dict(ms=v0.elapsed_time(v1) / 2, **score(batch))
        finally:
            reset()
            batch.run(sg.MODE_COARSE)   # re-capture the default graph
    variants = None
    if args.variants:
        variants = {
            "default_ms": ms_local,
            "polish_lu_cuda_cores": variant_ms(lambda: ctx.set_arithmetic(sg.STAGE_POLISH_LU, sg.ARITH_FP32),
                                                  ctx.reset_arithmetic),
            "polish_lu_tensor_no_tma": variant_ms(lambda: ctx.set_option(sg.OPT_POLISH_LU_TMA, 0),
                                                     lambda: ctx.set_option(sg.OPT_POLISH_LU_TMA, 1)),
            "seed_qr_shared_memory": variant_ms(lambda: ctx.set_option(sg.OPT_SEED_QR_SHARED, 1),
                                                   lambda: ctx.set_option(sg.OPT_SEED_QR_SHARED, 0)),
        }
        # the batch eigensolver with 3 instances in flight per SM instead of
        # the occupancy's four (1 and 2 measured slower still)
        variants["eig_resident_3_per_sm"] = variant_ms(lambda: ctx.set_option(sg.OPT_EIG_RESIDENT, 3),
                                                          lambda: ctx.set_option(sg.OPT_EIG_RESIDENT, 0))
        # 64-thread eigensolver CTAs, eight per SM
        variants["eig_64_thread_ctas"] = variant_ms(lambda: ctx.set_option(sg.OPT_EIG_THREADS, 64),
                                                       lambda: ctx.set_option(sg.OPT_EIG_THREADS, 128))
        # the top candidate's polish started from a factorisation at the
        # shift and two inverse-iteration steps instead of the seed level's
        # eigenvector
        variants["no_seed_vectors"] = variant_ms(lambda: ctx.set_option(sg.OPT_SEED_VECTORS, 0),
                                                 lambda: ctx.set_option(sg.OPT_SEED_VECTORS, 1))
        # the N = 48 level's four candidates in rounds one after another
        # instead of side by side
        variants["sequential_candidates"] = variant_ms(
            lambda: ctx.set_option(sg.OPT_PARALLEL_CANDIDATES, 0),
            lambda: ctx.set_option(sg.OPT_PARALLEL_CANDIDATES, 1))
        # no double-word retry at the first candidate level (its failed and
        # slow instances go to the second level directly)
        variants["no_first_retry"] = variant_ms(lambda: ctx.set_option(sg.OPT_FIRST_RETRY, 0),
                                                lambda: ctx.set_option(sg.OPT_FIRST_RETRY, 1))
        # second-level trust only by the N = 48 top candidate's own quick
        # accept (without the agreement of the two seed levels)
        variants["no_level_consistency"] = variant_ms(lambda: ctx.set_option(sg.OPT_LEVEL_CONSISTENCY, 0),
                                                      lambda: ctx.set_option(sg.OPT_LEVEL_CONSISTENCY, 1))
        # the second candidate level at N = 40 or 24 instead of 48
        variants["medium_ny_40"] = variant_ms(lambda: ctx.set_option(sg.OPT_MEDIUM_NY, 40),
                                              lambda: ctx.set_option(sg.OPT_MEDIUM_NY, 48))
        variants["medium_ny_24"] = variant_ms(lambda: ctx.set_option(sg.OPT_MEDIUM_NY, 24),
                                              lambda: ctx.set_option(sg.OPT_MEDIUM_NY, 48))
        # the small N = 48 level batch on the 128-thread persistent grid
        # instead of the default 256-thread CTAs
        variants["eig_mid_off"] = variant_ms(lambda: ctx.set_option(sg.OPT_EIG_MID, 0),
                                                lambda: ctx.set_option(sg.OPT_EIG_MID, 1))
        # seed spectra at another N: a batch of its own (the seed size applies
        # to batches created afterwards), timed and checked like the default
        for sny in (28,):
            if sny == args.seed_ny:
                continue
            ctx.set_seed_size(sny)
            try:
                bs = ctx.batch(sp, profiles)
                bs.run(sg.MODE_COARSE)
                torch.cuda.synchronize()
                v0, v1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                v0.record(stream)
                for _ in range(2):
                    bs.run(sg.MODE_COARSE)
                v1.record(stream)
                torch.cuda.synchronize()
                variants["seed_ny_%d" % sny] = dict(ms=v0.elapsed_time(v1) / 2, **score(bs))
                bs.close()
            finally:
                ctx.set_seed_size(args.seed_ny)

    spatial = spatial_leg(ctx, stream, args.spatial) if (args.spatial and rank == 0) else None
    sur = surrogate_leg(ctx, stream, args) if (args.surrogate and rank == 0) else None
    single = single_instance_leg(ctx, stream, cpu=args.cpu_sample > 0) if rank == 0 else None
    serving = serving_leg(ctx, args) if (rank == 0 and args.serve_seconds > 0) else None

    # end-to-end through the C ABI call with host buffers (pinned), results read back
    barrier(world)
    torch.cuda.synchronize()
    te = time.perf_counter()
    for _ in range(args.e2e_steps):
        w_e2e, err_e2e, iters_e2e, st_e2e, _ = ctx.solve_batch(sp, profiles, sg.MODE_COARSE)
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - te) / args.e2e_steps
    ok_e2e = int(np.sum((np.abs(w_e2e - ref_eig) / np.maximum(np.abs(ref_eig), 1e-300) <= TOL)
                        & np.isin(st_e2e, [sg.ST_OK, sg.ST_FELLBACK])))

    ms = reduce_max(ms_local, world)
    converged = reduce_sum(converged_local, world)
    e2e_s = reduce_max(e2e_s, world)
    ok_e2e = reduce_sum(ok_e2e, world)
    plain_ms = reduce_max(plain_ms, world)
    if rank != 0:
        return 0

    value = converged / (ms / 1000.0)
    total = args.count * world
    # dominant kernel and its roofline; every kernel with counted work gets one
    dom = max(stats.items(), key=lambda kv: kv[1][1])
    dname = dom[0]
    rooflines = {}
    # a work counter can cover several kernels (the tensor-core LU's two
    # forms): its rate is over the time of all of them
    key_ms = {}
    for kname, (kl, kms) in stats.items():
        if kname in KERNEL_WORK:
            key_ms[KERNEL_WORK[kname][0]] = key_ms.get(KERNEL_WORK[kname][0], 0.0) + kms
    for kname, (kl, kms_own) in stats.items():
        if kname not in KERNEL_WORK or kms_own <= 0:
            continue
        wkey, bound, note = KERNEL_WORK[kname]
        kms = key_ms[wkey]
        if bound == "hbm":
            hp, hsrc = hbm_peak()
            ach = work[wkey] / 8.0 / (kms / 1000.0) / 1e9   # bytes over the same launches
            rooflines[kname] = {"bound": "hbm", "achieved": ach, "peak": hp, "unit": "GB/s", "frac": ach / hp,
                                "traffic": None, "kernel": kname, "launches": kl, "ms": kms_own,
                                "ms_of_work_counter": kms, "algorithmic": note, "peak_source": hsrc}
            continue
        # pipe-bound kernels: the multiply-add rate of their arithmetic,
        # measured in this run (stab_peak_rates)
        peak = {"fp64": peaks["fp64"], "fp32": peaks["fp32"], "dw": peaks["double_word_complex"]}[bound]
        ach = work[wkey] / (kms / 1000.0) / 1e12    # flops and time of the same launches
        rooflines[kname] = {"bound": bound, "achieved": ach, "peak": peak, "unit": "TFLOP/s",
                            "frac": ach / peak, "traffic": None, "kernel": kname, "launches": kl,
                            "ms": kms_own, "ms_of_work_counter": kms, "algorithmic": note,
                            "peak_source": "measured in this run: independent multiply-add chains on every SM "
                                           "(stab_peak_rates, %s)" % {"fp64": "FP64 FMA", "fp32": "FP32 FMA",
                                                                     "dw": "double-word complex"}[bound],
                            "frac_of_bf16_tensor_peak": ach / bf16_peak()[0] if bf16_peak() else None}
    if "k_eig_plain_coarse" in rooflines:
        # DRAM bytes per launch from the committed ncu capture of the same kernel
        # at 1024 instances, scaled by the instances of this launch (the
        # per-instance traffic is the same at 512 and 1024)
        rooflines["k_eig_plain_coarse"]["traffic"] = COARSE_TRAFFIC_PER_INSTANCE * args.count
        rooflines["k_eig_plain_coarse"]["traffic_unit"] = "bytes per launch (ncu capture at 1024, scaled)"
        # the same kernel against the measured copy bandwidth: its algorithmic
        # bytes (each m x m double-word matrix, 16 B entries, read once) and its
        # DRAM traffic, per second of the launch
        kl, kms = stats["k_eig_plain_coarse"]
        hp, hsrc = hbm_peak()
        seed_m = 5 * args.seed_ny
        alg = 16.0 * seed_m * seed_m * args.count
        rooflines["k_eig_plain_coarse"]["hbm_view"] = {
            "algorithmic_bytes": alg, "achieved_algorithmic_GBs": alg / (kms / 1000.0) / 1e9,
            "traffic_GBs": COARSE_TRAFFIC_PER_INSTANCE * args.count / (kms / 1000.0) / 1e9, "peak": hp,
            "frac_traffic": COARSE_TRAFFIC_PER_INSTANCE * args.count / (kms / 1000.0) / 1e9 / hp,
            "unit": "GB/s", "peak_source": hsrc,
            "note": "the N = 32 launch's bytes over both launches' time (the N = 48 level adds its own)"}
    roof = rooflines.get(dname, {"bound": "unknown", "kernel": dname, "achieved": None, "peak": None,
                                 "unit": None, "frac": None, "traffic": None})
    h2d = int(prof.nbytes + len(sp) * 120 + len(sp) * 4)
    d2h = int(len(sp) * (16 + 8 + 4 + 4))
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": "c64 LU, double-word seed eigensolve and retry LU, f64 residuals (plain path c128)",
        "data": "synthetic",
        "config": {"workload": "temporal sweep: 4096 instances/GPU, N in {48,64,96,128} (n = 240-640), "
                               "alpha~U[.05,.4], beta~U[0,.3], Re~logU[300,3000], M~U[0,2], seed 20261203",
                   "count_per_gpu": args.count, "seeds": f"double-word full spectrum at N={args.seed_ny}",
                   "l2": "working set > L2 (393 MB profiles, GBs of matrices); no flush"},
        "e2e": {"value": ok_e2e / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": 1000.0 * e2e_s, "call": "stab_solve_batch (host buffers, pinned)"},
        "converged": {"count": int(converged), "of": total, "fell_back": fell,
                      "criteria": "|d omega|/|omega| <= 1e-10 and eigenvector within 1e-8 after phase normalisation",
                      "eigenvalue_only": int(np.sum(ok_val)),
                      "status_histogram": st_hist, "stages": counts_last,
                      "trusted_but_wrong": int(wrong_trusted.size),
                      "unverified": int(np.sum((status == sg.ST_UNVERIFIED) & (ref_st == sg.ST_OK))),
                      "unverified_matching": int(np.sum((status == sg.ST_UNVERIFIED) & (ref_st == sg.ST_OK)
                                                        & (rel <= TOL))),
                      "trusted_but_wrong_examples": [
                          {"index": int(q), "got": [float(eig[q].real), float(eig[q].imag)],
                           "plain": [float(ref_eig[q].real), float(ref_eig[q].imag)], "status": int(status[q])}
                          for q in wrong_trusted[:16]],
                      "max_rel_err": float(np.nanmax(rel[ok])) if np.any(ok) else None,
                      "max_vec_err": float(np.nanmax(vdiff[ok])) if np.any(ok) else None},
        "plain_fp64": {"value": total / (plain_ms / 1000.0), "unit": UNIT, "ms_per_step": plain_ms,
                       "ms_repeats": plain_times, "warmup": 1,
                       "speedup_seeded_over_plain": value / (total / (plain_ms / 1000.0))},
        "roofline": roof,
        "kernel_rooflines": rooflines,
        "pipe_peaks_tflops": peaks,
        "kernels": {k: {"launches": v[0], "ms": round(v[1], 3)} for k, v in sorted(stats.items(),
                                                                               key=lambda kv: -kv[1][1])},
        "gpu_launches": int(launches_per_step * args.steps),
        "round_ms": stages,
        "variants": variants,
        "spatial_sweep": spatial,
        "eig_phase_share": {k: round(v / max(1, sum(phases.values())), 4) for k, v in phases.items()},
        "autotune_lu_panel": {str(n): {"c64": v["c64"][0], "c128": v["c128"][0]} for n, v in tune.items()},
        "cuda_graph": "device part of each timed pass replayed from a captured CUDA graph",
        "surrogate": sur,
        "single_instance": single,
        "serving": serving,
        "clocks": clk,
        "cpu_baseline": cpu,
    }
    if cpu is not None and args.cpu_sample > 0:
        s = args.cpu_sample
        d = np.abs(eig[:s] - cpu_eig) / np.abs(cpu_eig)
        bad = [int(q) for q in np.nonzero(~(d <= TOL))[0]]
        line["oracle_check"] = {"sample": s, "max_rel_err_vs_cpu_oracle": float(np.nanmax(d)),
                                "within_1e-10": int(np.sum(d <= TOL)),
                                "plain_gpu_vs_cpu_within_1e-10": int(np.sum(np.abs(ref_eig[:s] - cpu_eig)
                                                                           / np.abs(cpu_eig) <= TOL)),
                                "mismatches": [{"index": q, "gpu": [float(eig[q].real), float(eig[q].imag)],
                                                "gpu_plain": [float(ref_eig[q].real), float(ref_eig[q].imag)],
                                                "cpu": [float(cpu_eig[q].real), float(cpu_eig[q].imag)]}
                                               for q in bad[:5]]}
    print(json.dumps(line), flush=True)
    batch.close()
    ctx.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
