"""CPU baseline worker (TEST / MEASUREMENT INFRASTRUCTURE, never the product).

Times the reference's own algorithm for the least-stable mode of one
instance, restated in ``oracle/stab_oracle.py``: assembly, ZGESV(B0, A0) and
ZGEEV('N','V') for the temporal problem (temporal.f90:771-855), or
ZGETRF/ZGETRS and ZGEEV on the companion matrix for the spatial one
(spatial.f90:972-1084), plus the least-stable selection rule of the GPU
path.  Only ``bench.py``'s cpu_baseline leg and its ``--impl reference`` arm
use it, through a spawn-started process pool (one LAPACK thread each).
"""
import math
import os

import numpy as np


def solve_one(d):
    """d: dict of run parameters + 'profile' (nym x 6).  Returns (least
    eigenvalue as (re, im), seconds)."""
    import time

    from oracle import stab_oracle as so
    t0 = time.perf_counter()
    prof = np.asarray(d["profile"])
    p = so.StabParams(mattyp=d["mattyp"], T0=d["T0"], Ma=d["Ma"], Re=d["Re"], Pr=d["Pr"], ny=d["ny"],
                      yi=d["yi"], ymax=d["ymax"], ievec=1, ider=1, top=d.get("top", 0), wall=0,
                      wallt=d.get("wallt", 0), curve=0, itype=d["itype"], alpha=complex(*d["alpha"]),
                      beta=complex(*d["beta"]), omega=complex(*d["omega"]))
    ym = prof[:, 0].copy()
    vt = prof[:, 1:6].copy()
    vt[:, 2] = 0.0
    es = so.solve(p, ym, vt, want_vectors=True)
    j = select_least(es.eig, d)
    t1 = time.perf_counter()
    w = es.eig[j] if j >= 0 else complex("nan")
    return (w.real, w.imag), t1 - t0


def select_least(eig, d):
    """The least-stable selection rule of post.cu (restated)."""
    M = d["Ma"]
    cmax = 10.0 * (1.0 + 1.0 / M)
    a, b, w = complex(*d["alpha"]), complex(*d["beta"]), complex(*d["omega"])
    kabs = max(abs(np.sqrt(a * a + b * b)), 1e-3)
    # spatial spectra: lambda = 1/alpha below 1e-6 max |lambda| is a zero
    # eigenvalue of the companion matrix at rounding level (large alpha of
    # arbitrary phase) and is not a candidate
    eig = np.asarray(eig)
    fin = eig[np.isfinite(eig) & (eig != 0)]
    amax = 1e6 * float(np.min(np.abs(fin))) if fin.size else math.inf
    best, bi = -math.inf, -1
    for q, x in enumerate(eig):
        if not np.isfinite(x):
            continue
        ax = abs(x)
        if d["itype"] == 1:
            if not ax > 1e-12 or ax > cmax * kabs:
                continue
            key = x.imag
        else:
            if ax == 0 or not x.real > 0 or abs(x.imag) > x.real or abs(w / x) > cmax or ax > amax:
                continue
            key = -x.imag
        if key > best:
            best, bi = key, q
    return bi


def pool(processes, threads=1):
    """Spawn-started pool with `threads` BLAS threads per process."""
    import multiprocessing as mp
    for k in ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS", "MKL_NUM_THREADS"):
        os.environ[k] = str(int(threads))
    return mp.get_context("spawn").Pool(processes)
