"""Serving loop over the batched path: Poisson-arriving solve requests,
admitted by free device memory, solved in batches on one GPU, with
throughput and latency percentiles (no counterpart in the reference, which
solves one instance per process run).

Requests are temporal or spatial instances (50/50) with N drawn from
U{32..192} and the other parameters drawn as in the temporal sweep; each
carries its arrival time on a simulated clock that runs with the wall clock
(arrivals are generated up front from the seed).  The server repeatedly
takes every request that has arrived, up to the batch that fits the free
device memory (an estimate of the path's pools per instance, checked against
cudaMemGetInfo), solves it with the coarse-seeded mixed path (plain FP64
fallback inside), and stamps each request's completion.

    python -m stab_gb300.serve --rate 2000 --seconds 2 --seed 20261205 [--workers 2]
"""
from __future__ import annotations

import argparse
import json
import math
import time
from dataclasses import dataclass, field
from typing import Callable, List, Optional

import numpy as np

T0_SUTHERLAND = 110.4 / 0.3815


@dataclass
class Request:
    rid: int
    arrival: float
    itype: int
    ny: int
    M: float
    Re: float
    alpha: float
    beta: float
    omega: float
    done: float = math.nan
    value: complex = complex("nan")
    status: int = -1


def make_requests(rate: float, seconds: float, seed: int) -> List[Request]:
    """Poisson arrivals at `rate` per second over `seconds`."""
    rng = np.random.Generator(np.random.PCG64(seed))
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t > seconds:
            break
        k = len(out)
        itype = 1 if rng.uniform() < 0.5 else 2
        out.append(Request(rid=k, arrival=t, itype=itype, ny=int(rng.integers(32, 193)),
                           M=max(float(rng.uniform(0.0, 2.0)), 1e-3),
                           Re=float(10.0 ** rng.uniform(math.log10(300.0), math.log10(3000.0))),
                           alpha=float(rng.uniform(0.05, 0.4)), beta=float(rng.uniform(0.0, 0.3)),
                           omega=float(rng.uniform(0.02, 0.12))))
    return out


def bytes_per_request(r: Request) -> int:
    """Device pools of one instance on the mixed path: complex64 and
    complex128 n x n factors, the N = 32 coarse matrices, vectors, blocks,
    plus the profile (2000 rows)."""
    n = 5 * r.ny
    m = n if r.itype == 1 else 2 * n
    return int(n * n * (8 + 16) + 2 * (160 if r.itype == 1 else 320) ** 2 * 16 + 12 * m * 16 + 2000 * 6 * 8
               + r.ny * 400)


def admit(queue: List[Request], free_bytes: int, max_batch: int, reserve: float = 0.5) -> int:
    """How many queued requests (in arrival order) fit in `reserve` of the
    free device memory, at most max_batch."""
    budget = reserve * free_bytes
    used, k = 0, 0
    for r in queue[:max_batch]:
        need = bytes_per_request(r)
        if used + need > budget and k > 0:
            break
        used += need
        k += 1
    return k


@dataclass
class ServeStats:
    completed: int = 0
    batches: int = 0
    wall: float = 0.0
    latencies: List[float] = field(default_factory=list)

    def summary(self) -> dict:
        lat = np.asarray(self.latencies)
        return {"completed": self.completed, "batches": self.batches, "wall_s": self.wall,
                "throughput_per_s": self.completed / self.wall if self.wall > 0 else 0.0,
                "p50_ms": float(np.percentile(lat, 50) * 1e3) if len(lat) else None,
                "p99_ms": float(np.percentile(lat, 99) * 1e3) if len(lat) else None,
                "mean_batch": self.completed / max(1, self.batches)}


def serve_concurrent(requests: List[Request], solvers: List[Callable[[List[Request]], None]],
                     free_bytes: Callable[[], int], max_batch: int = 4096,
                     clock: Callable[[], float] = time.perf_counter) -> ServeStats:
    """The loop with one worker thread per solver (each a library context with
    its own stream): a worker takes every request that has arrived, up to its
    share of the free device memory, and solves it while the others take the
    next arrivals, so one batch's latency-bound tail overlaps another's
    throughput-bound start on the GPU.  The library calls release the
    interpreter lock."""
    import threading
    st = ServeStats()
    lock = threading.Lock()
    pending = sorted(requests, key=lambda r: r.arrival)
    state = {"i": 0, "queue": []}
    start = clock()
    share = 0.5 / max(1, len(solvers))
    errors: List[BaseException] = []

    def worker(solve):
        try:
            while True:
                with lock:
                    now = clock() - start
                    while state["i"] < len(pending) and pending[state["i"]].arrival <= now:
                        state["queue"].append(pending[state["i"]])
                        state["i"] += 1
                    q = state["queue"]
                    if not q and state["i"] >= len(pending):
                        return
                    batch = []
                    if q:
                        k = admit(q, free_bytes(), max_batch, reserve=share)
                        batch, state["queue"] = q[:k], q[k:]
                    wait = 0.0 if batch else pending[state["i"]].arrival - now
                if not batch:
                    if wait > 0:
                        time.sleep(min(wait, 0.01))
                    continue
                solve(batch)
                with lock:
                    t = clock() - start
                    for r in batch:
                        r.done = t
                        st.latencies.append(t - r.arrival)
                    st.completed += len(batch)
                    st.batches += 1
        except BaseException as e:   # surfaced in the caller's thread
            errors.append(e)

    threads = [threading.Thread(target=worker, args=(sv,)) for sv in solvers]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    if errors:
        raise errors[0]
    st.wall = clock() - start
    return st


def serve(requests: List[Request], solve: Callable[[List[Request]], None], free_bytes: Callable[[], int],
          max_batch: int = 4096, clock: Callable[[], float] = time.perf_counter) -> ServeStats:
    """Run the loop: the simulated arrival clock starts at the first call of
    `clock`; `solve` fills value/status of a batch in place."""
    st = ServeStats()
    start = clock()
    pending = sorted(requests, key=lambda r: r.arrival)
    i = 0
    queue: List[Request] = []
    while i < len(pending) or queue:
        now = clock() - start
        while i < len(pending) and pending[i].arrival <= now:
            queue.append(pending[i])
            i += 1
        if not queue:
            # idle until the next arrival
            wait = pending[i].arrival - now
            if wait > 0:
                time.sleep(min(wait, 0.01))
            continue
        k = admit(queue, free_bytes(), max_batch)
        batch, queue = queue[:k], queue[k:]
        solve(batch)
        t = clock() - start
        for r in batch:
            r.done = t
            st.latencies.append(t - r.arrival)
        st.completed += len(batch)
        st.batches += 1
    st.wall = clock() - start
    return st


def gpu_solver(ctx, mode: int):
    """A `solve` callable over the library: profiles of the erf family."""
    import stab_gb300 as sg
    from stab_gb300.surrogate import erf_profile
    cache = {}

    def prof(M):
        key = round(M, 6)
        if key not in cache:
            cache[key] = erf_profile(M)
        return cache[key]

    def solve(batch: List[Request]) -> None:
        params = [sg.StabParams.make(itype=r.itype, ny=r.ny, Ma=r.M, Re=r.Re, Pr=0.72, mattyp=1, T0=T0_SUTHERLAND,
                                     yi=1.0 / 23.0, ymax=50.0, alpha=r.alpha if r.itype == 1 else 0.0,
                                     beta=r.beta, omega=r.omega if r.itype == 2 else 0.0) for r in batch]
        eig, err, iters, st, _ = ctx.solve_batch(params, [prof(r.M) for r in batch], mode)
        for r, e, s in zip(batch, eig, st):
            r.value, r.status = complex(e), int(s)

    return solve


def main(argv: Optional[list] = None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--rate", type=float, default=2000.0)
    ap.add_argument("--seconds", type=float, default=2.0)
    ap.add_argument("--seed", type=int, default=20261205)
    ap.add_argument("--max-batch", type=int, default=4096)
    ap.add_argument("--workers", type=int, default=1,
                    help="concurrent batches (one context and stream each); measured on the 2000/s mix: "
                         "1 worker 936/s, 2 workers 773/s, 3 workers 653/s")
    args = ap.parse_args(argv)
    import torch

    import stab_gb300 as sg
    ctxs = [sg.Context(0) for _ in range(max(1, args.workers))]
    reqs = make_requests(args.rate, args.seconds, args.seed)
    solvers = [gpu_solver(c, sg.MODE_COARSE) for c in ctxs]
    # warm each context (derivative tables, pools) on a few requests
    for sv in solvers:
        sv(make_requests(200.0, 0.05, args.seed + 1))
    free = lambda: torch.cuda.mem_get_info()[0]
    st = (serve_concurrent(reqs, solvers, free, args.max_batch) if len(solvers) > 1
          else serve(reqs, solvers[0], free, args.max_batch))
    out = st.summary()
    ok = sum(1 for r in reqs if r.status in (sg.ST_OK, sg.ST_FELLBACK))
    out.update({"requests": len(reqs), "rate_per_s": args.rate, "arrival_window_s": args.seconds,
                "solved_ok_or_fellback": ok, "mix": "50/50 temporal/spatial, N~U{32..192}"})
    print(json.dumps(out))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
