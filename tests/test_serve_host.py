"""The serving loop's host logic with a fake solver (no GPU): Poisson
arrivals, admission by free memory, completion stamps and percentiles."""
import numpy as np

from stab_gb300 import serve as sv


def test_poisson_arrivals():
    reqs = sv.make_requests(2000.0, 1.0, 5)
    assert 1800 < len(reqs) < 2200
    t = np.array([r.arrival for r in reqs])
    assert np.all(np.diff(t) > 0) and t[-1] <= 1.0
    gaps = np.diff(t)
    assert abs(gaps.mean() - 1 / 2000) < 1e-4
    assert {r.itype for r in reqs} == {1, 2} and min(r.ny for r in reqs) >= 32 and max(r.ny for r in reqs) <= 192


def test_admission_respects_memory():
    reqs = sv.make_requests(2000.0, 0.5, 6)
    per = [sv.bytes_per_request(r) for r in reqs]
    k = sv.admit(reqs, free_bytes=int(2 * sum(per[:10])), max_batch=4096, reserve=0.5)
    assert k == 10 or sum(per[:k]) <= sum(per[:10])
    assert sv.admit(reqs, free_bytes=1, max_batch=4096) == 1          # always makes progress
    assert sv.admit(reqs, free_bytes=10 ** 15, max_batch=7) == 7


def test_serve_loop_with_fake_solver():
    reqs = sv.make_requests(1000.0, 0.2, 7)
    now = [0.0]

    def clock():
        return now[0]

    def solve(batch):
        now[0] += 0.01 + 1e-5 * len(batch)      # a batch costs 10 ms + 10 us per request
        for r in batch:
            r.status = 0

    def sleep_free():
        return 10 ** 12

    # the fake clock only advances in solve(): advance it while idle too
    orig = sv.time.sleep
    sv.time.sleep = lambda s: now.__setitem__(0, now[0] + s)
    try:
        st = sv.serve(reqs, solve, sleep_free, max_batch=64, clock=clock)
    finally:
        sv.time.sleep = orig
    s = st.summary()
    assert s["completed"] == len(reqs) and all(r.status == 0 for r in reqs)
    assert all(r.done >= r.arrival for r in reqs)
    assert s["p50_ms"] <= s["p99_ms"] and s["batches"] >= len(reqs) / 64


def test_concurrent_workers_overlap_batches():
    """serve_concurrent: two workers (fake solvers that sleep, as a library
    call that releases the interpreter lock does) take batches while the
    other solves; every request completes once, after its arrival, and the
    two solvers run at the same time."""
    import threading
    import time

    reqs = sv.make_requests(2000.0, 0.15, 8)
    active = [0]
    peak = [0]
    lock = threading.Lock()

    def make_solver():
        def solve(batch):
            with lock:
                active[0] += 1
                peak[0] = max(peak[0], active[0])
            time.sleep(0.01 + 2e-5 * len(batch))
            for r in batch:
                assert r.status == -1          # solved once
                r.status = 0
            with lock:
                active[0] -= 1
        return solve

    st = sv.serve_concurrent(reqs, [make_solver(), make_solver()], lambda: 10 ** 12, max_batch=4096)
    s = st.summary()
    assert s["completed"] == len(reqs) and all(r.status == 0 for r in reqs)
    assert all(r.done >= r.arrival for r in reqs)
    assert peak[0] == 2 and s["batches"] >= 4
