"""The benchmark configurations against the CPU oracle on the same inputs.

  config 0  temporal, N = 64 (n = 320), Streett map ymax = 50 with half the
            points below y = 2 (Yi = 1/23), U = erf(y/2), Crocco-Busemann T,
            Sutherland (S/T_inf = 0.3815), M = 0.5, Re = 1000, alpha = 0.2:
            full spectrum and the least-stable eigenvector;
  config 1  spatial, N = 96 (companion order m = 960), crossflow
            W = 0.08 y exp(1 - y/1.5)/1.5, M = 0.8, Re = 2000, omega = 0.05,
            beta = 0.1: full spectrum, then the polish of the least-stable
            alpha;
  config 2  128 instances of the batched temporal sweep (N in
            {48, 64, 96, 128}, PCG64(20261203)) through STAB_MODE_COARSE.

Tolerances: least-stable eigenvalue within 1e-10 relative of the oracle's;
eigenvectors within 1e-8 after dividing both by their first max-modulus
entry; every oracle eigenvalue with |value| < 2 matched within
1e-8 * max(1, |value|).  In config 2 every instance the library reports as
STAB_ST_OK or STAB_ST_FELLBACK must match the oracle within 1e-10; any other
status is a flag the caller sees, and at most 2 % may carry one.
"""
import numpy as np
import pytest

import stab_gb300 as sg
from oracle import stab_oracle as so
from tests import helpers as H

pytestmark = pytest.mark.gpu

EIG_REL = 1e-10
VEC_ABS = 1e-8


def _spectrum_matches(eig, ref, bound=2.0, tol=1e-8):
    for w in ref[(np.abs(ref) > 0) & (np.abs(ref) < bound)]:
        assert np.min(np.abs(eig - w)) <= tol * max(1.0, abs(w)), w


def test_config0_temporal_n64_full_spectrum_and_vector(ctx):
    d, prof = H.synth_case(1, 64, 0.5, 1000.0, a=0.2, ymax=50.0, yi=1.0 / 23.0)
    eig, vec, li, st = ctx.full_spectrum(H.stab_params(d), prof, want_vector=True)
    assert st == sg.ST_OK and li >= 0
    assert eig.size == 320
    es = H.oracle_solve(d, prof)
    assert np.sum(eig == 0) == np.sum(es.eig == 0)
    _spectrum_matches(eig, es.eig)
    jo = H.select_least(es.eig, d)
    assert abs(eig[li] - es.eig[jo]) / abs(es.eig[jo]) < EIG_REL
    assert np.max(np.abs(H.phase_normalize(vec) - H.phase_normalize(es.evec[:, jo]))) < VEC_ABS
    # the same instance through the batched plain path and the coarse-seeded path
    for mode in (sg.MODE_PLAIN, sg.MODE_COARSE):
        w, err, iters, status, vecs = ctx.solve_batch([H.stab_params(d)], [prof], mode, want_vectors=True)
        assert status[0] in (sg.ST_OK, sg.ST_FELLBACK)
        assert abs(w[0] - es.eig[jo]) / abs(es.eig[jo]) < EIG_REL
        assert np.max(np.abs(H.phase_normalize(vecs[0]) - H.phase_normalize(es.evec[:, jo]))) < VEC_ABS


def test_config1_spatial_n96_crossflow(ctx):
    d, prof = H.synth_case(2, 96, 0.8, 2000.0, w=0.05, b=0.1, crossflow=True, ymax=50.0, yi=1.0 / 23.0)
    eig, vec, li, st = ctx.full_spectrum(H.stab_params(d), prof, want_vector=True)
    assert st == sg.ST_OK and li >= 0
    assert eig.size == 960
    es = H.oracle_solve(d, prof)
    _spectrum_matches(eig, es.eig, bound=1.0)
    jo = H.select_least(es.eig, d)
    assert jo >= 0
    assert abs(eig[li] - es.eig[jo]) / abs(es.eig[jo]) < EIG_REL
    vo = H.phase_normalize(es.evec[:, jo])
    assert np.max(np.abs(H.phase_normalize(vec) - vo)) < VEC_ABS
    # polish of the least-stable alpha from the full spectrum's value
    w, err, iters, status, vecs = ctx.solve_batch([H.stab_params(d)], [prof], sg.MODE_SEEDED, seeds=[eig[li]],
                                                  want_vectors=True)
    assert status[0] == sg.ST_OK
    assert abs(w[0] - es.eig[jo]) / abs(es.eig[jo]) < EIG_REL
    assert np.max(np.abs(H.phase_normalize(vecs[0]) - vo)) < VEC_ABS


def test_config2_sweep_128_coarse_never_wrong_when_ok(ctx):
    import bench
    from oracle import baseline
    params, prof = bench.workload(128, 20261203)
    jobs = []
    for k, dd in enumerate(params):
        j = dict(dd)
        j["profile"] = prof[k]
        jobs.append(j)
    pool = baseline.pool(16)
    try:
        out = pool.map(baseline.solve_one, jobs, chunksize=1)
    finally:
        pool.close()
        pool.join()
    ref = np.array([complex(*o[0]) for o in out])
    sp = [bench.to_stab(dd) for dd in params]
    w, err, iters, status, vecs = ctx.solve_batch(sp, [prof[k] for k in range(128)], sg.MODE_COARSE)
    rel = np.abs(w - ref) / np.abs(ref)
    trusted = np.isin(status, [sg.ST_OK, sg.ST_FELLBACK])
    bad = np.nonzero(trusted & ~(rel <= EIG_REL))[0]
    assert bad.size == 0, [(int(k), w[k], ref[k], int(status[k])) for k in bad[:5]]
    assert np.sum(~trusted) <= 2, np.unique(status, return_counts=True)


def test_spatial_crossflow_batch_coarse_trusts_level_agreement(ctx):
    """Batched spatial crossflow instances around configuration 1 (N in
    {64, 96}, companion orders 640 and 960) through STAB_MODE_COARSE.  Their
    least-stable alpha converges algebraically with N (about 1e-3 relative at
    N = 24, 1e-5 at N = 32), so the seed levels' own 1e-7 quick accept rarely
    certifies it; with STAB_OPT_LEVEL_CONSISTENCY (default) the agreement of
    the N = 32 level with the spatial second level (N = 24 by default)
    does.  Every trusted result matches the plain FP64
    path within 1e-10 (the plain path is checked against the oracle by the
    configuration-1 test), at most 10 % carry a flag, and without the option
    the same batch trusts fewer instances."""
    import bench
    params, prof = bench.spatial_workload(24, 20261206)
    sp = [bench.to_stab(d) for d in params]
    b = ctx.batch(sp, [prof[k] for k in range(24)])
    try:
        b.run(sg.MODE_PLAIN)
        ref, _, _, ref_st, _ = b.results()
        b.run(sg.MODE_COARSE)
        w, _, _, st, _ = b.results()
        ctx.set_option(sg.OPT_LEVEL_CONSISTENCY, 0)
        b.run(sg.MODE_COARSE)
        w0, _, _, st0, _ = b.results()
    finally:
        ctx.set_option(sg.OPT_LEVEL_CONSISTENCY, 1)
        b.close()
    assert np.all(ref_st == sg.ST_OK)
    rel = np.abs(w - ref) / np.abs(ref)
    trusted = np.isin(st, [sg.ST_OK, sg.ST_FELLBACK])
    bad = np.nonzero(trusted & ~(rel <= EIG_REL))[0]
    assert bad.size == 0, [(int(k), w[k], ref[k], int(st[k])) for k in bad]
    assert np.sum(~trusted) <= 0.1 * 24, np.unique(st, return_counts=True)
    trusted0 = np.isin(st0, [sg.ST_OK, sg.ST_FELLBACK])
    assert np.sum(trusted0) < np.sum(trusted), (np.unique(st0, return_counts=True), np.unique(st, return_counts=True))
    assert np.all(np.abs(w0 - ref)[trusted0] <= EIG_REL * np.abs(ref)[trusted0])
