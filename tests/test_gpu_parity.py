"""GPU path against the oracle and the reference's golden files.

Tolerances (stated per check):
  operators     max |GPU - oracle| <= 1e-12 * max |oracle|   (FP64 assembly)
  eigenvalue    |GPU - oracle| / |oracle| <= 1e-10            (least-stable mode)
  eigenvector   max |GPU - oracle| <= 1e-8 after dividing both by their
                first max-modulus entry
  golden files  ndiff -abserr 1e-8 on every number of space.N / time.N
                (thesis/TStest/run.sh:36-39)
"""
import numpy as np
import pytest

import stab_gb300 as sg
from oracle import stab_oracle as so
from tests import helpers as H

pytestmark = pytest.mark.gpu

EIG_REL = 1e-10
VEC_ABS = 1e-8
NDIFF_ABS = 1e-8


def _mat_close(a, b, tol=1e-12):
    scale = max(np.max(np.abs(b)), 1e-300)
    return np.max(np.abs(a - b)) / scale


@pytest.mark.parametrize("wallt", [0, 2])
def test_assemble_temporal_matches_oracle(ctx, wallt):
    d, prof = H.synth_case(1, 24, 0.7, 1500.0, a=0.2, b=0.1)
    d["wallt"] = wallt
    A0, B0 = ctx.assemble(H.stab_params(d), prof)
    p = H.oracle_params(d)
    ms = so.mean_state(p, prof[:, 0], np.where(np.arange(5) == 2, 0.0, prof[:, 1:6]))
    A0o, B0o = so.temporal_pencil(p, ms)
    assert _mat_close(A0, A0o) < 1e-12
    assert _mat_close(B0, B0o) < 1e-12


@pytest.mark.parametrize("top,wallt", [(0, 0), (1, 0), (0, 2)])
def test_assemble_spatial_matches_oracle(ctx, top, wallt):
    d, prof = H.synth_case(2, 20, 0.8, 2000.0, w=0.05, b=0.1, crossflow=True)
    d["top"], d["wallt"] = top, wallt
    mats = ctx.assemble(H.stab_params(d), prof)
    p = H.oracle_params(d)
    ms = so.mean_state(p, prof[:, 0], np.where(np.arange(5) == 2, 0.0, prof[:, 1:6]))
    ref = so.spatial_operators(p, ms)
    for a, b in zip(mats, ref):
        assert _mat_close(a, b) < 1e-12


def test_assemble_constant_viscosity_infinite_map(ctx):
    c = H.cases()["test_spatial_n32"]
    mats = ctx.assemble(H.stab_params(c), H.ts_profile())
    p = H.oracle_params(c)
    prof = H.ts_profile()
    ms = so.mean_state(p, prof[:, 0], np.where(np.arange(5) == 2, 0.0, prof[:, 1:6]))
    for a, b in zip(mats, so.spatial_operators(p, ms)):
        assert _mat_close(a, b) < 1e-12


@pytest.mark.parametrize("name", ["thesis_temporal_n96", "test_spatial_n32"])
def test_full_spectrum_golden_eigenvalue(ctx, name):
    c = H.cases()[name]
    eig, vec, li, st = ctx.full_spectrum(H.stab_params(c), H.ts_profile(), want_vector=False)
    assert st in (sg.ST_OK, sg.ST_NOMODE)
    es = H.oracle_solve(c, H.ts_profile(), want_vectors=False)
    g = complex(*c["golden"])
    j = so.getevec_select(eig, g)
    jo = so.getevec_select(es.eig, g)
    assert abs(eig[j] - es.eig[jo]) / abs(es.eig[jo]) < EIG_REL
    assert abs(eig[j] - g) / abs(g) < 1e-9     # reference platform band ~1e-11
    # sorted ascending by imaginary part (PIKSR2 order)
    assert np.all(np.diff(eig.imag[np.isfinite(eig.imag)]) >= 0)


def test_full_spectrum_set_matches_oracle(ctx):
    d, prof = H.synth_case(1, 32, 0.5, 1000.0, a=0.2)
    eig, vec, li, st = ctx.full_spectrum(H.stab_params(d), prof, want_vector=True)
    es = H.oracle_solve(d, prof)
    assert np.sum(eig == 0) == np.sum(es.eig == 0) == 8
    # every oracle eigenvalue of modest size is reproduced
    for w in es.eig[(np.abs(es.eig) > 0) & (np.abs(es.eig) < 2.0)]:
        assert np.min(np.abs(eig - w)) <= 1e-8 * max(1.0, abs(w))
    # least-stable selection and its eigenvector
    jo = H.select_least(es.eig, d)
    assert li >= 0
    assert abs(eig[li] - es.eig[jo]) / abs(es.eig[jo]) < EIG_REL
    vo = H.phase_normalize(es.evec[:, jo])
    assert np.max(np.abs(H.phase_normalize(vec) - vo)) < VEC_ABS


def test_full_spectrum_spatial_selection(ctx):
    d, prof = H.synth_case(2, 32, 0.8, 2000.0, w=0.05, b=0.1, crossflow=True)
    eig, vec, li, st = ctx.full_spectrum(H.stab_params(d), prof, want_vector=True)
    es = H.oracle_solve(d, prof)
    jo = H.select_least(es.eig, d)
    assert li >= 0 and jo >= 0
    assert abs(eig[li] - es.eig[jo]) / abs(es.eig[jo]) < EIG_REL
    # eigenvector: [lambda phi; phi] with the ZGEEV scaling
    assert abs(np.linalg.norm(vec) - 1.0) < 1e-12
    k = int(np.argmax(np.abs(vec)))
    assert vec[k].imag == 0.0 and vec[k].real > 0
    assert np.max(np.abs(H.phase_normalize(vec) - H.phase_normalize(es.evec[:, jo]))) < VEC_ABS


@pytest.mark.parametrize("name,ref", [("test_spatial_n32", "space1.ref"),
                                      ("thesis_temporal_n96", "thesis_time.ref"),
                                      ("thesis_spatial_n96", "thesis_space.ref")])
def test_polish_reproduces_golden_eigenfunction(ctx, name, ref):
    """getevec -v on the reference's value, then the eigenfunction file."""
    c = H.cases()[name]
    g = complex(*c["golden"])
    p = H.stab_params(c)
    eig, err, iters, status, vecs = ctx.solve_batch([p], [H.ts_profile()], sg.MODE_SEEDED, seeds=[g],
                                                    want_vectors=True)
    assert status[0] == sg.ST_OK, (status, err, iters)
    es = H.oracle_solve(c, H.ts_profile(), want_vectors=False)
    jo = so.getevec_select(es.eig, g)
    assert abs(eig[0] - es.eig[jo]) / abs(es.eig[jo]) < EIG_REL
    ms = so.mean_state(H.oracle_params(c), H.ts_profile()[:, 0],
                       np.where(np.arange(5) == 2, 0.0, H.ts_profile()[:, 1:6]))
    rows = H.eigfunction_rows(vecs[0], c["ny"], ms.y)
    refr = H.ref_rows(ref)
    assert np.max(np.abs(rows[:, 1:] - refr[:, 1:])) < NDIFF_ABS


def test_polish_from_perturbed_seed_temporal(ctx):
    d, prof = H.synth_case(1, 48, 1.2, 800.0, a=0.25, b=0.05)
    es = H.oracle_solve(d, prof)
    jo = H.select_least(es.eig, d)
    w = es.eig[jo]
    seed = w * (1 + 1e-7 * (1 + 1j))
    eig, err, iters, status, vecs = ctx.solve_batch([H.stab_params(d)], [prof], sg.MODE_SEEDED, seeds=[seed],
                                                    want_vectors=True)
    assert status[0] == sg.ST_OK
    assert abs(eig[0] - w) / abs(w) < EIG_REL
    assert np.max(np.abs(H.phase_normalize(vecs[0]) - H.phase_normalize(es.evec[:, jo]))) < VEC_ABS


def _mixed_batch():
    rng = np.random.Generator(np.random.PCG64(7))
    cases = []
    for k in range(6):
        N = int(rng.choice([16, 24, 32]))
        if k % 3 == 2:
            d, prof = H.synth_case(2, N, float(rng.uniform(0.3, 1.5)), float(rng.uniform(500, 2500)),
                                   w=0.05, b=float(rng.uniform(0, 0.2)), crossflow=True)
        else:
            d, prof = H.synth_case(1, N, float(rng.uniform(0.1, 2.0)), float(10 ** rng.uniform(2.5, 3.5)),
                                   a=float(rng.uniform(0.05, 0.4)), b=float(rng.uniform(0, 0.3)))
        cases.append((d, prof))
    return cases


def test_batch_plain_mixed_sizes_and_types(ctx):
    cases = _mixed_batch()
    eig, err, iters, status, vecs = ctx.solve_batch([H.stab_params(d) for d, _ in cases],
                                                    [p for _, p in cases], sg.MODE_PLAIN, want_vectors=True)
    for k, (d, prof) in enumerate(cases):
        es = H.oracle_solve(d, prof)
        jo = H.select_least(es.eig, d)
        assert status[k] == sg.ST_OK
        assert abs(eig[k] - es.eig[jo]) / abs(es.eig[jo]) < EIG_REL, k
        assert np.max(np.abs(H.phase_normalize(vecs[k]) - H.phase_normalize(es.evec[:, jo]))) < VEC_ABS


def test_batch_coarse_seeded_matches_oracle(ctx):
    rng = np.random.Generator(np.random.PCG64(11))
    cases = [H.synth_case(1, int(rng.choice([48, 64])), float(rng.uniform(0.2, 1.5)),
                          float(10 ** rng.uniform(2.5, 3.4)), a=float(rng.uniform(0.05, 0.4)),
                          b=float(rng.uniform(0, 0.3))) for _ in range(4)]
    eig, err, iters, status, vecs = ctx.solve_batch([H.stab_params(d) for d, _ in cases],
                                                    [p for _, p in cases], sg.MODE_COARSE)
    # every instance: the oracle's least-stable mode, with a trusted status
    for k, (d, prof) in enumerate(cases):
        es = H.oracle_solve(d, prof, want_vectors=False)
        w = es.eig[H.select_least(es.eig, d)]
        assert status[k] in (sg.ST_OK, sg.ST_FELLBACK), (k, status[k])
        assert abs(eig[k] - w) / abs(w) < EIG_REL, (k, eig[k], w)


def test_batch_outliving_its_context_is_safe():
    """Destroying the context first orphans live batches instead of leaving
    dangling device state (stab_destroy releases them)."""
    import gc
    c = sg.Context(0)
    d, prof = H.synth_case(1, 16, 0.5, 1000.0, a=0.2)
    b = c.batch([H.stab_params(d)], [prof])
    b.run(sg.MODE_PLAIN)
    c.lib.stab_destroy(c.h)        # bypass Context.close(): the batch is still open
    c.h = None
    with pytest.raises(sg.StabError):
        b.ctx._check(c.lib.stab_batch_run(b.h, sg.MODE_PLAIN) or -5)
    b.close()
    gc.collect()


def test_bad_profile_is_reported_not_solved(ctx):
    d, prof = H.synth_case(1, 16, 0.5, 1000.0, a=0.2)
    bad = prof.copy()
    bad[100, 1] = np.nan
    eig, err, iters, status, _ = ctx.solve_batch([H.stab_params(d), H.stab_params(d)], [prof, bad], sg.MODE_PLAIN)
    assert status[0] == sg.ST_OK
    assert status[1] != sg.ST_OK


def test_coarse_graph_replay_matches_eager(ctx):
    """The second and later STAB_MODE_COARSE passes replay a captured CUDA
    graph of the device sequence; results must equal the eager first pass."""
    rng = np.random.Generator(np.random.PCG64(23))
    cases = [H.synth_case(1, int(rng.choice([24, 32, 48])), float(rng.uniform(0.2, 1.5)),
                          float(10 ** rng.uniform(2.5, 3.4)), a=float(rng.uniform(0.05, 0.4)),
                          b=float(rng.uniform(0, 0.3))) for _ in range(6)]
    b = ctx.batch([H.stab_params(d) for d, _ in cases], [p for _, p in cases])
    outs = []
    for _ in range(3):
        b.run(sg.MODE_COARSE)
        outs.append(b.results())
    for o in outs[1:]:
        assert np.array_equal(o[0], outs[0][0]) and np.array_equal(o[3], outs[0][3])
    b.close()


def test_batch_spectra_equal_single_instance_spectra(ctx):
    cases = [H.synth_case(1, 24, 0.5, 1000.0, a=0.2), H.synth_case(2, 16, 0.8, 2000.0, w=0.05, b=0.1),
             H.synth_case(1, 32, 1.2, 800.0, a=0.3, b=0.1)]
    b = ctx.batch([H.stab_params(d) for d, _ in cases], [p for _, p in cases])
    b.run(sg.MODE_PLAIN)
    spec = b.spectra()
    for (d, prof), s in zip(cases, spec):
        eig, _, _, _ = ctx.full_spectrum(H.stab_params(d), prof, want_vector=False)
        assert np.array_equal(s, eig)
    b.close()


def test_double_word_spectra_match_fp64(ctx):
    """Full spectra at the seed size (N = 32) in double-word arithmetic against
    FP64.  Tolerances: selected least-stable eigenvalue within 1e-9 relative
    (the seeds need that); each of the 8 least-stable eigenvalues within 1e-10
    relative of the nearest double-word one (exact zeros exactly)."""
    rng = np.random.Generator(np.random.PCG64(21))
    cases = [H.synth_case(1, 32, float(rng.uniform(0.05, 2.0)), float(10 ** rng.uniform(2.5, 3.5)),
                          a=float(rng.uniform(0.05, 0.4)), b=float(rng.uniform(0, 0.3))) for _ in range(16)]
    out = {}
    try:
        for prec in (sg.ARITH_FP64, sg.ARITH_DOUBLE_WORD):
            ctx.set_arithmetic(sg.STAGE_PLAIN_EIG, prec)
            b = ctx.batch([H.stab_params(d) for d, _ in cases], [p for _, p in cases])
            b.run(sg.MODE_PLAIN)
            eig, _, _, status, _ = b.results()
            out[prec] = (eig, status, b.spectra())
            b.close()
    finally:
        ctx.reset_arithmetic()
    e64, s64, sp64 = out[sg.ARITH_FP64]
    edw, sdw, spdw = out[sg.ARITH_DOUBLE_WORD]
    assert np.all(s64 == sg.ST_OK) and np.all(sdw == sg.ST_OK)
    assert np.max(np.abs(edw - e64) / np.abs(e64)) < 1e-9
    for a, d in zip(sp64, spdw):
        for r in a[np.argsort(-a.imag)[:8]]:   # exact zeros (isolated rows) must match exactly
            assert np.min(np.abs(d - r)) <= 1e-10 * abs(r)


def test_double_word_retry_lu_matches_fp64(ctx):
    """The complex128 inverse-iteration retry of the coarse-seeded polish with
    its LU in double-word form against the same retry with an FP64 LU.
    Tolerance: every instance converged in both, eigenvalues within 1e-10
    relative (the bench's convergence bar)."""
    rng = np.random.Generator(np.random.PCG64(33))
    cases = [H.synth_case(1, int(rng.choice([48, 64])), float(rng.uniform(0.05, 2.0)),
                          float(10 ** rng.uniform(2.5, 3.5)), a=float(rng.uniform(0.05, 0.4)),
                          b=float(rng.uniform(0, 0.3))) for _ in range(64)]
    out = {}
    try:
        for ar in (sg.ARITH_FP64, sg.ARITH_DOUBLE_WORD):
            ctx.set_arithmetic(sg.STAGE_RETRY_LU, ar)
            b = ctx.batch([H.stab_params(d) for d, _ in cases], [p for _, p in cases])
            b.run(sg.MODE_COARSE)
            eig, _, _, status, _ = b.results()
            out[ar] = (eig, status, b.work()["lu_c128"])
            b.close()
    finally:
        ctx.reset_arithmetic()
    e64, s64, w64 = out[sg.ARITH_FP64]
    edw, sdw, wdw = out[sg.ARITH_DOUBLE_WORD]
    assert wdw > 0, "no instance took the retry"
    both = (s64 == sg.ST_OK) & (sdw == sg.ST_OK)
    assert np.array_equal(s64 == sg.ST_OK, sdw == sg.ST_OK)
    assert np.max(np.abs(edw[both] - e64[both]) / np.abs(e64[both])) < 1e-10


@pytest.mark.parametrize("itype", [1, 2])
def test_external_derivatives_ider0_match_oracle(ctx, itype):
    """ider = 0 (getmean2.f90): the mean derivatives from first/second
    tables instead of the collocation matrices.  Operators within 1e-12 of
    the oracle's largest entry; least-stable eigenvalue within 1e-10 and its
    eigenvector within 1e-8; the same instance with ider = 1 on the same
    profile agrees to 1e-6 (the tables are the profile's exact derivatives)."""
    if itype == 1:
        d, prof = H.synth_case(1, 32, 0.8, 1500.0, a=0.2, b=0.05)
    else:
        d, prof = H.synth_case(2, 32, 0.8, 2000.0, w=0.05, b=0.1, crossflow=True)
    tab = H.derivative_tables(prof, d["Ma"], crossflow=(itype == 2))
    d0 = dict(d, ider=0)
    mats = ctx.assemble(H.stab_params(d0), tab)
    p = H.oracle_params(d0)
    vt = np.where(np.arange(5) == 2, 0.0, prof[:, 1:6])
    ms = so.mean_state(p, prof[:, 0], vt, tab[:, 6:12], tab[:, 12:18])
    ref = so.temporal_pencil(p, ms) if itype == 1 else so.spatial_operators(p, ms)
    for a, b in zip(mats, ref):
        assert _mat_close(a, b) < 1e-12
    eig, vec, li, st = ctx.full_spectrum(H.stab_params(d0), tab, want_vector=True)
    es = H.oracle_solve(d0, tab)
    jo = H.select_least(es.eig, d0)
    assert st == sg.ST_OK and li >= 0 and jo >= 0
    assert abs(eig[li] - es.eig[jo]) / abs(es.eig[jo]) < EIG_REL
    assert np.max(np.abs(H.phase_normalize(vec) - H.phase_normalize(es.evec[:, jo]))) < VEC_ABS
    e1, _, l1, _ = ctx.full_spectrum(H.stab_params(d), prof, want_vector=False)
    assert abs(e1[l1] - eig[li]) / abs(eig[li]) < 1e-6


def test_assemble_curved_wall_matches_oracle(ctx):
    """curve = 2 (the circle of circh.f90, radius x): C0, C1, C2 within
    1e-12 of the oracle's largest entry, on the CFtest case at N = 24 and
    with a small radius where the metric departs far from 1."""
    for name, x in (("cftest_spatial_n64", 500.0), ("fsctest_spatial_n64", 2.0)):
        c = dict(H.cases()[name], ny=24, x=x)
        prof = H.case_profile(c)
        mats = ctx.assemble(H.stab_params(c), prof)
        p = H.oracle_params(c)
        ms = so.mean_state(p, prof[:, 0], np.where(np.arange(5) == 2, 0.0, prof[:, 1:6]))
        for a, b in zip(mats, so.spatial_operators(p, ms)):
            assert _mat_close(a, b) < 1e-12


@pytest.mark.parametrize("name", ["cftest_spatial_n64", "cftest_spatial_n96", "fsctest_spatial_n64"])
def test_curved_wall_golden_eigenvalues(ctx, name):
    """The curved-wall golden cases (CFtest, FSCtest; curve = 2): the polish
    from the reference's eigenvalue lands on it within 1e-9 relative (the
    reference platforms' band) and on the oracle's within 1e-10."""
    c = H.cases()[name]
    prof = H.case_profile(c)
    g = complex(*c["golden"])
    eig, err, iters, status, vecs = ctx.solve_batch([H.stab_params(c)], [prof], sg.MODE_SEEDED, seeds=[g],
                                                    want_vectors=True)
    assert status[0] == sg.ST_OK, (status, err, iters)
    es = H.oracle_solve(c, prof, want_vectors=False)
    jo = so.getevec_select(es.eig, g)
    assert abs(eig[0] - es.eig[jo]) / abs(es.eig[jo]) < EIG_REL
    assert abs(eig[0] - g) / abs(g) < 1e-9
    if "eigfunction_rows" in c:
        # space.ref rows (wall first or free stream first), matched by y
        ny = c["ny"]
        ref = np.loadtxt(H.GOLDEN + "/" + c["eigfunction_rows"], comments="#")
        rows = H.eigfunction_rows(vecs[0], ny, es.ms.y)
        order = [int(np.argmin(np.abs(rows[:, 0] - yr))) for yr in ref[:, 0]]
        assert len(set(order)) == ny
        got = rows[order][:, 1::2] + 1j * rows[order][:, 2::2]
        want = ref[:, 1::2] + 1j * ref[:, 2::2]
        kg = np.unravel_index(np.argmax(np.abs(got)), got.shape)
        kw = np.unravel_index(np.argmax(np.abs(want)), want.shape)
        assert kg == kw
        assert np.max(np.abs(got / got[kg] - want / want[kw])) < NDIFF_ABS


def test_curved_wall_full_spectrum_fsctest(ctx):
    """FSCtest at N = 64 (companion order 640, curve = 2): the full FP64
    spectrum holds the reference's eigenvalue within 1e-9 and the oracle's
    within 1e-10."""
    c = H.cases()["fsctest_spatial_n64"]
    prof = H.case_profile(c)
    eig, vec, li, st = ctx.full_spectrum(H.stab_params(c), prof, want_vector=False)
    g = complex(*c["golden"])
    j = so.getevec_select(eig, g)
    es = H.oracle_solve(c, prof, want_vectors=False)
    jo = so.getevec_select(es.eig, g)
    assert abs(eig[j] - es.eig[jo]) / abs(es.eig[jo]) < EIG_REL
    assert abs(eig[j] - g) / abs(g) < 1e-9


def test_curve1_parabola_matches_oracle(ctx):
    """curve = 1 (calch.f90, the parabolic cylinder y = sqrt(2x) at arc
    length x from its nose): operators within 1e-12 of the oracle's largest
    entry and the least-stable eigenvalue within 1e-10, eigenvector within
    1e-8, near the nose (x = 2, strong curvature) and downstream (x = 50).
    Unpinned by the reference: its tests hold no curve = 1 case."""
    for x in (2.0, 50.0):
        c, prof = H.synth_case(2, 32, 0.8, 2000.0, w=0.05, b=0.1, crossflow=True)
        c.update(curve=1, x=x)
        mats = ctx.assemble(H.stab_params(c), prof)
        p = H.oracle_params(c)
        ms = so.mean_state(p, prof[:, 0], np.where(np.arange(5) == 2, 0.0, prof[:, 1:6]))
        for a, b in zip(mats, so.spatial_operators(p, ms)):
            assert _mat_close(a, b) < 1e-12
        eig, vec, li, st = ctx.full_spectrum(H.stab_params(c), prof, want_vector=True)
        es = H.oracle_solve(c, prof)
        jo = H.select_least(es.eig, c)
        assert st == sg.ST_OK and li >= 0 and jo >= 0
        assert abs(eig[li] - es.eig[jo]) / abs(es.eig[jo]) < EIG_REL
        assert np.max(np.abs(H.phase_normalize(vec) - H.phase_normalize(es.evec[:, jo]))) < VEC_ABS


def test_bad_curves_are_rejected(ctx):
    """curve values outside 0..2, and curve = 1 where false position finds
    no wall point in 30 steps (x = 0.5) or x <= 0, are refused with
    STAB_ERR_ARG before any device work; the context stays usable."""
    c = dict(H.cases()["cftest_spatial_n64"], ny=16)
    prof = H.case_profile(c)
    for curve, x in ((3, 500.0), (1, 0.5), (1, 0.0), (1, -2.0)):
        with pytest.raises(sg.StabError):
            ctx.full_spectrum(H.stab_params(dict(c, curve=curve, x=x)), prof, want_vector=False)
    eig, _, _, st = ctx.full_spectrum(H.stab_params(c), prof, want_vector=False)
    assert eig.size == 160


@pytest.mark.parametrize("option,value,default", [(sg.OPT_EIG_THREADS, 64, 128), (sg.OPT_EIG_MID, 0, 1)])
def test_eigensolver_cta_sizes_agree(ctx, option, value, default):
    """STAB_OPT_EIG_THREADS = 64 (eight 64-thread CTAs per SM) and
    STAB_OPT_EIG_MID (on by default: one 256-thread CTA per instance for
    batches of at most two per SM; 180 instances here) against the
    128-thread persistent grid: the same spectra to rounding, FP64 and
    double-word, and the same coarse-seeded results."""
    cases = [H.synth_case(1, N, 0.5 + 0.1 * k, 1000.0 + 100 * k, a=0.2)[0] for k, N in enumerate((24, 32, 40))]
    profs = [H.synth_case(1, c["ny"], c["Ma"], c["Re"], a=0.2)[1] for c in cases]
    sp = [H.stab_params(c) for c in cases] * 60          # enough instances for the persistent batch grid
    pr = profs * 60
    out = {}
    try:
        for t in (default, value):
            ctx.set_option(option, t)
            b = ctx.batch(sp, pr)
            b.run(sg.MODE_PLAIN)
            spec = b.spectra()
            w, err, it, st, _ = b.results()
            b.run(sg.MODE_COARSE)
            wc, _, _, stc, _ = b.results()
            b.close()
            out[t] = (spec, w, st, wc, stc)
    finally:
        ctx.set_option(option, default)
    s128, w128, st128, wc128, stc128 = out[default]
    s64, w64, st64, wc64, stc64 = out[value]
    assert np.array_equal(st128, st64) and np.array_equal(stc128, stc64)
    assert np.max(np.abs(w64 - w128) / np.abs(w128)) < 1e-12
    assert np.max(np.abs(wc64 - wc128) / np.abs(wc128)) < 1e-12
    for a, b in zip(s128[:3], s64[:3]):
        for w in a[(np.abs(a) > 0) & (np.abs(a) < 2.0)]:
            assert np.min(np.abs(b - w)) <= 1e-10 * max(1.0, abs(w)), w


def test_coarse_with_seed_vectors_matches_plain(ctx):
    """STAB_OPT_SEED_VECTORS: the top candidate's polish starts from the
    N = 32 eigenvector interpolated to the full grid.  On 256 instances of
    the benchmark sweep the trusted results that differ from the plain FP64
    path's least-stable eigenvalue (two of them without the option: modes
    the seed spectra misplace) are no more than without it, and at most 2 %
    carry a flag."""
    import bench
    params, prof = bench.workload(256, 20261203)
    sp = [bench.to_stab(d) for d in params]
    b = ctx.batch(sp, [prof[k] for k in range(256)])
    try:
        b.run(sg.MODE_PLAIN)
        ref, _, _, ref_st, _ = b.results()
        out = {}
        for on in (0, 1):
            ctx.set_option(sg.OPT_SEED_VECTORS, on)
            b.run(sg.MODE_COARSE)
            w, err, it, st, _ = b.results()
            out[on] = (w, st)
    finally:
        ctx.set_option(sg.OPT_SEED_VECTORS, 1)
        b.close()
    wrong = {}
    for on in (0, 1):
        w, st = out[on]
        trusted = np.isin(st, [sg.ST_OK, sg.ST_FELLBACK]) & (ref_st == sg.ST_OK)
        rel = np.abs(w - ref) / np.abs(ref)
        wrong[on] = set(np.nonzero(trusted & ~(rel <= 1e-10))[0].tolist())
        assert np.sum(~np.isin(st, [sg.ST_OK, sg.ST_FELLBACK])) <= 0.02 * 256, np.unique(st, return_counts=True)
    assert len(wrong[0]) <= 3 and wrong[1] <= wrong[0], wrong


def test_parallel_candidates_match_sequential_rounds(ctx):
    """STAB_OPT_PARALLEL_CANDIDATES: the second candidate level (N = 48 for
    these temporal instances) polishes its four shift
    candidates side by side (one sub-batch copy per candidate) instead of in
    four rounds.  On 256 instances of the benchmark sweep (about 16 of them
    reach that level) both forms return the same statuses and eigenvalues
    within 1e-13 relative, and the eigenvectors within 1e-10."""
    import bench
    params, prof = bench.workload(256, 20261203)
    sp = [bench.to_stab(d) for d in params]
    b = ctx.batch(sp, [prof[k] for k in range(256)])
    out = {}
    try:
        for on in (0, 1):
            ctx.set_option(sg.OPT_PARALLEL_CANDIDATES, on)
            b.run(sg.MODE_COARSE)
            out[on] = b.results(want_vectors=True)
            counts = b.counts()
    finally:
        ctx.set_option(sg.OPT_PARALLEL_CANDIDATES, 1)
        b.close()
    w0, _, _, st0, v0 = out[0]
    w1, _, _, st1, v1 = out[1]
    assert counts["fp64_fallback"] >= 4, counts    # the level ran on several instances
    assert np.array_equal(st0, st1), (np.unique(st0, return_counts=True), np.unique(st1, return_counts=True))
    fin = np.isfinite(w0)
    assert np.array_equal(fin, np.isfinite(w1))
    assert np.max(np.abs(w1[fin] - w0[fin]) / np.abs(w0[fin])) <= 1e-13
    for k in np.nonzero(fin)[0]:
        a, r = np.asarray(v1[k]), np.asarray(v0[k])
        pa, pr = int(np.argmax(np.abs(a))), int(np.argmax(np.abs(r)))
        assert np.max(np.abs(a / a[pa] - r / r[pr])) <= 1e-10, k


def test_two_contexts_in_two_threads_match_one(ctx):
    """Two contexts (each with its own stream) solving from two host threads at
    the same time, as the serving loop's workers do, return what one context
    returns for the same batches: the library keeps no shared mutable state
    between contexts."""
    import threading
    import bench
    params, prof = bench.workload(96, 20261203)
    sp = [bench.to_stab(d) for d in params]
    halves = [(sp[:48], [prof[k] for k in range(48)]), (sp[48:], [prof[k] for k in range(48, 96)])]
    ref = [ctx.solve_batch(p, pr, sg.MODE_COARSE)[::3] for p, pr in halves]
    ctxs = [sg.Context(0), sg.Context(0)]
    out = [None, None]
    errs = []

    def run(i):
        try:
            for _ in range(2):
                out[i] = ctxs[i].solve_batch(halves[i][0], halves[i][1], sg.MODE_COARSE)[::3]
        except BaseException as e:
            errs.append(e)
    th = [threading.Thread(target=run, args=(i,)) for i in range(2)]
    try:
        for t in th:
            t.start()
        for t in th:
            t.join()
    finally:
        for c in ctxs:
            c.close()
    assert not errs, errs
    for i in range(2):
        (w0, st0), (w1, st1) = ref[i], out[i]
        assert np.array_equal(st0, st1)
        fin = np.isfinite(w0)
        assert np.array_equal(fin, np.isfinite(w1))
        assert np.max(np.abs(w1[fin] - w0[fin]) / np.abs(w0[fin])) <= 1e-13
