"""The finite-difference temporal solver (input itype 3, fd_temporal.f90) on
the GPU against the oracle's restatement on the same inputs.

The case is the reference's thesis TStest FD input (M = 0.3, Re = 1000,
Pr = 1, alpha = 0.30862069, Yi = 1, Ymax = 50, constant viscosity) at
reduced N, and a Sutherland / Crocco-Busemann synthetic profile.
Tolerances: operators within 1e-12 of the oracle's largest entry; the
least-stable and the TS eigenvalue within 1e-10 relative; eigenvectors
within 1e-8 after dividing by the first max-modulus entry; the eigenfunction
file within the reference's ndiff -abserr 1e-8.
"""
import os
import subprocess

import numpy as np
import pytest

import stab_gb300 as sg
from oracle import stab_oracle as so
from tests import helpers as H

pytestmark = pytest.mark.gpu
EIG_REL = 1e-10
VEC_ABS = 1e-8
BIN = os.path.join(os.path.dirname(sg.__file__), "bin")
TS_GUESS = 0.1146620194 + 0.0023517213j      # the TS mode with this solver's adiabatic wall


def _ts_case(N, **kw):
    d = dict(mattyp=0, T0=0.0, Ma=0.3, Re=1000.0, Pr=1.0, ny=N, yi=1.0, ymax=50.0, ievec=1, ider=1, top=0,
             wall=0, wallt=0, curve=0, itype=3, alpha=[0.30862069, 0.0], beta=[0.0, 0.0], omega=[0.0, 0.0])
    d.update(kw)
    return d


def _synth(N):
    d, prof = H.synth_case(1, N, 0.8, 1500.0, a=0.2, b=0.05, ymax=50.0, yi=2.0)
    d["itype"] = 3
    return d, prof


def _mat_close(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def _oracle_pencil(d, prof):
    p = H.oracle_params(d)
    vt = prof[:, 1:6].copy()
    vt[:, 2] = 0.0
    return so.fd_temporal_pencil(p, so.fd_mean_state(p, prof[:, 0], vt))


@pytest.mark.parametrize("which", ["ts", "synthetic"])
def test_fd_assemble_matches_oracle(ctx, which):
    d, prof = (_ts_case(40), H.ts_profile()) if which == "ts" else _synth(32)
    A0, B0 = ctx.assemble(H.stab_params(d), prof)
    A0o, B0o = _oracle_pencil(d, prof)
    assert _mat_close(A0, A0o) < 1e-12
    assert _mat_close(B0, B0o) < 1e-12


@pytest.mark.parametrize("which", ["ts", "synthetic"])
def test_fd_full_spectrum_matches_oracle(ctx, which):
    d, prof = (_ts_case(96), H.ts_profile()) if which == "ts" else _synth(64)
    eig, vec, li, st = ctx.full_spectrum(H.stab_params(d), prof, want_vector=True)
    es = H.oracle_solve(d, prof)
    assert eig.size == 5 * d["ny"]
    assert np.sum(eig == 0) == np.sum(es.eig == 0)
    jo = H.select_least(es.eig, d)
    assert st == sg.ST_OK and li >= 0 and jo >= 0
    assert abs(eig[li] - es.eig[jo]) / abs(es.eig[jo]) < EIG_REL
    assert np.max(np.abs(H.phase_normalize(vec) - H.phase_normalize(es.evec[:, jo]))) < VEC_ABS
    for w in es.eig[(np.abs(es.eig) > 0) & (np.abs(es.eig) < 2.0)]:
        assert np.min(np.abs(eig - w)) <= 1e-8 * max(1.0, abs(w))
    if which == "ts":
        j, jo = so.getevec_select(eig, TS_GUESS), so.getevec_select(es.eig, TS_GUESS)
        assert abs(eig[j] - es.eig[jo]) / abs(es.eig[jo]) < EIG_REL
        assert abs(es.eig[jo] - TS_GUESS) / abs(TS_GUESS) < 1e-5     # the N = 96 discretisation error


def test_fd_polish_and_coarse_modes(ctx):
    d = _ts_case(128)
    prof = H.ts_profile()
    es = H.oracle_solve(d, prof)
    jo = so.getevec_select(es.eig, TS_GUESS)
    w0 = es.eig[jo]
    p = H.stab_params(d)
    for mode in (sg.MODE_SEEDED, sg.MODE_TRACK):
        w, err, iters, status, vecs = ctx.solve_batch([p], [prof], mode, seeds=[w0 * (1 + 1e-7)],
                                                      want_vectors=True)
        assert status[0] == sg.ST_OK, (status, err, iters)
        assert abs(w[0] - w0) / abs(w0) < EIG_REL
        assert np.max(np.abs(H.phase_normalize(vecs[0]) - H.phase_normalize(es.evec[:, jo]))) < VEC_ABS
    # the coarse path on finite-difference instances takes its seeds from the
    # same solver at N = 32; trusted results equal the oracle's least-stable
    cases = [_synth(N) for N in (48, 64)] + [(_ts_case(80), prof)]
    w, err, iters, status, _ = ctx.solve_batch([H.stab_params(c) for c, _ in cases], [q for _, q in cases],
                                               sg.MODE_COARSE)
    for k, (c, q) in enumerate(cases):
        e = H.oracle_solve(c, q, want_vectors=False)
        j = H.select_least(e.eig, c)
        if status[k] in (sg.ST_OK, sg.ST_FELLBACK):
            assert abs(w[k] - e.eig[j]) / abs(e.eig[j]) < EIG_REL, (k, w[k], e.eig[j], status[k])
        else:
            assert status[k] in (sg.ST_UNVERIFIED, sg.ST_NOMODE), status[k]


def test_fd_cli_writes_evec_and_eigenfunction(tmp_path):
    """stab_gpu < input with itype 3 (the reference's FD input protocol),
    then getevec_gpu -v at the TS mode: evec.dat records itype 1 and the
    ogengrid grid (fd_temporal.f90:1050-1056), and time.1 equals the
    oracle's eigenfunction text within 1e-8."""
    N = 64
    with open(tmp_path / "profile.0", "w") as fh:
        for r in H.ts_profile():
            fh.write(" ".join(repr(float(v)) for v in r) + "\n")
    text = "0\n0.3 1000 1\n%d 1.0 50.0\n1\n1\n0 0 0 0\n3\n0.30862069, 0\n0 0\n0\n" % N
    r = subprocess.run([os.path.join(BIN, "stab_gpu")], cwd=tmp_path, input=text, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    h, y, eig, vec = sg.read_evec(str(tmp_path / "evec.dat"))
    assert h.itype == 1 and h.ny == N
    yo = sg.fd_grid(N, 1.0, 50.0)[0]
    assert np.array_equal(y, yo)
    es = H.oracle_solve(_ts_case(N), H.ts_profile())
    jo = so.getevec_select(es.eig, TS_GUESS)
    g = complex(es.eig[jo])
    r = subprocess.run([os.path.join(BIN, "getevec_gpu"), "-v"], cwd=tmp_path, capture_output=True, text=True,
                       input=f"evec.dat\n{g.real!r} {g.imag!r}\n0 0\n", timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    got = [ln.split() for ln in open(tmp_path / "time.1").read().splitlines() if ln.strip() and not ln.startswith("#")]
    want = [ln.split() for ln in so.eigfunction_text(es, jo).splitlines() if ln.strip() and not ln.startswith("#")]
    assert len(got) == len(want) == N
    assert max(abs(float(a) - float(b)) for u, v in zip(got, want) for a, b in zip(u, v)) <= 1e-8


def _ts_spatial(N, **kw):
    d = _ts_case(N, itype=4, alpha=[0.0, 0.0], omega=[0.08, 0.0])
    d.update(kw)
    return d


@pytest.mark.parametrize("kw", [dict(), dict(top=1), dict(wallt=2), dict(wallt=2, top=1), dict(curve=1, x=5.0),
                                dict(curve=2, x=500.0)])
def test_fd_spatial_assemble_matches_oracle(ctx, kw):
    """C0, C1, C2 of fd_spatial.f90 for both free-stream conditions, both
    wall temperature conditions (with the wall energy row's G from another
    node, as the reference writes it), calch's curvature, and curve = 2,
    which this solver treats as a flat wall."""
    d = _ts_spatial(24, **kw)
    prof = H.ts_profile()
    mats = ctx.assemble(H.stab_params(d), prof)
    p = H.oracle_params(d)
    vt = prof[:, 1:6].copy()
    vt[:, 2] = 0.0
    ms = so.fd_mean_state(p, prof[:, 0], vt)
    for a, b in zip(mats, so.fd_spatial_operators(p, ms)):
        assert _mat_close(a, b) < 1e-12


@pytest.mark.parametrize("kw", [dict(), dict(wallt=2, top=1)])
def test_fd_spatial_full_spectrum_and_polish(ctx, kw):
    d = _ts_spatial(64, **kw)
    prof = H.ts_profile()
    eig, vec, li, st = ctx.full_spectrum(H.stab_params(d), prof, want_vector=True)
    es = H.oracle_solve(d, prof)
    assert eig.size == 10 * d["ny"]
    g = 2.2804739411185E-001 - 6.5163146952733E-003j
    j, jo = so.getevec_select(eig, g), so.getevec_select(es.eig, g)
    assert abs(eig[j] - es.eig[jo]) / abs(es.eig[jo]) < EIG_REL
    # the companion's zero eigenvalues come out at rounding level (alpha ~
    # 1e14, arbitrary phase); the selection rule leaves them out
    lo = H.select_least(es.eig, d)
    assert li >= 0 and lo >= 0
    assert abs(eig[li] - es.eig[lo]) / abs(es.eig[lo]) < EIG_REL
    assert np.max(np.abs(H.phase_normalize(vec) - H.phase_normalize(es.evec[:, lo]))) < VEC_ABS
    w, err, iters, status, vecs = ctx.solve_batch([H.stab_params(d)], [prof], sg.MODE_SEEDED,
                                                  seeds=[es.eig[jo] * (1 + 1e-7)], want_vectors=True)
    assert status[0] == sg.ST_OK, (status, err, iters)
    assert abs(w[0] - es.eig[jo]) / abs(es.eig[jo]) < EIG_REL
    assert np.max(np.abs(H.phase_normalize(vecs[0]) - H.phase_normalize(es.evec[:, jo]))) < VEC_ABS


def test_fd_spatial_cli_evec(tmp_path):
    """stab_gpu < input with itype 4: evec.dat records itype 2, the x read
    after the index, and ogengrid's grid."""
    N = 32
    with open(tmp_path / "profile.0", "w") as fh:
        for r in H.ts_profile():
            fh.write(" ".join(repr(float(v)) for v in r) + "\n")
    text = "0\n0.3 1000 1\n%d 1.0 50.0\n1\n1\n0 0 0 0\n4\n0.08, 0\n0 0\n0\n123.5\n" % N
    r = subprocess.run([os.path.join(BIN, "stab_gpu")], cwd=tmp_path, input=text, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    h, y, eig, vec = sg.read_evec(str(tmp_path / "evec.dat"))
    assert h.itype == 2 and h.ny == N and h.x == 123.5
    assert np.array_equal(y, sg.fd_grid(N, 1.0, 50.0)[0])
    es = H.oracle_solve(_ts_spatial(N), H.ts_profile(), want_vectors=False)
    g = 2.2804739411185E-001 - 6.5163146952733E-003j
    j, jo = so.getevec_select(eig, g), so.getevec_select(es.eig, g)
    assert abs(eig[j] - es.eig[jo]) / abs(es.eig[jo]) < EIG_REL
