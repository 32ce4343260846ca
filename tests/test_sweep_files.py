"""The multi-point drivers' protocol and the sweep post-processors, on the
host (no GPU): stdin parsing of itypes 7 and 8, the drivers' loop order
(mtemporal.f90:25-39, mspatial.f90:65-96) against the oracle's restatement,
delta.dat / body.dat readers, and getab_gpu / getax_gpu / getalpha_gpu run
on eig.<iver> files written by the oracle: their stab.out / parm.new must
equal, byte for byte, the oracle's picks (getab.f90:161-201,
getalpha.f90:120-146) written in the reference's formats.
"""
import os
import subprocess

import numpy as np
import pytest

import stab_gb300 as sg
from oracle import stab_oracle as so
from tests import helpers as H

BIN = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "stab_gb300", "bin")

HEAD = "1\n289.38\n0.5 1000 0.72\n16 0.0434782608695652 50\n1\n1\n0 0 0 0\n"


def test_parse_temporal_sweep():
    p, sw = sg.parse_sweep_input(HEAD + "7\n0.1 0.3 0.05\n0.0 0.1 0.05\n")
    assert sw.itype == 7 and p.itype == 1 and p.ind == 0
    assert (sw.p_min, sw.p_max, sw.p_inc, sw.b_min, sw.b_max, sw.b_inc) == (0.1, 0.3, 0.05, 0.0, 0.1, 0.05)
    pts = sg.sweep_points(p, sw)
    ref = so.mtemporal_points(0.1, 0.3, 0.05, 0.0, 0.1, 0.05)
    assert len(pts) == len(ref) == 4 * 2          # amax and bmax are not reached (nint without + 1)
    for q, (a, b) in zip(pts, ref):
        assert (q.alpha[0], q.alpha[1], q.beta[0], q.beta[1]) == (a, 0.0, b, 0.0)
        assert q.itype == 1 and q.ind == 0 and q.ny == 16


def test_parse_spatial_sweep_and_stations(tmp_path):
    p, sw = sg.parse_sweep_input(HEAD + "8\n0.05 0.07 0.01\n0 0 0\n2 3 1\n0\n")
    assert sw.itype == 8 and p.itype == 2
    assert (sw.ind1, sw.ind2, sw.ind_inc, sw.dtype) == (2, 3, 1, 0)
    text = "# x delta\n100.0 0.5\n# comment\n200.0 0.75\n300.0 1.0\n"
    (tmp_path / "delta.dat").write_text(text)
    xb, de = sg.read_delta(str(tmp_path / "delta.dat"))
    rx, rd = so.read_delta(text)
    assert np.array_equal(xb, rx) and np.array_equal(de, rd)
    pts = sg.sweep_points(p, sw, xb, de)
    ref = so.mspatial_points(0.05, 0.07, 0.01, 0.0, 0.0, 0.0, 2, 3, 1, rx, rd)
    assert len(pts) == len(ref) == 2 * 3 * 1       # zero beta increment becomes one: one beta
    for q, (ind, x, yi, w, b) in zip(pts, ref):
        assert (q.ind, q.x, q.yi, q.omega[0], q.beta[0]) == (ind, x, yi, w, b)
    with pytest.raises(sg.StabError):
        sg.parse_sweep_input(HEAD + "8\n0.05 0.07 0.01\n0 0 0\n1 2 1\n1\n")   # dtype 1: finite differences
    with pytest.raises(sg.StabError):
        sg.parse_input(HEAD + "7\n0.1 0.3 0.05\n0.0 0.1 0.05\n")               # the single-point parser
    bad = sg.Sweep(itype=8, ind1=1, ind2=4, ind_inc=1, p_inc=1.0, b_inc=1.0)
    with pytest.raises(sg.StabError):
        sg.sweep_points(p, bad, xb, de)                                        # beyond delta.dat


def _spectra(betas, ny=16, xs=None):
    c = dict(H.cases()["thesis_temporal_n96"], ny=ny)
    out = []
    for j, b in enumerate(betas):
        d = dict(c, beta=[float(b), 0.0])
        p = H.oracle_params(d)
        if xs is not None:
            p.x = float(xs[j])
            p.ind = j + 1
        prof = H.ts_profile()
        ym, vt = prof[:, 0].copy(), prof[:, 1:6].copy()
        vt[:, 2] = 0.0
        out.append(so.solve(p, ym, vt, want_vectors=True))
    return out


def _run(tool, cwd, stdin, *args):
    r = subprocess.run([os.path.join(BIN, tool), *args], input=stdin, cwd=cwd, capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0, r.stderr
    return r


@pytest.fixture(scope="module")
def beta_files(tmp_path_factory):
    d = tmp_path_factory.mktemp("sweep")
    betas = np.linspace(0.0, 0.08, 5)
    xs = np.linspace(100.0, 180.0, 5)
    es = _spectra(betas, xs=xs)
    for j, e in enumerate(es):
        (d / f"eig.{j + 1}").write_bytes(so.evec_dat_bytes(e))
    (d / "body.dat").write_text("".join(f"{j + 1} {x}\n" for j, x in enumerate(xs)))
    return d, betas, xs, es


def test_getab_matches_oracle_picks(beta_files):
    d, betas, xs, es = beta_files
    first = [es[0].eig[-1], es[1].eig[-1]]        # the most unstable (sorted by Im), typed as approximations
    stdin = f"1 5 1\n{first[0].real} {first[0].imag}\n{first[1].real} {first[1].imag}\n"
    _run("getab_gpu", d, stdin, "-v")
    picks = so.getab_picks([e.eig for e in es], betas, first)
    assert (d / "stab.out").read_text() == so.stab_out_text(betas, picks)
    # by index: the same modes
    jl = [int(np.argmin(np.abs(es[k].eig - first[k]))) + 1 for k in range(2)]
    _run("getab_gpu", d, f"1 5 1\n{jl[0]}\n{jl[1]}\n", "-i")
    assert (d / "stab.out").read_text() == so.stab_out_text(betas, picks)


def test_getax_matches_oracle_picks(beta_files):
    d, betas, xs, es = beta_files
    first = [es[0].eig[-1], es[1].eig[-1]]
    _run("getax_gpu", d, f"1 5 1\n{first[0].real} {first[0].imag}\n{first[1].real} {first[1].imag}\n", "-v")
    picks = so.getab_picks([e.eig for e in es], xs, first)
    assert (d / "stab.out").read_text() == so.stab_out_text(xs, picks, ind=list(range(1, 6)))


def test_getalpha_matches_oracle_picks(beta_files):
    d, betas, xs, es = beta_files
    jloc = len(es[0].eig)                          # the most unstable, by index
    _run("getalpha_gpu", d, f"1 5 1\n{jloc}\n")
    picks = so.getalpha_picks([e.eig for e in es], jloc)
    assert (d / "parm.new").read_text() == so.stab_out_text(xs, picks, ind=list(range(1, 6)))
    r = subprocess.run([os.path.join(BIN, "getalpha_gpu")], input="1 9 1\n", cwd=d, capture_output=True, text=True)
    assert r.returncode != 0 and "illegal index" in r.stdout


def test_stab_out_line_matches_oracle_format():
    for p, v, ind in [(0.02, 0.1 - 2e-3j, None), (150.0, -1.5e-120 + 3j, 7), (0.0, 0j, 12345)]:
        want = so.stab_out_text([p], [v], ind=None if ind is None else [ind]).rstrip("\n")
        if ind == 12345:
            want = "****" + want[len(str(ind)):]     # i4 overflow prints asterisks
        assert sg.stab_out_line(p, v, ind) == want
