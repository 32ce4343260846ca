"""Mode tracking along a sweep on the GPU (MODE_TRACK) against the oracle's
restatement of the reference's picks (full spectrum per point, then getab's
extrapolation or getalpha's nearest-previous rule).

Tolerance: every tracked eigenvalue within 1e-10 relative of the oracle's pick.
"""
import numpy as np
import pytest

import stab_gb300 as sg
from oracle import stab_oracle as so
from stab_gb300 import sweep as sw
from tests import helpers as H

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("rule", ["extrapolate", "nearest"])
def test_track_beta_sweep_matches_reference_picks(ctx, rule):
    base = dict(H.cases()["thesis_temporal_n96"], ny=32)
    prof = H.ts_profile()
    betas = np.linspace(0.0, 0.1, 6)
    lines, profs, oracle_picks, starts = [], [], [], []
    for Re in (1000.0, 1200.0):
        pts, spectra = [], []
        for b in betas:
            d = dict(base, Re=Re, beta=[float(b), 0.0])
            pts.append(H.stab_params(d))
            spectra.append(H.oracle_solve(d, prof, want_vectors=False).eig)
        start = [so.getevec_select(spectra[0], 0.1147 + 0.0024j), so.getevec_select(spectra[1], 0.1147 + 0.0024j)]
        start = [spectra[0][start[0]], spectra[1][start[1]]][: 2 if rule == "extrapolate" else 1]
        lines.append(pts)
        profs.append([prof] * len(betas))
        starts.append(start)
        oracle_picks.append(so.track_pick(spectra, betas, start, rule))
    vals, st = sw.track_lines(ctx, lines, profs, betas, starts, rule)
    ref = np.asarray(oracle_picks)
    assert np.all(np.isin(st, [sg.ST_OK, sg.ST_FELLBACK]))
    assert np.max(np.abs(vals - ref) / np.abs(ref)) < 1e-10
    # stab.out: the library's writer and the oracle's restatement of the
    # reference's format give the same bytes for the same values, and the
    # numbers read back agree with the oracle's picks
    text = sw.stab_out_lines(betas, vals[0])
    assert text == so.stab_out_text(betas, vals[0])
    back = np.array([[float(t) for t in ln.split()] for ln in text.splitlines()])
    assert back.shape == (len(betas), 3)
    assert np.max(np.abs(back[:, 1] + 1j * back[:, 2] - ref[0]) / np.abs(ref[0])) < 1e-10
    assert np.allclose(back[:, 0], betas, rtol=1e-12, atol=1e-15)


def _write_profile(path, prof):
    with open(path, "w") as fh:
        fh.write("# y rho u v w T\n")
        for row in prof:
            fh.write(" ".join(f"{v:.17e}" for v in row) + "\n")


def _run(tool, cwd, stdin, *args):
    import os
    import subprocess
    b = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "stab_gb300", "bin", tool)
    r = subprocess.run([b, *args], input=stdin, cwd=cwd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return r


def test_temporal_driver_writes_eig_files_and_getab_follows_the_mode(tmp_path):
    """itype 7 through stab_gpu (mtemporal.f90: an alpha x beta sweep on
    profile.0, one eig.<iver> per point), then getab_gpu -v on the beta
    sweep.  Each eig.<iver>: header as the reference writes it, least-stable
    eigenvalue within 1e-10 of the oracle's spectrum at that point, every
    oracle eigenvalue with |omega| < 2 within 1e-8, and the eigenvector
    record (R5) present.  stab.out: the oracle's getab picks over the
    oracle's spectra, each within 1e-10."""
    c = dict(H.cases()["thesis_temporal_n96"], ny=24)
    prof = H.ts_profile()
    _write_profile(tmp_path / "profile.0", prof)
    text = ("0\n0.3 1000 1\n24 1.0 0.0\n1\n1\n0 0 0 0\n7\n"
            "0.30862069 0.40862069 0.1\n0.0 0.1 0.02\n")
    _run("stab_gpu", tmp_path, text)
    betas = [0.02 * k for k in range(5)]     # nb = nint(0.1 / 0.02) = 5; na = 1
    spectra = []
    for j, b in enumerate(betas):
        h, y, eig, vec = sg.read_evec(str(tmp_path / f"eig.{j + 1}"))
        assert h.itype == 1 and h.ny == 24 and h.ind == 0 and vec is not None
        assert abs(h.beta[0] - b) < 1e-15 and abs(h.alpha[0] - 0.30862069) < 1e-15
        d = dict(c, beta=[b, 0.0])
        ref = H.oracle_solve(d, prof, want_vectors=False).eig
        jo = H.select_least(ref, d)
        je = H.select_least(eig, d)
        assert abs(eig[je] - ref[jo]) / abs(ref[jo]) < 1e-10
        for w in ref[(np.abs(ref) > 0) & (np.abs(ref) < 2.0)]:
            assert np.min(np.abs(eig - w)) <= 1e-8 * max(1.0, abs(w))
        spectra.append((eig, ref, jo))
    assert not (tmp_path / f"eig.{len(betas) + 1}").exists()
    (tmp_path / "body.dat").write_text("1 0.0\n")
    first = [spectra[0][1][spectra[0][2]], spectra[1][1][spectra[1][2]]]   # the least-stable mode
    _run("getab_gpu", tmp_path, f"1 5 1\n{first[0].real} {first[0].imag}\n{first[1].real} {first[1].imag}\n", "-v")
    want = so.getab_picks([r for _, r, _ in spectra], betas, first)
    got = np.array([[float(t) for t in ln.split()] for ln in (tmp_path / "stab.out").read_text().splitlines()])
    assert got.shape == (5, 3)
    assert np.max(np.abs(got[:, 1] + 1j * got[:, 2] - np.array(want)) / np.abs(want)) < 1e-10


def test_spatial_driver_stations_and_getalpha(tmp_path):
    """itype 8 through stab_gpu (mspatial.f90: stations of delta.dat with
    x = xb(ind), Yi = 2 delta(ind), each on its own profile.<ind>), then
    getalpha_gpu (nearest previous value) and getax_gpu.  Each station's
    least-stable alpha within 1e-10 of the oracle at that station's Yi; the
    parm.new picks within 1e-10 of the oracle's getalpha picks."""
    prof = H.ts_profile()
    base = H.cases()["test_spatial_n32"]
    delta = [0.5, 0.55, 0.6]
    xs = [100.0, 110.0, 120.0]
    (tmp_path / "delta.dat").write_text("# x delta\n" + "".join(f"{x} {d}\n" for x, d in zip(xs, delta)))
    (tmp_path / "body.dat").write_text("".join(f"{k + 1} {x}\n" for k, x in enumerate(xs)))
    for k in (1, 2, 3):
        _write_profile(tmp_path / f"profile.{k}", prof)
    d0 = dict(base, ny=24)
    text = (f"{d0['mattyp']}\n{d0['Ma']} {d0['Re']} {d0['Pr']}\n24 1.0 0.0\n1\n1\n{d0['top']} 0 0 0\n8\n"
            "0.08 0.08 0\n0 0 0\n1 3 1\n0\n")
    _run("stab_gpu", tmp_path, text)
    spectra = []
    for k in range(3):
        h, y, eig, vec = sg.read_evec(str(tmp_path / f"eig.{k + 1}"))
        assert h.itype == 2 and h.ind == k + 1 and abs(h.x - xs[k]) < 1e-12 and abs(h.yi - 2 * delta[k]) < 1e-12
        d = dict(d0, yi=2 * delta[k], omega=[0.08, 0.0], beta=[0.0, 0.0])
        ref = H.oracle_solve(d, prof, want_vectors=False).eig
        jo, je = H.select_least(ref, d), H.select_least(eig, d)
        assert jo >= 0 and je >= 0
        assert abs(eig[je] - ref[jo]) / abs(ref[jo]) < 1e-10
        spectra.append((eig, ref, jo, je))
    # the least-stable mode of the first station, by its index in each file's own sorted list
    _run("getalpha_gpu", tmp_path, f"1 3 1\n{spectra[0][3] + 1}\n")
    want = so.getalpha_picks([r for _, r, _, _ in spectra], spectra[0][2] + 1)
    got = np.array([[float(t) for t in ln.split()] for ln in (tmp_path / "parm.new").read_text().splitlines()])
    assert got.shape == (3, 4) and np.array_equal(got[:, 0], [1, 2, 3]) and np.allclose(got[:, 1], xs)
    assert np.max(np.abs(got[:, 2] + 1j * got[:, 3] - np.array(want)) / np.abs(want)) < 1e-10
    first = [want[0], want[1]]
    _run("getax_gpu", tmp_path, f"1 3 1\n{first[0].real} {first[0].imag}\n{first[1].real} {first[1].imag}\n", "-v")
    want_x = so.getab_picks([r for _, r, _, _ in spectra], xs, first)
    got = np.array([[float(t) for t in ln.split()] for ln in (tmp_path / "stab.out").read_text().splitlines()])
    assert np.max(np.abs(got[:, 2] + 1j * got[:, 3] - np.array(want_x)) / np.abs(want_x)) < 1e-10
