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
