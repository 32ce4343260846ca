"""Sweep tracking rules and output files on the host (no GPU), against the
oracle's restatement of getab / getax / getalpha."""
import numpy as np

from oracle import stab_oracle as so
from stab_gb300 import sweep as sw


def test_extrapolation_rule_matches_reference():
    param = np.array([0.0, 0.1, 0.2, 0.35])
    vals = np.array([1 + 1j, 1.5 + 0.5j, 0, 0])
    assert sw.guess("extrapolate", 0, param, vals, [1 + 1j, 1.5 + 0.5j]) == 1 + 1j
    assert sw.guess("extrapolate", 1, param, vals, [1 + 1j, 1.5 + 0.5j]) == 1.5 + 0.5j
    g = sw.guess("extrapolate", 2, param, vals, [1 + 1j, 1.5 + 0.5j])
    assert abs(g - (2.0 + 0.0j)) < 1e-15
    assert sw.guess("nearest", 2, param, vals, [1 + 1j]) == vals[1]


def test_track_pick_follows_a_moving_mode():
    rng = np.random.default_rng(0)
    param = np.linspace(0, 1, 9)
    true = 0.3 + 0.1 * param + 1j * (0.01 - 0.02 * param)
    spectra = [np.concatenate([[t], rng.normal(size=20) + 1j * rng.normal(size=20)]) for t in true]
    picks = so.track_pick(spectra, param, [true[0] + 1e-3, true[1] - 1e-3], "extrapolate")
    assert np.allclose(picks, true)
    picks = so.track_pick(spectra, param, [true[0]], "nearest")
    assert np.allclose(picks, true)


def test_stab_out_format_matches_oracle():
    param = np.array([0.05, 0.1, 1e-120])
    vals = np.array([0.2280502265 - 0.0065136925j, -1.5e-3 + 2e105j, 0j])
    assert sw.stab_out_lines(param, vals) == so.stab_out_text(param, vals)
    assert sw.stab_out_lines(param, vals, ind=[1, 2, 13]) == so.stab_out_text(param, vals, ind=[1, 2, 13])
    first = sw.stab_out_lines(param, vals).splitlines()[0]
    assert first == "  5.0000000000000E-02  2.2805022650000E-01 -6.5136925000000E-03"
