"""The file-interface drop-ins on the GPU: every eigenvector of a spectrum
(the evec.dat R5 record), and `stab_gpu < input` followed by `getevec_gpu -v`
as the reference's run script does it (thesis/TStest/run.sh:16-30), checked
against the reference's golden eigenfunction files.

Tolerances: eigenpair residual |A x - w B x| <= 1e-10 |A| |x| for every pair;
eigenvectors of well-separated eigenvalues within 1e-8 of the oracle's after
phase normalisation; golden files ndiff -abserr 1e-8 (run.sh:36-39).
"""
import os
import subprocess

import numpy as np
import pytest

import stab_gb300 as sg
from tests import helpers as H

pytestmark = pytest.mark.gpu
BIN = os.path.join(os.path.dirname(sg.__file__), "bin")


def test_all_eigenvectors_temporal(ctx):
    d, prof = H.synth_case(1, 16, 0.5, 1000.0, a=0.2)
    p = H.stab_params(d)
    eig, _, li, st = ctx.full_spectrum(p, prof, want_vector=False)
    vec, vst = ctx.eigenvectors(p, prof, eig)
    assert vec.shape == (80, 80) and np.all(vst == sg.ST_OK)
    A0, B0 = ctx.assemble(p, prof)
    scale = np.linalg.norm(A0, 2)
    for j in range(80):
        x = vec[:, j]
        r = A0 @ x - eig[j] * (B0 @ x)
        assert np.linalg.norm(r) <= 1e-10 * scale * np.linalg.norm(x), j
    # temporal columns are divided by their first max-modulus entry
    k = np.argmax(np.abs(vec), axis=0)
    assert np.allclose(vec[k, np.arange(80)], 1.0, atol=1e-14)
    es = H.oracle_solve(d, prof)
    for j in range(80):
        gap = np.min(np.abs(np.delete(eig, j) - eig[j]))
        if abs(eig[j]) > 1e-8 and gap > 1e-3 * max(1.0, abs(eig[j])):
            jo = int(np.argmin(np.abs(es.eig - eig[j])))
            assert np.max(np.abs(H.phase_normalize(vec[:, j]) - H.phase_normalize(es.evec[:, jo]))) < 1e-8, j


def _write_profile(path, prof):
    with open(path, "w") as fh:
        fh.write("# y rho u v w T\n")
        for r in prof:
            fh.write(" ".join(repr(float(v)) for v in r) + "\n")


def _ndiff_ok(a_text, b_text, tol):
    ra = [ln.split() for ln in a_text.splitlines() if ln.strip() and not ln.startswith("#")]
    rb = [ln.split() for ln in b_text.splitlines() if ln.strip() and not ln.startswith("#")]
    assert len(ra) == len(rb)
    return max(abs(float(x) - float(y)) for u, v in zip(ra, rb) for x, y in zip(u, v)) <= tol


@pytest.mark.parametrize("inp,case,out,ref", [
    ("test_input.inp", "test_spatial_n32", "space.1", "space1.ref"),
    ("thesis_temporal.inp", "thesis_temporal_n96", "time.1", "thesis_time.ref"),
    ("thesis_spatial.inp", "thesis_spatial_n96", "space.1", "thesis_space.ref"),
])
def test_cli_run_script_reproduces_golden(tmp_path, inp, case, out, ref):
    _write_profile(tmp_path / "profile.0", H.ts_profile())
    text = open(os.path.join(H.GOLDEN, inp)).read()
    r = subprocess.run([os.path.join(BIN, "stab_gpu")], cwd=tmp_path, input=text, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    g = complex(*H.cases()[case]["golden"])
    r = subprocess.run([os.path.join(BIN, "getevec_gpu"), "-v"], cwd=tmp_path, capture_output=True, text=True,
                       input=f"evec.dat\n{g.real!r} {g.imag!r}\n0 0\n", timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    got = open(tmp_path / out).read()
    assert _ndiff_ok(got, open(os.path.join(H.GOLDEN, ref)).read(), 1e-8)
    h, y, eig, vec = sg.read_evec(str(tmp_path / "evec.dat"))
    assert np.all(np.diff(eig.imag) >= 0)          # PIKSR2 order
    assert h.has_vectors == 1 and np.all(np.isfinite(vec))
