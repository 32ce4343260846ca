"""The reference's file interface on the host (no GPU): the stdin protocol,
profile.<ind>, the collocation grid, evec.dat and the time.N / space.N
eigenfunction files, each against the oracle or the reference's own files.

Tolerances: grid 1e-15 relative; evec.dat records R1, R2, R4, R5 bit-exact
(they pass through), R3 within 1e-15 relative (the grid); eigenfunction text
identical to the oracle's for the same eigenpair; golden files ndiff
-abserr 1e-8 (thesis/TStest/run.sh:36-39).
"""
import os
import struct
import subprocess

import numpy as np
import pytest

import stab_gb300 as sg
from oracle import stab_oracle as so
from tests import helpers as H

GOLD = H.GOLDEN
INPUTS = {"test_spatial_n32": "test_input.inp", "tstest_spatial_n96": "tstest_input.inp",
          "thesis_temporal_n96": "thesis_temporal.inp", "thesis_spatial_n96": "thesis_spatial.inp"}
BIN = os.path.join(os.path.dirname(sg.__file__), "bin")


@pytest.fixture(scope="module", autouse=True)
def built():
    if not (os.path.exists(sg.LIB_PATH) and os.path.exists(os.path.join(BIN, "getevec_gpu"))):
        from stab_gb300 import build
        build.build()
    sg.load()


def _text(name):
    return open(os.path.join(GOLD, name)).read()


@pytest.mark.parametrize("case,fname", sorted(INPUTS.items()))
def test_parse_input_matches_oracle(case, fname):
    text = _text(fname)
    p = sg.parse_input(text)
    o = so.parse_input(text)
    for k in ("mattyp", "ny", "ievec", "top", "wall", "wallt", "curve", "itype", "ind"):
        assert getattr(p, k) == getattr(o, k), k
    assert p.ider == (1 if o.ider else 0)
    for k in ("Ma", "Re", "Pr", "yi", "ymax", "x"):
        assert getattr(p, k) == getattr(o, k), k
    for k in ("alpha", "beta", "omega"):
        assert complex(*getattr(p, k)) == getattr(o, k), k
    c = H.cases()[case]
    assert (p.itype, p.ny, p.Ma, p.Re) == (c["itype"], c["ny"], c["Ma"], c["Re"])


def test_parse_input_list_directed_rules():
    # values spread over records, '/' ending a read, D exponents, bad mattyp and
    # itype read again (input.f90:15-17, :120-121), Sutherland T0 line
    text = "\n".join(["7", "1", "288.0", "0.5,", "1000 0.72", "64 0.043478 50.0 extra", "1", "1",
                      "0 0 2 0", "12", "1", "2.0D-1 0", "0.1 /", "3", ""])
    p = sg.parse_input(text)
    assert (p.mattyp, p.T0, p.Ma, p.Re, p.Pr) == (1, 288.0, 0.5, 1000.0, 0.72)
    assert (p.ny, p.yi, p.ymax, p.wallt, p.itype, p.ind) == (64, 0.043478, 50.0, 2, 1, 3)
    assert complex(*p.alpha) == 0.2 and complex(*p.beta) == 0.1


@pytest.mark.parametrize("text,needle", [
    ("0\n0.3 1000 1\n32 1 0\n1\n1\n0 0 0 0\n5\n0.1 0\n0 0\n0\n", "outside"),
    ("0\n0.3 1000 1\n32 1 0\n1\n1\n0 0 0 0\n6\n0.1 0\n0 0\n0\n", "outside"),
    ("0\n0.3 1000 1\n32 1 0\n1\n1\n0 0 0 0\n2\n0.1 0\n", "beta"),
    ("0\n0.3 x 1\n", "bad real"),
])
def test_parse_input_errors(text, needle):
    with pytest.raises(sg.StabError, match=needle):
        sg.parse_input(text)


def test_read_profile_skips_comments(tmp_path):
    prof = H.ts_profile()
    path = tmp_path / "profile.0"
    with open(path, "w") as fh:
        fh.write("# y rho u v w T\n")
        for r in prof:
            fh.write(" ".join(repr(float(v)) for v in r) + "\n")
        fh.write("\n")
    rows = sg.read_profile(str(path))
    assert rows.shape == prof.shape and np.array_equal(rows, prof)
    assert sg.profile_name(0) == "profile.0" and sg.profile_name(12) == "profile.12"
    with pytest.raises(sg.StabError):
        sg.read_profile(str(tmp_path / "missing.0"))


@pytest.mark.parametrize("ny,yi,ymax", [(32, 1.0, 0.0), (64, 1.0 / 23.0, 50.0), (17, 0.05, 20.0)])
def test_grid_matches_oracle(ny, yi, ymax):
    got = sg.grid(ny, yi, ymax)
    ref = so.sgengrid(ny, yi, ymax)
    for a, b in zip(got, ref):
        assert np.allclose(a, b, rtol=1e-15, atol=0)


def _records(data: bytes):
    out, i = [], 0
    while i < len(data):
        n = struct.unpack_from("<i", data, i)[0]
        out.append(data[i + 4:i + 4 + n])
        assert struct.unpack_from("<i", data, i + 4 + n)[0] == n
        i += 8 + n
    return out


def _small_system(itype):
    if itype == 1:
        d, prof = H.synth_case(1, 16, 0.5, 1000.0, a=0.2)
    else:
        d, prof = H.synth_case(2, 12, 0.8, 2000.0, w=0.05, b=0.1, crossflow=True)
    return d, prof, H.oracle_solve(d, prof)


@pytest.mark.parametrize("itype", [1, 2])
def test_write_evec_matches_oracle_layout(tmp_path, itype):
    d, prof, es = _small_system(itype)
    p = H.stab_params(d)
    path = str(tmp_path / "evec.dat")
    sg.write_evec(path, p, es.eig, es.evec)
    got = _records(open(path, "rb").read())
    ref = _records(so.evec_dat_bytes(es))
    assert len(got) == len(ref) == 5
    assert got[0] == ref[0] and got[1] == ref[1] and got[3] == ref[3] and got[4] == ref[4]
    a, b = np.frombuffer(got[2], dtype=np.float64), np.frombuffer(ref[2], dtype=np.float64)
    assert np.allclose(a, b, rtol=1e-15, atol=0)
    h, y, eig, vec = sg.read_evec(path)
    assert (h.ny, h.itype, h.nmax, h.has_vectors) == (d["ny"], itype, len(es.eig), 1)
    assert np.array_equal(eig, es.eig) and np.array_equal(vec, es.evec)


def test_spatial_evec_without_vectors(tmp_path):
    d, prof, es = _small_system(2)
    d = dict(d, ievec=0)
    path = str(tmp_path / "evec.dat")
    sg.write_evec(path, H.stab_params(d), es.eig, None)
    assert len(_records(open(path, "rb").read())) == 4
    h, y, eig, vec = sg.read_evec(path)
    assert h.has_vectors == 0 and vec is None


def test_eigfunction_text_matches_oracle(tmp_path):
    d, prof, es = _small_system(1)
    path = str(tmp_path / "evec.dat")
    sg.write_evec(path, H.stab_params(d), es.eig, es.evec)
    h, y, eig, vec = sg.read_evec(path)
    for j in (H.select_least(es.eig, d), 0, len(eig) - 1):
        assert sg.eigfunction_text(h, es.ms.y, eig[j], vec[:, j]) == so.eigfunction_text(es, j)
    assert sg.getevec_select(eig, eig[5] + 1e-9) == so.getevec_select(es.eig, eig[5] + 1e-9)


def _ndiff(a_text, b_text, tol):
    ra = [ln.split() for ln in a_text.splitlines() if ln.strip() and not ln.startswith("#")]
    rb = [ln.split() for ln in b_text.splitlines() if ln.strip() and not ln.startswith("#")]
    assert len(ra) == len(rb)
    return max(abs(float(x) - float(y)) for u, v in zip(ra, rb) for x, y in zip(u, v)) <= tol


def test_getevec_tool_on_oracle_system_reproduces_golden(tmp_path):
    """getevec -v on an evec.dat of the oracle's spectrum: the test/space.1 run
    (test/README.md) through the file chain, no GPU."""
    c = H.cases()["test_spatial_n32"]
    es = H.oracle_solve(c, H.ts_profile())
    p = sg.parse_input(_text("test_input.inp"))
    sg.write_evec(str(tmp_path / "evec.dat"), p, es.eig, es.evec)
    g = complex(*c["golden"])
    r = subprocess.run([os.path.join(BIN, "getevec_gpu"), "-v"], cwd=tmp_path, capture_output=True, text=True,
                       input=f"evec.dat\n{g.real!r} {g.imag!r}\n0 0\n", timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    out = open(tmp_path / "space.1").read()
    assert _ndiff(out, _text("space1.ref"), 1e-8)


def test_parse_fd_inputs():
    """itypes 3 and 4 (the finite-difference solvers, stab.f90:56-67) ask
    the temporal and the spatial questions: alpha or omega, beta, index, and
    x for the spatial one."""
    p = sg.parse_input("0\n0.3 1000 1\n128 1.0 50.0\n1\n1\n0 0 0 0\n3\n0.30862069, 0\n0 0\n0\n")
    assert p.itype == 3 and p.ny == 128 and p.ind == 0
    assert complex(*p.alpha) == 0.30862069 and complex(*p.beta) == 0
    p = sg.parse_input("0\n0.3 1000 1\n128 1.0 50.0\n1\n1\n0 0 0 1\n4\n0.08 0\n0 0\n0\n2.5\n")
    assert p.itype == 4 and p.curve == 1 and p.x == 2.5 and complex(*p.omega) == 0.08
