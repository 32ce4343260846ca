"""The oracle against the reference's own golden files (parity pin)."""
import numpy as np
import pytest

from oracle import stab_oracle as so
from tests import helpers as H

NDIFF_ABS = 1e-8        # thesis/TStest/run.sh:36-39 (ndiff -abserr 1e-8)
EIG_REL = 1e-10         # least-stable eigenvalue, relative


@pytest.mark.parametrize("name", ["test_spatial_n32", "tstest_spatial_n64", "tstest_spatial_n96",
                                  "thesis_temporal_n96", "thesis_spatial_n96"])
def test_oracle_eigenvalue_matches_reference(name):
    c = H.cases()[name]
    es = H.oracle_solve(c, H.ts_profile(), want_vectors=("eigfunction" in c))
    g = complex(*c["golden"])
    j = so.getevec_select(es.eig, g)   # getevec -v
    assert abs(es.eig[j] - g) / abs(g) < EIG_REL
    if "eigfunction" in c:
        rows = H.eigfunction_rows(es.evec[:, j], c["ny"], es.ms.y)
        ref = H.ref_rows(c["eigfunction"])
        assert rows.shape == ref.shape
        assert np.max(np.abs(rows[:, 1:] - ref[:, 1:])) < NDIFF_ABS
        assert np.allclose(rows[:-1, 0], ref[:-1, 0], rtol=1e-12, atol=1e-13)


def test_oracle_text_format_matches_space1():
    c = H.cases()["test_spatial_n32"]
    es = H.oracle_solve(c, H.ts_profile())
    j = so.getevec_select(es.eig, complex(*c["golden"]))
    txt = so.eigfunction_text(es, j).splitlines()
    ref = open(H.GOLDEN + "/space1.ref").read().splitlines()
    assert txt[0] == ref[0] and txt[1] == ref[1] and txt[3] == ref[3]
    assert len(txt) == len(ref)
    assert all(len(a) == len(b) for a, b in zip(txt[4:], ref[4:]))


def test_temporal_dirichlet_rows_give_exact_zero_eigenvalues():
    d, prof = H.synth_case(1, 24, 0.5, 1000.0, a=0.2)
    es = H.oracle_solve(d, prof, want_vectors=False)
    assert np.sum(es.eig == 0) == 8


def test_evec_dat_record_layout():
    d, prof = H.synth_case(1, 8, 0.5, 1000.0, a=0.2)
    es = H.oracle_solve(d, prof)
    raw = so.evec_dat_bytes(es)
    import struct
    n1 = struct.unpack("<i", raw[:4])[0]
    assert n1 == 40
    assert struct.unpack("<10i", raw[4:44])[:4] == (0, 8, 5, 1)


def test_oracle_external_derivatives_agree_with_internal():
    """getmean2 (ider = 0) restated: with the profile's exact derivative
    tables the least-stable eigenvalue equals the ider = 1 one (collocation
    derivatives of the splined profile) to 1e-6 relative (N = 32)."""
    from tests import helpers as H
    for itype, kw in ((1, dict(a=0.2, b=0.05)), (2, dict(w=0.05, b=0.1, crossflow=True))):
        d, prof = H.synth_case(itype, 32, 0.8, 1500.0, **kw)
        tab = H.derivative_tables(prof, 0.8, crossflow=kw.get("crossflow", False))
        e1 = H.oracle_solve(d, prof, want_vectors=False).eig
        d0 = dict(d, ider=0)
        e0 = H.oracle_solve(d0, tab, want_vectors=False).eig
        j1, j0 = H.select_least(e1, d), H.select_least(e0, d0)
        assert abs(e1[j1] - e0[j0]) / abs(e1[j1]) < 1e-6


@pytest.mark.parametrize("name", ["cftest_spatial_n64", "cftest_spatial_n96", "fsctest_spatial_n64"])
def test_oracle_curved_wall_matches_reference(name):
    """Curved walls (curve = 2, the circle of circh.f90 with radius x = 500):
    the crossflow case CFtest (N = 64 on SGI and N = 96 on MacOS, its README)
    and the Falkner-Skan-Cooke case FSCtest (N = 64, the header of its
    space.ref).  Eigenvalue within 1e-10 relative; at N = 64 the eigenfunction
    rows of space.ref (the first 5N entries of the companion eigenvector),
    matched by y and divided by their largest-modulus entry, within 1e-8."""
    c = H.cases()[name]
    prof = H.case_profile(c)
    es = H.oracle_solve(c, prof, want_vectors="eigfunction_rows" in c)
    g = complex(*c["golden"])
    j = so.getevec_select(es.eig, g)
    assert abs(es.eig[j] - g) / abs(g) < EIG_REL
    if "eigfunction_rows" in c:
        ref = np.loadtxt(H.GOLDEN + "/" + c["eigfunction_rows"], comments="#")
        ny = c["ny"]
        v = es.evec[:5 * ny, j].reshape(ny, 5)
        ys = es.ms.y
        assert ref.shape == (ny, 11)
        # rows matched by y (the files list them wall first or free stream first)
        order = [int(np.argmin(np.abs(ys - yr))) for yr in ref[:, 0]]
        assert len(set(order)) == ny
        assert np.allclose(ys[order], ref[:, 0], rtol=1e-10, atol=1e-12)
        got = v[order]
        want = ref[:, 1::2] + 1j * ref[:, 2::2]
        kg = np.unravel_index(np.argmax(np.abs(got)), got.shape)
        kw = np.unravel_index(np.argmax(np.abs(want)), want.shape)
        assert kg == kw
        assert np.max(np.abs(got / got[kg] - want / want[kw])) < NDIFF_ABS


def test_oracle_calch_scalars_follow_the_parabola():
    """curve = 1 (calch.f90): the eight wall scalars against central
    differences of the geometry itself, the wall point located to full
    precision by bisection on the arc length (independent of the
    false-position search calch uses).  Agreement to 1e-5 relative (the
    difference step's error); x = 0.5 is where calch's search gives up."""
    import math

    def wall(s):
        lo, hi = 0.0, 2.0 * s + 1.0
        for _ in range(200):
            mid = 0.5 * (lo + hi)
            if so.parabola_arc(0.0, mid) < s:
                lo = mid
            else:
                hi = mid
        x = 0.5 * (lo + hi)
        th = math.atan2(1.0, math.sqrt(2.0 * x))
        return np.array([x, math.sqrt(2.0 * x), -math.sin(th), math.cos(th)])

    for s in (1.0, 2.0, 5.0, 50.0):
        h = 1e-3 * max(1.0, s)
        a, c, b = wall(s - h), wall(s), wall(s + h)
        d1 = (b - a) / (2 * h)
        d2 = (b - 2 * c + a) / h ** 2
        sc = so.calch_scalars(s)
        want = [d1[0], d1[1], d1[2], d1[3], d2[0], d2[1], d2[2], d2[3]]
        for got, w in zip(sc, want):
            assert abs(got - w) <= 1e-5 * max(abs(w), 1e-3), (s, sc, want)
    with pytest.raises(ValueError):
        so.calch_scalars(0.5)
    p = so.StabParams(curve=1, x=-1.0, itype=2, ny=8)
    assert np.array_equal(so.wall_metrics(p, np.linspace(0, 1, 8))[0], np.ones(8))


def test_oracle_fd_temporal_converges_to_the_spectral_adiabatic_solution():
    """Finite-difference temporal solver (itype 3, fd_temporal.f90), thesis
    TStest fd_temporal.inp (M = 0.3, Re = 1000, Pr = 1, alpha = 0.30862069,
    Yi = 1, Ymax = 50, constant viscosity).  Its wall energy row is the
    energy equation with the temperature column's first-derivative term left
    out, an adiabatic condition whatever wallt says, so it converges to the
    Chebyshev solver's TS mode with wallt = 2 (pinned to the reference's
    golden files) rather than to the isothermal golden value of the
    README.  Fourth-order stencils: at N = 256 within 5e-8 relative, and the
    error falls by more than 4x from N = 64 to N = 128 (third-order
    closures at the boundaries)."""
    prof = H.ts_profile()
    ym, vt = prof[:, 0].copy(), prof[:, 1:6].copy()
    vt[:, 2] = 0.0
    base = dict(mattyp=0, T0=0.0, Ma=0.3, Re=1000.0, Pr=1.0, yi=1.0, ymax=50.0, ievec=1, ider=1, top=0, wall=0,
                curve=0, alpha=0.308620690 + 0j, beta=0j, omega=0j)
    spec = so.solve(so.StabParams(ny=96, wallt=2, itype=1, **base), ym, vt, want_vectors=False)
    g = 1.1467880189410E-001 + 2.3844535276592E-003j        # the isothermal value, to find the mode
    ref = spec.eig[so.getevec_select(spec.eig, g)]
    err = {}
    for N in (64, 128, 256):
        es = so.solve(so.StabParams(ny=N, wallt=0, itype=3, **base), ym, vt, want_vectors=False)
        assert es.params.itype == 1                          # stab.f90:59: recorded as temporal
        w = es.eig[so.getevec_select(es.eig, ref)]
        err[N] = abs(w - ref) / abs(ref)
    assert err[256] < 5e-8, err
    assert err[128] < err[64] / 4, err
    # the grid: uniform eta from the wall, y(0) = 0, y(1) = ymax
    y, eta, deta, d2eta, dy = so.ogengrid(33, 1.0, 50.0)
    assert y[0] == 0.0 and abs(y[-1] - 50.0) < 1e-12 and abs(eta[1] - 1.0 / 32) < 1e-15


def test_oracle_fd_spatial_converges_to_the_spectral_solution():
    """Finite-difference spatial solver (itype 4, fd_spatial.f90), thesis
    TStest case at omega = 0.08 (its spatial TS mode, README.md), Ymax = 50:
    with the isothermal wall (wallt = 0) and either free-stream condition it
    converges at fourth order to the Chebyshev solver's TS alpha (pinned to
    the reference's golden files): within 2e-7 at N = 128 and 3e-8 at
    N = 192, the error falling more than 10x from N = 64 to N = 128.  (With
    wallt = 2 it does not: its wall energy row takes G from another node, a
    quirk the restatement keeps.)"""
    prof = H.ts_profile()
    ym, vt = prof[:, 0].copy(), prof[:, 1:6].copy()
    vt[:, 2] = 0.0
    g = 2.2804739411185E-001 - 6.5163146952733E-003j
    for top in (0, 1):
        base = dict(mattyp=0, T0=0.0, Ma=0.3, Re=1000.0, Pr=1.0, yi=1.0, ymax=50.0, ievec=1, ider=1, top=top,
                    wall=0, wallt=0, curve=0, alpha=0j, beta=0j, omega=0.08 + 0j)
        spec = so.solve(so.StabParams(ny=96, itype=2, **base), ym, vt, want_vectors=False)
        ref = spec.eig[so.getevec_select(spec.eig, g)]     # the same TS mode on this grid (Ymax = 50)
        err = {}
        for N in (64, 128) if top else (64, 128, 192):
            es = so.solve(so.StabParams(ny=N, itype=4, **base), ym, vt, want_vectors=False)
            assert es.params.itype == 2                     # stab.f90:66: recorded as spatial
            w = es.eig[so.getevec_select(es.eig, ref)]
            err[N] = abs(w - ref) / abs(ref)
        assert err[128] < 2.5e-7 and err[128] < err[64] / 10, err
        if 192 in err:
            assert err[192] < 3e-8, err
