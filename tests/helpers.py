"""Shared helpers of the test-suite: fixtures, the oracle bridge, and the
Python statement of the least-stable selection rule used by post.cu."""
import json
import math
import os

import numpy as np

from oracle import stab_oracle as so

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
T0_SUTH = 110.4 / 0.3815   # S/T_inf = 0.3815 with Sutherland's S = 110.4 K


def ts_profile() -> np.ndarray:
    return np.load(os.path.join(GOLDEN, "ts_profile.npy"))


def cases() -> dict:
    with open(os.path.join(GOLDEN, "cases.json")) as fh:
        return json.load(fh)


def stab_params(d: dict):
    import stab_gb300
    return stab_gb300.StabParams.make(
        itype=d["itype"], ny=d["ny"], Ma=d["Ma"], Re=d["Re"], Pr=d["Pr"], mattyp=d["mattyp"], T0=d["T0"],
        yi=d["yi"], ymax=d["ymax"], alpha=complex(*d["alpha"]), beta=complex(*d["beta"]),
        omega=complex(*d["omega"]), top=d["top"], wall=d["wall"], wallt=d["wallt"], ievec=d["ievec"])


def oracle_params(d: dict) -> so.StabParams:
    return so.StabParams(mattyp=d["mattyp"], T0=d["T0"], Ma=d["Ma"], Re=d["Re"], Pr=d["Pr"], ny=d["ny"],
                         yi=d["yi"], ymax=d["ymax"], ievec=d["ievec"], ider=1, top=d["top"], wall=d["wall"],
                         wallt=d["wallt"], curve=0, itype=d["itype"], alpha=complex(*d["alpha"]),
                         beta=complex(*d["beta"]), omega=complex(*d["omega"]))


def synth_case(itype, N, M, Re, a=0.0, b=0.0, w=0.0, ymax=50.0, yi=1.0 / 23.0, crossflow=False, width=2.0):
    """Run parameters + profile with the shapes of the benchmark configurations."""
    d = dict(mattyp=1, T0=T0_SUTH, Ma=M, Re=Re, Pr=0.72, ny=N, yi=yi, ymax=ymax, ievec=1, ider=1, top=0,
             wall=0, wallt=0, curve=0, itype=itype, alpha=[a, 0.0], beta=[b, 0.0], omega=[w, 0.0])
    y, vt = so.synthetic_profile(M, ymax, erf_width=width, crossflow=crossflow)
    prof = np.column_stack([y, vt])
    return d, prof


def oracle_solve(d: dict, prof: np.ndarray, want_vectors=True):
    p = oracle_params(d)
    ym = prof[:, 0].copy()
    vt = prof[:, 1:6].copy()
    vt[:, 2] = 0.0
    return so.solve(p, ym, vt, want_vectors)


def select_least(eig: np.ndarray, d: dict) -> int:
    """Index of the least-stable mode in `eig` (post.cu's rule)."""
    M = d["Ma"]
    cmax = 10.0 * (1.0 + 1.0 / M)
    a, b, w = complex(*d["alpha"]), complex(*d["beta"]), complex(*d["omega"])
    kabs = max(abs(np.sqrt(a * a + b * b)), 1e-3)
    best, bi = -math.inf, -1
    for q, x in enumerate(eig):
        if not np.isfinite(x):
            continue
        ax = abs(x)
        if d["itype"] == 1:
            if not ax > 1e-12 or ax > cmax * kabs:
                continue
            key = x.imag
        else:
            if ax == 0 or not x.real > 0 or abs(x.imag) > x.real or abs(w / x) > cmax:
                continue
            key = -x.imag
        if key > best:
            best, bi = key, q
    return bi


def phase_normalize(v: np.ndarray) -> np.ndarray:
    """Divide by the first max-modulus entry (the reference's evec scaling)."""
    k = int(np.argmax(np.abs(v)))
    return v / v[k]


def eigfunction_rows(vec: np.ndarray, ny: int, y: np.ndarray) -> np.ndarray:
    """The numeric block of a time.N / space.N file (getevec.f90:179-227):
    rows wall first, columns y then Re/Im of rho u v w T."""
    v = so.getevec_scale(np.asarray(vec), ny)
    out = np.zeros((ny, 11))
    for r, i in enumerate(range(ny - 1, -1, -1)):
        out[r, 0] = y[i]
        for e in range(5):
            out[r, 1 + 2 * e] = v[5 * i + e].real
            out[r, 2 + 2 * e] = v[5 * i + e].imag
    return out


def ref_rows(name: str) -> np.ndarray:
    _, rows = so.parse_eigfunction(open(os.path.join(GOLDEN, name)).read())
    return rows
