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
    q = _stab_params(d)
    q.ider = int(d.get("ider", 1))
    q.curve = int(d.get("curve", 0))
    q.x = float(d.get("x", 0.0))
    return q


def case_profile(c: dict) -> np.ndarray:
    """The profile rows of a golden case (the TStest profile unless named)."""
    return np.load(os.path.join(GOLDEN, c.get("profile", "ts_profile.npy")))


def _stab_params(d: dict):
    import stab_gb300
    return stab_gb300.StabParams.make(
        itype=d["itype"], ny=d["ny"], Ma=d["Ma"], Re=d["Re"], Pr=d["Pr"], mattyp=d["mattyp"], T0=d["T0"],
        yi=d["yi"], ymax=d["ymax"], alpha=complex(*d["alpha"]), beta=complex(*d["beta"]),
        omega=complex(*d["omega"]), top=d["top"], wall=d["wall"], wallt=d["wallt"], ievec=d["ievec"])


def oracle_params(d: dict) -> so.StabParams:
    return so.StabParams(mattyp=d["mattyp"], T0=d["T0"], Ma=d["Ma"], Re=d["Re"], Pr=d["Pr"], ny=d["ny"],
                         yi=d["yi"], ymax=d["ymax"], ievec=d["ievec"], ider=int(d.get("ider", 1)), top=d["top"],
                         wall=d["wall"], wallt=d["wallt"], curve=int(d.get("curve", 0)), x=float(d.get("x", 0.0)),
                         itype=d["itype"], alpha=complex(*d["alpha"]),
                         beta=complex(*d["beta"]), omega=complex(*d["omega"]))


def synth_case(itype, N, M, Re, a=0.0, b=0.0, w=0.0, ymax=50.0, yi=1.0 / 23.0, crossflow=False, width=2.0):
    """Run parameters + profile with the shapes of the benchmark configurations."""
    d = dict(mattyp=1, T0=T0_SUTH, Ma=M, Re=Re, Pr=0.72, ny=N, yi=yi, ymax=ymax, ievec=1, ider=1, top=0,
             wall=0, wallt=0, curve=0, itype=itype, alpha=[a, 0.0], beta=[b, 0.0], omega=[w, 0.0])
    y, vt = so.synthetic_profile(M, ymax, erf_width=width, crossflow=crossflow)
    prof = np.column_stack([y, vt])
    return d, prof


def derivative_tables(prof: np.ndarray, M: float, width=2.0, crossflow=False) -> np.ndarray:
    """Rows of 18 values for ider = 0: the synthetic profile row (y rho u v w
    T), then the exact first and second y-derivatives of its fields on the
    same y (U = erf(y/s), T by Crocco-Busemann, rho = 1/T, W the crossflow
    profile), each table "y f1..f5" as first.<ind> / second.<ind>."""
    import math
    y = prof[:, 0]
    s = width
    U = prof[:, 2]
    T = prof[:, 5]
    U1 = 2.0 / (s * math.sqrt(math.pi)) * np.exp(-(y / s) ** 2)
    U2 = -2.0 * y / s ** 2 * U1
    Tw = 1.0 + 0.2 * math.sqrt(0.72) * M ** 2
    c = 0.2 * M ** 2
    T1 = ((1.0 - Tw) + c * (1.0 - 2.0 * U)) * U1
    T2 = ((1.0 - Tw) + c * (1.0 - 2.0 * U)) * U2 - 2.0 * c * U1 ** 2
    r1 = -T1 / T ** 2
    r2 = -T2 / T ** 2 + 2.0 * T1 ** 2 / T ** 3
    if crossflow:
        e = np.exp(1.0 - y / 1.5)
        W1 = 0.08 / 1.5 * e * (1.0 - y / 1.5)
        W2 = -0.08 / 1.5 / 1.5 * e * (2.0 - y / 1.5)
    else:
        W1 = W2 = np.zeros_like(y)
    z = np.zeros_like(y)
    first = np.column_stack([y, r1, U1, z, W1, T1])
    second = np.column_stack([y, r2, U2, z, W2, T2])
    return np.hstack([prof, first, second])


def oracle_solve(d: dict, prof: np.ndarray, want_vectors=True):
    p = oracle_params(d)
    ym = prof[:, 0].copy()
    vt = prof[:, 1:6].copy()
    vt[:, 2] = 0.0
    if prof.shape[1] == 18:   # ider = 0: the derivative tables ride along
        p.ider = 0
        return so.solve(p, ym, vt, want_vectors, first=prof[:, 6:12], second=prof[:, 12:18])
    return so.solve(p, ym, vt, want_vectors)


def select_least(eig: np.ndarray, d: dict) -> int:
    """Index of the least-stable mode in `eig` (post.cu's rule)."""
    M = d["Ma"]
    cmax = 10.0 * (1.0 + 1.0 / M)
    a, b, w = complex(*d["alpha"]), complex(*d["beta"]), complex(*d["omega"])
    kabs = max(abs(np.sqrt(a * a + b * b)), 1e-3)
    # spatial spectra: lambda = 1/alpha below 1e-6 max |lambda| is a zero
    # eigenvalue of the companion matrix at rounding level (large alpha of
    # arbitrary phase) and is not a candidate
    eig = np.asarray(eig)
    fin = eig[np.isfinite(eig) & (eig != 0)]
    amax = 1e6 * float(np.min(np.abs(fin))) if fin.size else math.inf
    best, bi = -math.inf, -1
    for q, x in enumerate(eig):
        if not np.isfinite(x):
            continue
        ax = abs(x)
        if d["itype"] in (1, 3):
            if not ax > 1e-12 or ax > cmax * kabs:
                continue
            key = x.imag
        else:
            if ax == 0 or not x.real > 0 or abs(x.imag) > x.real or abs(w / x) > cmax or ax > amax:
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
