"""CPU oracle for the stab Chebyshev linear-stability path (TEST INFRASTRUCTURE).

This module is the checker, never the product.  Only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference`` legs
of ``bench.py`` may import it.  It restates, in numpy/scipy, the algorithm of
the reference Fortran (sscollis/stab), routine by routine, with the
reference's own LAPACK calls (ZGESV, ZGETRF, ZGETRS, ZGEEV) taken from
scipy's bundled LAPACK:

  grid            sgengrid.f90:2-45       (algebraic maps only)
  mean profile    getmean.f90:2-122, spline.f90:2-75 (SPLINE / SPEVAL);
                  getmean2.f90:2-195 (ider = 0: derivative tables)
  materials       getmat.f90:2-37, input.f90:19-43 (incl. Te = T0 quirk)
  derivative mat  chebyd.f90:2-60 (CHEBYD, brute-force Lagrange form)
  temporal        temporal.f90:88-890
  spatial         spatial.f90:89-1126 (curve = 0, and curve = 2 with circh.f90)
  PIKSR2          stable ascending sort carrying an index
  getevec         getevec.f90:154-227 (selection, real-scale quirk, format)
  makename        mtemporal.f90:53-76
  sweep drivers   mtemporal.f90:25-39, mspatial.f90:29-96 (loops, delta.dat)
  post-processors getab.f90:161-201, getax.f90:161-201, getalpha.f90:120-146

Parity pins: ``tests/test_oracle_golden.py`` checks this restatement against
the reference's golden files (test/space.1, TStest/README.md,
thesis/TStest/{time,space}.ref), through the fixtures in ``tests/golden``.
"""
from __future__ import annotations

import dataclasses
import math
import struct
from typing import Optional

import numpy as np

# Physical constants of module `stuff` (stuff.f90:43-45); with
# -fdefault-real-8 every default-real literal is binary64.
GAMMA = 1.4
GAMMA1 = 0.4
CP = 1003.1
PT66 = 6.6666666666666666666e-1
PI = 3.1415926535897932385
NDOF = 5
BIG = 1.0e98


@dataclasses.dataclass
class StabParams:
    """Mirror of the run parameters the reference keeps in module `stuff`
    (stuff.f90:11-55), filled the way input.f90:15-81 fills them."""

    mattyp: int = 0
    T0: float = 0.0
    Ma: float = 0.3
    Re: float = 1000.0
    Pr: float = 1.0
    ny: int = 32
    yi: float = 1.0
    ymax: float = 0.0
    ievec: int = 1
    ider: int = 1
    top: int = 0
    wall: int = 0
    wallt: int = 0
    curve: int = 0
    itype: int = 1
    alpha: complex = 0j
    beta: complex = 0j
    omega: complex = 0j
    ind: int = 0
    x: float = 0.0

    # --- derived quantities (input.f90:19-43) -------------------------
    def datmat(self):
        if self.mattyp == 1:
            return (1.715336725523065e-05, 273.0, 110.4)
        return (1.0, 0.0, 0.0)

    def Te(self) -> float:
        # input.f90:25 evaluates te = t0/(1+0.5*gamma1*Ma**2) BEFORE Ma is
        # read (Ma is still 0), so Te == T0 for Sutherland; for constant mu
        # te is never assigned and stays 0.
        if self.mattyp == 1:
            return self.T0 / (1.0 + 0.5 * GAMMA1 * 0.0 ** 2)
        return 0.0

    def navier(self) -> bool:
        # temporal.f90:88-91, spatial.f90:91-94
        return not (self.Re >= BIG or self.Re == 0.0)


# ---------------------------------------------------------------------------
# input.dat (stdin protocol, input.f90:15-81 and stab.f90:46-55)
# ---------------------------------------------------------------------------
def _fields(line: str):
    """List-directed read: leading values of the line, stop at '!'."""
    line = line.split("!")[0].replace(",", " ")
    return line.split()


def parse_input(text: str) -> StabParams:
    lines = [ln for ln in text.splitlines()]
    it = iter(lines)

    def nxt():
        while True:
            ln = next(it)
            f = _fields(ln)
            if f:
                return f

    p = StabParams()
    p.mattyp = int(nxt()[0])
    if p.mattyp == 1:
        p.T0 = float(nxt()[0])
    f = nxt()
    p.Ma, p.Re, p.Pr = float(f[0]), float(f[1]), float(f[2])
    f = nxt()
    p.ny, p.yi, p.ymax = int(f[0]), float(f[1]), float(f[2])
    p.ievec = int(nxt()[0])
    p.ider = int(nxt()[0])
    f = nxt()
    p.top, p.wall, p.wallt, p.curve = (int(v) for v in f[:4])
    p.itype = int(nxt()[0])
    f = nxt()
    a = complex(float(f[0]), float(f[1]))
    f = nxt()
    b = complex(float(f[0]), float(f[1]))
    if p.itype == 1:
        p.alpha, p.beta = a, b
    elif p.itype == 2:
        p.omega, p.beta = a, b
    else:
        raise ValueError(f"itype {p.itype} is outside the Chebyshev path")
    p.ind = int(nxt()[0])
    if p.itype == 2:
        try:
            p.x = float(nxt()[0])
        except StopIteration:
            p.x = 0.0
    return p


def makename(base: str, iver: int) -> str:
    """mtemporal.f90:53-76 / getevec.f90:236-254: base + '.' + digits."""
    if iver < 0 or iver >= 10000:
        raise ValueError("iver out of range")
    return f"{base}.{iver}"


# ---------------------------------------------------------------------------
# grid, profile, materials, derivative matrices
# ---------------------------------------------------------------------------
def sgengrid(ny: int, yi: float, ymax: float):
    """sgengrid.f90:2-45 (algebraic maps).  Returns y, eta, deta, d2eta."""
    dth = PI / float(ny - 1)
    eta = np.cos(np.arange(ny, dtype=np.float64) * dth)
    if yi == 0.0:
        raise ValueError("tanh map (Yi = 0) is interactive in the reference; not supported")
    if ymax == 0.0:  # infinite domain
        L = yi
        deta = (eta - 1.0) ** 2 / (2.0 * L)
        d2eta = (eta - 1.0) ** 3 / (2.0 * L ** 2)
        with np.errstate(divide="ignore"):
            y = np.where(eta != 1.0, L * (1.0 + eta) / np.where(eta != 1.0, 1.0 - eta, 1.0), 1.0e99)
    else:  # Streett map
        y = ymax * yi * (1.0 + eta) / (1.0 + 2.0 * yi - eta)
        deta = (2.0 * yi + 1.0 - eta) ** 2 / (2.0 * ymax * yi * (yi + 1.0))
        d2eta = -0.5 * (2.0 * yi + 1.0 - eta) ** 3 / (ymax * yi * (yi + 1.0)) ** 2
    return y, eta, deta, d2eta


def read_profile(path: str):
    """getmean.f90:40-80: rows 'y rho u v w T', lines starting '#' skipped,
    v forced to zero.  Returns ym (nym,), vt (nym, 5)."""
    rows = []
    with open(path) as fh:
        for ln in fh:
            if ln[:1] == "#":
                continue
            f = ln.replace(",", " ").split()
            if not f:
                continue
            rows.append([float(v) for v in f[:6]])
    a = np.asarray(rows, dtype=np.float64)
    ym = a[:, 0].copy()
    vt = a[:, 1:6].copy()
    vt[:, 2] = 0.0
    return ym, vt


def spline(x: np.ndarray, y: np.ndarray) -> np.ndarray:
    """SPLINE, spline.f90:2-49: second derivatives with the cantilever end
    condition (lambda = 1, FDP(1)=FDP(2), FDP(N)=FDP(N-1)); direct
    tridiagonal elimination.  Works on a trailing axis of fields."""
    n = x.shape[0]
    y = np.asarray(y, dtype=np.float64)
    if y.ndim == 1:
        return spline(x, y[:, None])[:, 0]
    c = np.zeros(n)
    a = np.zeros(n)
    b = np.zeros(n)
    r = np.zeros((n, y.shape[1]))
    c[0] = x[1] - x[0]
    for i in range(1, n - 1):
        c[i] = x[i + 1] - x[i]
        a[i] = c[i - 1]
        b[i] = 2.0 * (a[i] + c[i])
        r[i] = 6.0 * ((y[i + 1] - y[i]) / c[i] - (y[i] - y[i - 1]) / c[i - 1])
    b[1] = b[1] + 1.0 * c[0]
    b[n - 2] = b[n - 2] + 1.0 * c[n - 2]
    for i in range(2, n - 1):
        t = a[i] / b[i - 1]
        b[i] = b[i] - t * c[i - 1]
        r[i] = r[i] - t * r[i - 1]
    fdp = np.zeros_like(r)
    fdp[n - 2] = r[n - 2] / b[n - 2]
    # back substitution FDP(NMI) = (R(NMI) - C(NMI)*FDP(NMI+1))/B(NMI), NMI = N-I, I=2..N-2
    for I in range(2, n - 1):
        nmi = n - I  # 1-based
        k = nmi - 1
        fdp[k] = (r[k] - c[k] * fdp[k + 1]) / b[k]
    fdp[0] = 1.0 * fdp[1]
    fdp[n - 1] = 1.0 * fdp[n - 2]
    return fdp


def speval(x, y, fdp, xx):
    """SPEVAL, spline.f90:52-75, with its linear interval scan (first I with
    XX <= X(I+1); falls through to the last interval)."""
    n = x.shape[0]
    i = int(np.searchsorted(x[1:], xx, side="left"))  # first i with xx <= x[i+1]
    if i > n - 2:
        i = n - 2
    dxm = xx - x[i]
    dxp = x[i + 1] - xx
    de = x[i + 1] - x[i]
    return (fdp[i] * dxp * (dxp * dxp / de - de) / 6.0
            + fdp[i + 1] * dxm * (dxm * dxm / de - de) / 6.0
            + y[i] * dxp / de + y[i + 1] * dxm / de)


def getmean(ym: np.ndarray, vt: np.ndarray, y: np.ndarray) -> np.ndarray:
    """getmean.f90:82-112: spline each field, evaluate at y, clamp to the last
    profile row above the profile's y range.  Returns vm (ny, 5)."""
    fdp = spline(ym, vt)
    ymaxm = ym[-1]
    vm = np.zeros((y.shape[0], NDOF))
    for j, yy in enumerate(y):
        if yy <= ymaxm:
            vm[j] = speval(ym, vt, fdp, yy)
        else:
            vm[j] = vt[-1]
    return vm


def getmean2(ym, vt, first, second, y):
    """getmean2.f90:24-175 (ider = 0): the mean field as getmean, and its
    first and second y-derivatives from their own tables (rows y f1..f5, the
    mean's row count, v forced to zero), splined on the tables' own y and
    clamped to each table's last row where y exceeds the MEAN profile's last
    y (ymaxm is taken before the derivative reads overwrite ym).
    Returns vm, g2vm, g22vm (ny, 5)."""
    vm = getmean(ym, vt, y)
    ymaxm = ym[-1]
    out = []
    for tab in (first, second):
        ty = np.asarray(tab[:, 0], dtype=np.float64)
        tv = np.asarray(tab[:, 1:6], dtype=np.float64).copy()
        tv[:, 2] = 0.0
        fdp = spline(ty, tv)
        g = np.zeros((y.shape[0], NDOF))
        for j, yy in enumerate(y):
            g[j] = speval(ty, tv, fdp, yy) if yy <= ymaxm else tv[-1]
        out.append(g)
    return vm, out[0], out[1]


def getmat(t, p: StabParams):
    """getmat.f90:2-37.  Returns (rmu, rlm, con, dmu, d2mu, dlm, d2lm, dcon, d2con)."""
    c0, c1, c2 = p.datmat()
    t = np.asarray(t, dtype=np.float64)
    if p.mattyp == 0:
        rmu = np.full_like(t, c0)
        dmu = np.zeros_like(t)
        d2mu = np.zeros_like(t)
    else:
        rmu = c0 * t / c1 * np.sqrt(t / c1) * (c1 + c2) / (t + c2)
        dmu = (c0 * (3.0 * c2 + t) * (c2 + c1) * np.sqrt(t / c1)) / (2.0 * (c2 + t) ** 2 * c1)
        d2mu = (c0 * (3.0 * c2 ** 2 - 6.0 * c2 * t - t ** 2) * (c2 + c1)) / (
            4.0 * (c2 + t) ** 3 * np.sqrt(t / c1) * c1 ** 2)
    con = rmu * CP / p.Pr
    dcon = dmu * CP / p.Pr
    d2con = d2mu * CP / p.Pr
    rlm = -PT66 * rmu
    dlm = -PT66 * dmu
    d2lm = -PT66 * d2mu
    return rmu, rlm, con, dmu, d2mu, dlm, d2lm, dcon, d2con


def chebyd(N: int) -> np.ndarray:
    """CHEBYD, chebyd.f90:2-60: (N+1)x(N+1) derivative matrix on the
    Gauss-Lobatto points, brute-force Lagrange form."""
    pi = math.acos(-1.0)
    x = np.cos(pi * np.arange(N + 1, dtype=np.float64) / float(N))
    diff = x[:, None] - x[None, :]
    np.fill_diagonal(diff, 1.0)
    a = np.prod(diff, axis=1)
    D = a[:, None] / (a[None, :] * diff)
    inv = 1.0 / diff
    np.fill_diagonal(inv, 0.0)
    np.fill_diagonal(D, inv.sum(axis=1))
    return D


# ---------------------------------------------------------------------------
# mean-flow preparation shared by temporal and spatial
# ---------------------------------------------------------------------------
@dataclasses.dataclass
class MeanState:
    y: np.ndarray
    eta: np.ndarray
    deta: np.ndarray
    d2eta: np.ndarray
    D1: np.ndarray
    D2: np.ndarray
    Dt1: np.ndarray
    Dt2: np.ndarray
    vm: np.ndarray
    g2vm: np.ndarray
    g22vm: np.ndarray


def mean_state(p: StabParams, ym: np.ndarray, vt: np.ndarray, first=None, second=None) -> MeanState:
    """Grid + mean flow + derivative matrices + mapped mean derivatives
    (temporal.f90:95-179, spatial.f90:96-163).  With p.ider == 0 the mean
    derivatives come from the tables `first` and `second` (getmean2) and
    skip the collocation derivatives and the chain rule
    (temporal.f90:149-179)."""
    ny = p.ny
    y, eta, deta, d2eta = sgengrid(ny, p.yi, p.ymax)
    if not p.ider:
        vm, g2, g22 = getmean2(ym, vt, first, second, y)
    else:
        vm = getmean(ym, vt, y)
    D1 = chebyd(ny - 1)
    D2 = D1 @ D1
    if p.wallt == 2:
        Dt1 = D1.copy()
        Dt1[ny - 1, :] = 0.0
        Dt2 = D1 @ Dt1
    else:
        Dt1, Dt2 = D1, D2
    if p.ider:
        g2 = D1 @ vm
        g22 = D2 @ vm
        g22 = g22 * (deta ** 2)[:, None] + g2 * d2eta[:, None]
        g2 = g2 * deta[:, None]
    return MeanState(y, eta, deta, d2eta, D1, D2, Dt1, Dt2, vm, g2, g22)


def _materials(p: StabParams, tm: np.ndarray):
    """Nondimensional mean properties (temporal.f90:262-277)."""
    Te = p.Te()
    rmue, rlme, cone, *_ = getmat(np.array([Te]), p)
    rmue, rlme, cone = float(rmue[0]), float(rlme[0]), float(cone[0])
    rmu, rlm, con, dmu, d2mu, dlm, d2lm, dcon, d2con = getmat(tm * Te, p)
    rmu = rmu / rmue
    dmu = dmu * Te / rmue
    d2mu = d2mu * Te ** 2 / rmue
    con = con / cone
    dcon = dcon * Te / cone
    d2con = d2con * Te ** 2 / cone
    rlm = rlm / rlme
    dlm = dlm * Te / rlme
    d2lm = d2lm * Te ** 2 / rlme
    return dict(rmue=rmue, rlme=rlme, cone=cone, rmu=rmu, rlm=rlm, con=con, dmu=dmu,
                d2mu=d2mu, dlm=dlm, d2lm=d2lm, dcon=dcon, d2con=d2con)


BLOCK_NAMES = ("G", "A", "B", "C", "D", "Vxx", "Vxy", "Vyy", "Vxz", "Vyz", "Vzz")


def _zero_blocks(ny):
    return {k: np.zeros((ny, NDOF, NDOF)) for k in BLOCK_NAMES}


def temporal_blocks(p: StabParams, ms: MeanState):
    """The eleven real 5x5 coefficient blocks per node of the temporal
    operator, temporal.f90:193-598.  Index convention [node, eq, var]."""
    ny = p.ny
    vm = ms.vm
    z = np.zeros(ny)
    rhom, u1m, u2m, u3m, tm = (vm[:, k] for k in range(5))
    # g1 and g3 derivatives of the mean vanish for a parallel flow;
    # the second-derivative tensors g11..g33 are zero except g22.
    g1vm = np.zeros((ny, 5))
    g3vm = np.zeros((ny, 5))
    g2vm = ms.g2vm
    g22vm = ms.g22vm
    g11vm = g12vm = g13vm = g21vm = g23vm = g31vm = g32vm = g33vm = np.zeros((ny, 5))
    gum = np.zeros((ny, 3, 3))
    for i, k in enumerate((1, 2, 3)):
        gum[:, i, 0] = g1vm[:, k]
        gum[:, i, 1] = g2vm[:, k]
        gum[:, i, 2] = g3vm[:, k]
    divum = gum[:, 0, 0] + gum[:, 1, 1] + gum[:, 2, 2]
    grhom = np.stack([g1vm[:, 0], g2vm[:, 0], g3vm[:, 0]], axis=1)
    gtm = np.stack([g1vm[:, 4], g2vm[:, 4], g3vm[:, 4]], axis=1)
    fact = 1.0 / (GAMMA * p.Ma ** 2)
    gpm = fact * (grhom * tm[:, None] + rhom[:, None] * gtm)
    g1divum = g11vm[:, 1] + g12vm[:, 2]
    g2divum = g12vm[:, 1] + g22vm[:, 2]
    g3divum = z
    S = 0.5 * (gum + np.transpose(gum, (0, 2, 1)))
    S1jj = 0.5 * (g11vm[:, 1] + g11vm[:, 1] + g22vm[:, 1] + g12vm[:, 2] + g33vm[:, 1] + g13vm[:, 3])
    S2jj = 0.5 * (g11vm[:, 2] + g21vm[:, 1] + g22vm[:, 2] + g22vm[:, 2] + g33vm[:, 2] + g23vm[:, 3])
    S3jj = 0.5 * (g11vm[:, 3] + g31vm[:, 1] + g22vm[:, 3] + g32vm[:, 2] + g33vm[:, 3] + g33vm[:, 3])
    m = _materials(p, tm)
    rmu, rlm, con = m["rmu"], m["rlm"], m["con"]
    dmu, d2mu, dlm, d2lm, dcon, d2con = m["dmu"], m["d2mu"], m["dlm"], m["d2lm"], m["dcon"], m["d2con"]
    g1mu, g2mu, g3mu = (dmu * gtm[:, k] for k in range(3))
    g1dmu, g2dmu, g3dmu = (d2mu * gtm[:, k] for k in range(3))
    g1con, g2con, g3con = (dcon * gtm[:, k] for k in range(3))
    g1dcon, g2dcon, g3dcon = (d2con * gtm[:, k] for k in range(3))
    g1lm, g2lm, g3lm = (dlm * gtm[:, k] for k in range(3))
    g1dlm, g2dlm, g3dlm = (d2lm * gtm[:, k] for k in range(3))
    rlme, rmue = m["rlme"], m["rmue"]
    ig = 1.0 / (GAMMA * p.Ma ** 2)
    nav = p.navier()
    Re, Pr, Ma = p.Re, p.Pr, p.Ma

    bl = _zero_blocks(ny)
    G, A, B, C, D = bl["G"], bl["A"], bl["B"], bl["C"], bl["D"]
    Vxx, Vxy, Vyy, Vxz, Vyz, Vzz = (bl[k] for k in ("Vxx", "Vxy", "Vyy", "Vxz", "Vyz", "Vzz"))

    # continuity (temporal.f90:313-327)
    G[:, 0, 0] = 1.0
    A[:, 0, 0] = u1m; A[:, 0, 1] = rhom
    B[:, 0, 0] = u2m; B[:, 0, 2] = rhom
    C[:, 0, 0] = u3m; C[:, 0, 3] = rhom
    D[:, 0, 0] = divum; D[:, 0, 1] = grhom[:, 0]; D[:, 0, 2] = grhom[:, 1]; D[:, 0, 3] = grhom[:, 2]

    # three momentum equations (temporal.f90:331-526); e = equation row,
    # c = the velocity component that carries the pressure gradient
    for e in (1, 2, 3):
        c = e - 1  # spatial direction of this momentum equation
        G[:, e, e] = rhom
        A[:, e, e] = rhom * u1m
        B[:, e, e] = rhom * u2m
        C[:, e, e] = rhom * u3m
        P = (A, B, C)[c]
        P[:, e, 0] = tm * ig
        P[:, e, 4] = rhom * ig
        D[:, e, 0] = u1m * gum[:, c, 0] + u2m * gum[:, c, 1] + u3m * gum[:, c, 2] + gtm[:, c] * ig
        D[:, e, 1] = rhom * gum[:, c, 0]
        D[:, e, 2] = rhom * gum[:, c, 1]
        D[:, e, 3] = rhom * gum[:, c, 2]
        D[:, e, 4] = grhom[:, c] * ig
    if nav:
        # x momentum, lambda then mu (temporal.f90:347-394)
        f = rlme / (rmue * Re)
        A[:, 1, 1] -= f * g1lm
        A[:, 1, 4] -= f * dlm * divum
        B[:, 1, 2] -= f * g1lm
        C[:, 1, 3] -= f * g1lm
        D[:, 1, 4] -= f * (g1dlm * divum + dlm * g1divum)
        Vxx[:, 1, 1] = f * rlm
        Vxy[:, 1, 2] = f * rlm
        Vxz[:, 1, 3] = f * rlm
        f = 1.0 / Re
        A[:, 1, 1] -= f * 2.0 * g1mu
        A[:, 1, 2] -= f * g2mu
        A[:, 1, 3] -= f * g3mu
        A[:, 1, 4] -= f * dmu * 2.0 * S[:, 0, 0]
        B[:, 1, 1] -= f * g2mu
        B[:, 1, 4] -= f * dmu * 2.0 * S[:, 0, 1]
        C[:, 1, 1] -= f * g3mu
        C[:, 1, 4] -= f * dmu * 2.0 * S[:, 0, 2]
        D[:, 1, 4] -= f * 2.0 * (g1dmu * S[:, 0, 0] + g2dmu * S[:, 0, 1] + g3dmu * S[:, 0, 2] + dmu * S1jj)
        Vxx[:, 1, 1] += f * 2.0 * rmu
        Vxy[:, 1, 2] += f * rmu
        Vyy[:, 1, 1] += f * rmu
        Vxz[:, 1, 3] += f * rmu
        Vzz[:, 1, 1] += f * rmu
        # y momentum (temporal.f90:418-459)
        f = rlme / (rmue * Re)
        A[:, 2, 1] -= f * g2lm
        B[:, 2, 2] -= f * g2lm
        B[:, 2, 4] -= f * dlm * divum
        C[:, 2, 3] -= f * g2lm
        D[:, 2, 4] -= f * (g2dlm * divum + dlm * g2divum)
        Vxy[:, 2, 1] = f * rlm
        Vyy[:, 2, 2] = f * rlm
        Vyz[:, 2, 3] = f * rlm
        f = 1.0 / Re
        A[:, 2, 2] -= f * g1mu
        A[:, 2, 4] -= f * dmu * 2.0 * S[:, 1, 0]
        B[:, 2, 1] -= f * g1mu
        B[:, 2, 2] -= f * 2.0 * g2mu
        B[:, 2, 3] -= f * g3mu
        B[:, 2, 4] -= f * dmu * 2.0 * S[:, 1, 1]
        C[:, 2, 2] -= f * g3mu
        C[:, 2, 4] -= f * dmu * 2.0 * S[:, 1, 2]
        D[:, 2, 4] -= f * 2.0 * (g1dmu * S[:, 1, 0] + g2dmu * S[:, 1, 1] + g3dmu * S[:, 1, 2] + dmu * S2jj)
        Vxx[:, 2, 2] += f * rmu
        Vxy[:, 2, 1] += f * rmu
        Vyy[:, 2, 2] += f * 2.0 * rmu
        Vyz[:, 2, 3] += f * rmu
        Vzz[:, 2, 2] += f * rmu
        # z momentum (temporal.f90:483-524)
        f = rlme / (rmue * Re)
        A[:, 3, 1] -= f * g3lm
        B[:, 3, 2] -= f * g3lm
        C[:, 3, 3] -= f * g3lm
        C[:, 3, 4] -= f * dlm * divum
        D[:, 3, 4] -= f * (g3dlm * divum + dlm * g3divum)
        Vxz[:, 3, 1] = f * rlm
        Vyz[:, 3, 2] = f * rlm
        Vzz[:, 3, 3] = f * rlm
        f = 1.0 / Re
        A[:, 3, 3] -= f * g1mu
        A[:, 3, 4] -= f * dmu * 2.0 * S[:, 2, 0]
        B[:, 3, 3] -= f * g2mu
        B[:, 3, 4] -= f * dmu * 2.0 * S[:, 2, 1]
        C[:, 3, 1] -= f * g1mu
        C[:, 3, 2] -= f * g2mu
        C[:, 3, 3] -= f * 2.0 * g3mu
        C[:, 3, 4] -= f * dmu * 2.0 * S[:, 2, 2]
        D[:, 3, 4] -= f * 2.0 * (g1dmu * S[:, 2, 0] + g2dmu * S[:, 2, 1] + g3dmu * S[:, 2, 2] + dmu * S3jj)
        Vxx[:, 3, 3] += f * rmu
        Vyy[:, 3, 3] += f * rmu
        Vxz[:, 3, 1] += f * rmu
        Vyz[:, 3, 2] += f * rmu
        Vzz[:, 3, 3] += f * 2.0 * rmu

    # energy (temporal.f90:530-598)
    G[:, 4, 0] = -GAMMA1 * tm / GAMMA
    G[:, 4, 4] = rhom / GAMMA
    A[:, 4, 0] = -GAMMA1 * u1m * tm / GAMMA
    A[:, 4, 4] = rhom * u1m / GAMMA
    B[:, 4, 0] = -GAMMA1 * u2m * tm / GAMMA
    B[:, 4, 4] = rhom * u2m / GAMMA
    C[:, 4, 0] = -GAMMA1 * u3m * tm / GAMMA
    C[:, 4, 4] = rhom * u3m / GAMMA
    D[:, 4, 0] = 1.0 / GAMMA * (u1m * gtm[:, 0] + u2m * gtm[:, 1] + u3m * gtm[:, 2])
    D[:, 4, 1] = rhom * gtm[:, 0] - GAMMA1 * Ma ** 2 * gpm[:, 0]
    D[:, 4, 2] = rhom * gtm[:, 1] - GAMMA1 * Ma ** 2 * gpm[:, 1]
    D[:, 4, 3] = rhom * gtm[:, 2] - GAMMA1 * Ma ** 2 * gpm[:, 2]
    D[:, 4, 4] = -GAMMA1 / GAMMA * (u1m * grhom[:, 0] + u2m * grhom[:, 1] + u3m * grhom[:, 2])
    if nav:
        f = 1.0 / (Pr * Re)
        A[:, 4, 4] -= f * (g1con + dcon * gtm[:, 0])
        B[:, 4, 4] -= f * (g2con + dcon * gtm[:, 1])
        C[:, 4, 4] -= f * (g3con + dcon * gtm[:, 2])
        D[:, 4, 4] -= f * (g1dcon * gtm[:, 0] + g2dcon * gtm[:, 1] + g3dcon * gtm[:, 2]
                           + dcon * (g11vm[:, 4] + g22vm[:, 4] + g33vm[:, 4]))
        Vxx[:, 4, 4] = f * con
        Vyy[:, 4, 4] = f * con
        Vzz[:, 4, 4] = f * con
        f = GAMMA1 * Ma ** 2 * rlme / (Re * rmue)
        A[:, 4, 1] -= f * 2.0 * rlm * divum
        B[:, 4, 2] -= f * 2.0 * rlm * divum
        C[:, 4, 3] -= f * 2.0 * rlm * divum
        D[:, 4, 4] -= f * dlm * divum * divum
        f = 2.0 * GAMMA1 * Ma ** 2 / Re
        for c in range(3):
            A[:, 4, 1 + c] -= f * 2.0 * rmu * S[:, c, 0]
            B[:, 4, 1 + c] -= f * 2.0 * rmu * S[:, c, 1]
            C[:, 4, 1 + c] -= f * 2.0 * rmu * S[:, c, 2]
        D[:, 4, 4] -= f * dmu * (S ** 2).sum(axis=(1, 2))
    return bl


INFTY = 1.0e30


def circh_scalars(s: float):
    """The station-independent part of circh (circh.f90:2-188, with xcloc and
    ycloc, :201-229): the wall of a circle of radius s (the caller's x),
    evaluated at arc position 0.  Returns dxbds, dybds, dbn1, dbn2, d2xbds2,
    d2ybds2, d2bn1, d2bn2 (the tangent, the normal's arc derivative and the
    second arc derivatives), from which circh_metrics forms h and its
    derivatives at distance r from the wall.  circh also sets its argument
    (the module's x) to zero (circh.f90:60)."""
    radius = s
    # xcloc(0, 0): th1 = atan2(sqrt(R^2 - x1^2), x1), xl = R cos(th1 - ds)
    th1 = math.atan2(math.sqrt(radius ** 2 - 0.0 ** 2), 0.0)
    xl = radius * math.cos(th1 - 0.0)
    yl = math.sqrt(radius ** 2 - xl ** 2)            # ycloc(xl)
    th = math.atan2(-xl, math.sqrt(radius ** 2 - xl ** 2))
    bn1 = -math.sin(th)
    bn2 = math.cos(th)
    dydx = -INFTY if xl == 0.0 else (-xl) / yl
    dxbds = 1.0 / math.sqrt(1.0 + dydx ** 2)
    dxdy = -INFTY if xl == 0.0 else yl / (-xl)
    dybds = 1.0 / math.sqrt(dxdy ** 2 + 1.0) if xl <= 0.0 else -1.0 / math.sqrt(dxdy ** 2 + 1.0)
    if yl == 0.0:
        dx, dy = 0.0, -xl
        ddxdx, ddydx, ddxdy, ddydy = -INFTY, -1.0, 1.0, 0.0
        d2dxdx2, d2dydx2, d2dxdy2, d2dydy2 = -INFTY, 0.0, 0.0, (xl ** 2 + yl ** 2) / xl ** 3
    elif xl == 0.0:
        dx, dy = yl, 0.0
        ddxdx, ddydx, ddxdy, ddydy = 0.0, -1.0, 1.0, INFTY
        d2dxdx2, d2dydx2, d2dxdy2, d2dydy2 = -(yl ** 2 + xl ** 2) / yl ** 3, 0.0, 0.0, INFTY
    else:
        dx, dy = yl, -xl
        ddxdx, ddydx, ddxdy, ddydy = -xl / yl, -1.0, 1.0, yl / xl
        d2dxdx2, d2dydx2, d2dxdy2, d2dydy2 = (-(yl ** 2 + xl ** 2) / yl ** 3, 0.0, 0.0,
                                              (xl ** 2 + yl ** 2) / xl ** 3)
    q = dx ** 2 + dy ** 2
    if abs(bn1) > abs(bn2):
        dbn1 = (-ddydy / q ** 0.5 + 0.5 * dy * (2.0 * dx * ddxdy + 2.0 * dy * ddydy) / q ** 1.5) * dybds
        dbn2 = (ddxdy / q ** 0.5 - 0.5 * dx * (2.0 * dx * ddxdy + 2.0 * dy * ddydy) / q ** 1.5) * dybds
    else:
        dbn1 = (-ddydx / q ** 0.5 + 0.5 * dy * (2.0 * dx * ddxdx + 2.0 * dy * ddydx) / q ** 1.5) * dxbds
        dbn2 = (ddxdx / q ** 0.5 - 0.5 * dx * (2.0 * dx * ddxdx + 2.0 * dy * ddydx) / q ** 1.5) * dxbds
    if abs(bn1) > abs(bn2):
        d2xdy2 = -(xl ** 2 + yl ** 2) / xl ** 3
        if xl <= 0:
            d2ybds2 = -(1.0 + dxdy ** 2) ** (-1.5) * dxdy * d2xdy2 * dybds
        else:
            d2ybds2 = (1.0 + dxdy ** 2) ** (-1.5) * dxdy * d2xdy2 * dybds
        d2xbds2 = d2xdy2 * dybds ** 2 + dxdy * d2ybds2
    else:
        d2ydx2 = -(xl ** 2 + yl ** 2) / yl ** 3
        d2xbds2 = -(1.0 + dydx ** 2) ** (-1.5) * dydx * d2ydx2 * dxbds
        d2ybds2 = d2ydx2 * dxbds ** 2 + dydx * d2xbds2
    if abs(bn1) > abs(bn2):
        t1 = dy * ddxdy - dx * ddydy
        t2 = dx * ddxdy + dy * ddydy
        d2bn1 = (((ddxdy * t1 + dx * (dy * d2dxdy2 - dx * d2dydy2)) / q ** 1.5
                  - (3.0 * dx * t1 * t2) / q ** 2.5) * dybds ** 2
                 + (-ddydy / q ** 0.5 + 0.5 * dy * (2.0 * dx * ddxdy + 2.0 * dy * ddydy) / q ** 1.5) * d2ybds2)
        d2bn2 = (((ddydy * t1 + dy * (dy * d2dxdy2 - dx * d2dydy2)) / q ** 1.5
                  - (3.0 * dy * t1 * t2) / q ** 2.5) * dybds ** 2
                 + (ddxdy / q ** 0.5 - 0.5 * dx * (2.0 * dx * ddxdy + 2.0 * dy * ddydy) / q ** 1.5) * d2ybds2)
    else:
        t1 = dy * ddxdx - dx * ddydx
        t2 = dx * ddxdx + dy * ddydx
        d2bn1 = (((ddxdx * t1 + dx * (dy * d2dxdx2 - dx * d2dydx2)) / q ** 1.5
                  - (3.0 * dx * t1 * t2) / q ** 2.5) * dxbds ** 2
                 + (-ddydx / q ** 0.5 + 0.5 * dy * (2.0 * dx * ddxdx + 2.0 * dy * ddydx) / q ** 1.5) * d2xbds2)
        d2bn2 = (((ddydx * t1 + dy * (dy * d2dxdx2 - dx * d2dydx2)) / q ** 1.5
                  - (3.0 * dy * t1 * t2) / q ** 2.5) * dxbds ** 2
                 + (ddxdx / q ** 0.5 - 0.5 * dx * (2.0 * dx * ddxdx + 2.0 * dy * ddydx) / q ** 1.5) * d2xbds2)
    if xl == 0.0:
        d2bn1 = 0.0
    return dxbds, dybds, dbn1, dbn2, d2xbds2, d2ybds2, d2bn1, d2bn2


def parabola_arc(x1: float, x2: float) -> float:
    """Arc length of the parabolic cylinder y = sqrt(2 x) from x1 to x2
    (calch.f90, function arc)."""
    def f(x):
        xi = math.sqrt(x)
        t = math.sqrt(1.0 + 2.0 * xi ** 2)
        return math.sqrt(2.0) * 0.5 * xi * t + 0.5 * math.log(math.sqrt(2.0) * xi + t)
    return f(x2) - f(x1)


def false_position(func, x1: float, x2: float, xacc: float, maxit: int = 30) -> float:
    """Root of func in [x1, x2] by the method of false position as published
    in Numerical Recipes (Press, Teukolsky, Vetterling, Flannery, 2nd ed.
    1992, section 9.2, routine rtflsp), which calch.f90's xloc calls and the
    reference does not ship: keep the endpoint with func < 0 and the one with
    func >= 0, replace the one on the side of the secant root, stop when the
    replaced endpoint moved less than xacc or func is exactly zero, and give
    up after maxit (30) secant steps.  Raises ValueError where that routine
    stops the program (no bracket, no convergence)."""
    fl, fh = func(x1), func(x2)
    if fl * fh > 0.0:
        raise ValueError("false position: root not bracketed")
    if fl < 0.0:
        lo, hi = x1, x2
    else:
        lo, hi = x2, x1
        fl, fh = fh, fl
    for _ in range(maxit):
        if fl == fh:
            raise ValueError("false position: flat secant")
        x = lo + (hi - lo) * fl / (fl - fh)
        f = func(x)
        if f < 0.0:
            moved = lo - x
            lo, fl = x, f
        else:
            moved = hi - x
            hi, fh = x, f
        if abs(moved) < xacc or f == 0.0:
            return x
    raise ValueError("false position: no convergence in %d steps" % maxit)


def calch_scalars(s: float):
    """The station-independent part of calch (calch.f90:31-148): the wall of
    the parabolic cylinder y = sqrt(2 x), at the point whose arc length from
    the nose is s (the caller's x), located by xloc (calch.f90:170-184) with
    false position on [0, 2 s] to 1e-12.  Returns the same eight scalars as
    circh_scalars; circh_metrics (the same closing formulas, calch.f90:
    152-167) forms h and its derivatives from them."""
    xl = false_position(lambda x: s - parabola_arc(0.0, x), 0.0, 0.0 + 2.0 * s, 1.0e-12)
    yl = math.sqrt(2.0 * xl)
    th = math.atan2(1.0, yl)
    bn1 = -math.sin(th)
    bn2 = math.cos(th)
    dydx = INFTY if xl == 0.0 else 1.0 / math.sqrt(2.0 * xl)
    dxbds = 1.0 / math.sqrt(1.0 + dydx ** 2)
    dxdy = 0.0 if xl == 0.0 else math.sqrt(2.0 * xl)
    dybds = 1.0 / math.sqrt(dxdy ** 2 + 1.0)
    if xl == 0.0:
        dx, dy = 0.0, 1.0
        ddxdx, ddydx, ddxdy, ddydy = INFTY, 0.0, 1.0, 0.0
        d2dxdx2 = INFTY
    else:
        dx, dy = yl, 1.0
        ddxdx, ddydx, ddxdy, ddydy = 1.0 / yl, 0.0, 1.0, 0.0
        d2dxdx2 = -math.sqrt(2.0) / (2.0 ** 2 * xl ** 1.5)
    d2dydx2 = d2dxdy2 = d2dydy2 = 0.0
    q = dx ** 2 + dy ** 2
    if abs(bn1) > abs(bn2):
        dbn1 = (-ddydy / q ** 0.5 + 0.5 * dy * (2.0 * dx * ddxdy + 2.0 * dy * ddydy) / q ** 1.5) * dybds
        dbn2 = (ddxdy / q ** 0.5 - 0.5 * dx * (2.0 * dx * ddxdy + 2.0 * dy * ddydy) / q ** 1.5) * dybds
        d2xdy2 = 1.0
        d2ybds2 = -(1.0 + dxdy ** 2) ** (-1.5) * dxdy * d2xdy2 * dybds
        d2xbds2 = d2xdy2 * dybds ** 2 + dxdy * d2ybds2
        t1 = dy * ddxdy - dx * ddydy
        t2 = dx * ddxdy + dy * ddydy
        d2bn1 = (((ddxdy * t1 + dx * (dy * d2dxdy2 - dx * d2dydy2)) / q ** 1.5
                  - (3.0 * dx * t1 * t2) / q ** 2.5) * dybds ** 2
                 + (-ddydy / q ** 0.5 + 0.5 * dy * (2.0 * dx * ddxdy + 2.0 * dy * ddydy) / q ** 1.5) * d2ybds2)
        d2bn2 = (((ddydy * t1 + dy * (dy * d2dxdy2 - dx * d2dydy2)) / q ** 1.5
                  - (3.0 * dy * t1 * t2) / q ** 2.5) * dybds ** 2
                 + (ddxdy / q ** 0.5 - 0.5 * dx * (2.0 * dx * ddxdy + 2.0 * dy * ddydy) / q ** 1.5) * d2ybds2)
    else:
        dbn1 = (-ddydx / q ** 0.5 + 0.5 * dy * (2.0 * dx * ddxdx + 2.0 * dy * ddydx) / q ** 1.5) * dxbds
        dbn2 = (ddxdx / q ** 0.5 - 0.5 * dx * (2.0 * dx * ddxdx + 2.0 * dy * ddydx) / q ** 1.5) * dxbds
        d2ydx2 = -1.0 / (2.0 * math.sqrt(2.0) * xl ** 1.5)
        d2xbds2 = -(1.0 + dydx ** 2) ** (-1.5) * dydx * d2ydx2 * dxbds
        d2ybds2 = d2ydx2 * dxbds ** 2 + dydx * d2xbds2
        t1 = dy * ddxdx - dx * ddydx
        t2 = dx * ddxdx + dy * ddydx
        d2bn1 = (((ddxdx * t1 + dx * (dy * d2dxdx2 - dx * d2dydx2)) / q ** 1.5
                  - (3.0 * dx * t1 * t2) / q ** 2.5) * dxbds ** 2
                 + (-ddydx / q ** 0.5 + 0.5 * dy * (2.0 * dx * ddxdx + 2.0 * dy * ddydx) / q ** 1.5) * d2xbds2)
        d2bn2 = (((ddydx * t1 + dy * (dy * d2dxdx2 - dx * d2dydx2)) / q ** 1.5
                  - (3.0 * dy * t1 * t2) / q ** 2.5) * dxbds ** 2
                 + (ddxdx / q ** 0.5 - 0.5 * dx * (2.0 * dx * ddxdx + 2.0 * dy * ddydx) / q ** 1.5) * d2xbds2)
    return dxbds, dybds, dbn1, dbn2, d2xbds2, d2ybds2, d2bn1, d2bn2


def circh_metrics(sc, r):
    """h, dh/ds, dh/dr, d2h/dsdr, d2h/dr2 at distances r from the wall
    (circh.f90:190-199) from the scalars of circh_scalars."""
    dxbds, dybds, dbn1, dbn2, d2xbds2, d2ybds2, d2bn1, d2bn2 = sc
    r = np.asarray(r, dtype=np.float64)
    a = dxbds + r * dbn1
    b = dybds + r * dbn2
    h = np.sqrt(a ** 2 + b ** 2)
    dads = d2xbds2 + r * d2bn1
    dbds = d2ybds2 + r * d2bn2
    dhds = (a * dads + b * dbds) / h
    dhdr = (a * dbn1 + b * dbn2) / h
    dhdrr = (-dhdr ** 2 + dbn1 ** 2 + dbn2 ** 2) / h
    dhdsr = -dhds / h ** 2 * (a * dbn1 + b * dbn2) + (dads * dbn1 + a * d2bn1 + dbds * dbn2 + b * d2bn2) / h
    return h, dhds, dhdr, dhdsr, dhdrr


def wall_metrics(p: StabParams, y):
    """The wall metrics of spatial.f90:110-125: curve = 1 the parabolic
    cylinder of calch at arc length x from its nose, curve = 2 a circle of
    radius x (circh), curve = 0 a flat wall (h = 1).  x = -1 turns the
    curvature off in both (calch.f90:31-39, circh.f90:46-53)."""
    ny = len(y)
    flat = (np.ones(ny), np.zeros(ny), np.zeros(ny), np.zeros(ny), np.zeros(ny))
    if p.curve == 0 or (p.curve in (1, 2) and p.x == -1.0):
        return flat
    if p.curve == 1:
        if not p.x > 0.0:
            raise ValueError("curve = 1 needs an arc length x > 0 (or -1)")
        return circh_metrics(calch_scalars(p.x), y)
    if p.curve == 2:
        return circh_metrics(circh_scalars(p.x), y)
    raise ValueError("curve must be 0, 1 or 2")


def spatial_blocks_curved(p: StabParams, ms: MeanState, met):
    """Coefficient blocks of the spatial operator on a curved wall,
    spatial.f90:230-673 term by term, with the metric h(y) of the wall and
    its derivatives (met = h, dhds, dhdr, dhdsr, dhdrr).  The parallel mean
    flow has u2m = 0 and no streamwise or spanwise gradients
    (spatial.f90:147, 167-185)."""
    h, dhds, dhdr, dhdsr, dhdrr = met
    ny = p.ny
    vm = ms.vm
    rhom, u1m, _, u3m, tm = (vm[:, k] for k in range(5))
    u2m = np.zeros(ny)
    z = np.zeros(ny)
    g2vm, g22vm = ms.g2vm, ms.g22vm
    g1vm = g3vm = np.zeros((ny, 5))
    g11vm = g12vm = g13vm = g23vm = g33vm = np.zeros((ny, 5))
    gum = np.zeros((ny, 3, 3))
    for i, k in enumerate((1, 2, 3)):
        gum[:, i, 0] = g1vm[:, k]
        gum[:, i, 1] = g2vm[:, k]
        gum[:, i, 2] = g3vm[:, k]
    divum = (gum[:, 0, 0] + u2m * dhdr) / h + gum[:, 1, 1] + gum[:, 2, 2]
    grhom = np.stack([g1vm[:, 0], g2vm[:, 0], g3vm[:, 0]], axis=1)
    gtm = np.stack([g1vm[:, 4], g2vm[:, 4], g3vm[:, 4]], axis=1)
    g1divum = (-dhds / h ** 3 * (gum[:, 0, 0] + u2m * dhdr)
               + 1.0 / h ** 2 * (g11vm[:, 1] + gum[:, 1, 0] * dhdr + u2m * dhdsr)
               + 1.0 / h * (g12vm[:, 2] + g13vm[:, 3]))
    g2divum = (-dhdr / h ** 2 * (gum[:, 0, 0] + u2m * dhdr)
               + 1.0 / h * (g12vm[:, 1] + gum[:, 1, 1] * dhdr + u2m * dhdrr) + (g22vm[:, 2] + g23vm[:, 3]))
    g3divum = 1.0 / h * (g13vm[:, 1] + gum[:, 1, 2] * dhdr) + g23vm[:, 2] + g33vm[:, 3]
    S = np.zeros((ny, 3, 3))
    S[:, 0, 0] = (gum[:, 0, 0] + u2m * dhdr) / h
    S[:, 0, 1] = 0.5 * ((gum[:, 1, 0] - u1m * dhdr) / h + gum[:, 0, 1])
    S[:, 0, 2] = 0.5 * (gum[:, 2, 0] / h + gum[:, 0, 2])
    S[:, 1, 0] = S[:, 0, 1]
    S[:, 1, 1] = gum[:, 1, 1]
    S[:, 1, 2] = 0.5 * (gum[:, 2, 1] + gum[:, 1, 2])
    S[:, 2, 0] = S[:, 0, 2]
    S[:, 2, 1] = S[:, 1, 2]
    S[:, 2, 2] = gum[:, 2, 2]
    S1jj = (-0.5 * (dhdr ** 2 + dhdrr * h) / h ** 2 * u1m + 0.5 * dhdr * gum[:, 0, 1] / h + 0.5 * g22vm[:, 1]
            - dhds * gum[:, 0, 0] / h ** 3 + g11vm[:, 1] / h ** 2 + 0.5 * g33vm[:, 1]
            + (h * dhdsr - dhdr * dhds) / h ** 3 * u2m + 3.0 * dhdr * gum[:, 1, 0] / (2.0 * h ** 2)
            + 0.5 * g12vm[:, 2] / h + 0.5 * g13vm[:, 3] / h)
    S2jj = (0.5 * (dhdr * dhds - h * dhdsr) / h ** 3 * u1m - 3.0 * dhdr * gum[:, 0, 0] / (2.0 * h ** 2)
            + 0.5 * g12vm[:, 1] / h - dhdr ** 2 * u2m / h ** 2 + dhdr * gum[:, 1, 1] / h + g22vm[:, 2]
            - 0.5 * dhds * gum[:, 1, 0] / h ** 3 + 0.5 * g11vm[:, 2] / h ** 2 + 0.5 * g33vm[:, 2]
            + 0.5 * g23vm[:, 3])
    S3jj = (0.5 * g13vm[:, 1] / h + 0.5 * g23vm[:, 2] + 0.5 * dhdr * gum[:, 1, 2] / h
            + 0.5 * dhdr * gum[:, 2, 1] / h + 0.5 * g22vm[:, 3] + 0.5 * g11vm[:, 3] / h ** 2 + g33vm[:, 3]
            - 0.5 * dhds * gum[:, 2, 0] / h ** 3)
    LapT = 1.0 / h * (-dhds / h ** 2 * gtm[:, 0] + 1.0 / h * g11vm[:, 4] + h * g22vm[:, 4] + gtm[:, 1] * dhdr
                      + h * g33vm[:, 4])
    m = _materials(p, tm)
    rmu, rlm, con = m["rmu"], m["rlm"], m["con"]
    dmu, d2mu, dlm, d2lm, dcon, d2con = m["dmu"], m["d2mu"], m["dlm"], m["d2lm"], m["dcon"], m["d2con"]
    g1mu, g2mu, g3mu = (dmu * gtm[:, k] for k in range(3))
    g1dmu, g2dmu, g3dmu = (d2mu * gtm[:, k] for k in range(3))
    g1con, g2con, g3con = (dcon * gtm[:, k] for k in range(3))
    g1dcon, g2dcon, g3dcon = (d2con * gtm[:, k] for k in range(3))
    g1lm, g2lm, g3lm = (dlm * gtm[:, k] for k in range(3))
    g1dlm, g2dlm, g3dlm = (d2lm * gtm[:, k] for k in range(3))
    rlme, rmue = m["rlme"], m["rmue"]
    gM2 = GAMMA * p.Ma ** 2
    nav = p.navier()
    Re, Pr, Ma = p.Re, p.Pr, p.Ma

    bl = _zero_blocks(ny)
    G, A, B, C, D = bl["G"], bl["A"], bl["B"], bl["C"], bl["D"]
    Vxx, Vxy, Vyy, Vxz, Vyz, Vzz = (bl[k] for k in ("Vxx", "Vxy", "Vyy", "Vxz", "Vyz", "Vzz"))
    # continuity (spatial.f90:356-371)
    G[:, 0, 0] = 1.0
    A[:, 0, 0] = u1m / h; A[:, 0, 1] = rhom / h
    B[:, 0, 0] = u2m; B[:, 0, 2] = rhom
    C[:, 0, 0] = u3m; C[:, 0, 3] = rhom
    D[:, 0, 0] = divum; D[:, 0, 1] = grhom[:, 0] / h; D[:, 0, 2] = grhom[:, 1] + rhom * dhdr / h
    D[:, 0, 3] = grhom[:, 2]
    # x_1 momentum (spatial.f90:375-455)
    G[:, 1, 1] = rhom
    A[:, 1, 0] = tm / (h * gM2); A[:, 1, 1] = rhom * u1m / h; A[:, 1, 4] = rhom / (h * gM2)
    B[:, 1, 1] = rhom * u2m
    C[:, 1, 1] = rhom * u3m
    D[:, 1, 0] = (u1m / h * (gum[:, 0, 0] + u2m * dhdr) + u2m * gum[:, 0, 1] + u3m * gum[:, 0, 2]
                  + gtm[:, 0] / (h * gM2))
    D[:, 1, 1] = rhom * (gum[:, 0, 0] + u2m * dhdr) / h
    D[:, 1, 2] = rhom * (gum[:, 0, 1] + u1m * dhdr / h)
    D[:, 1, 3] = rhom * gum[:, 0, 2]
    D[:, 1, 4] = grhom[:, 0] / (h * gM2)
    if nav:
        f = rlme / (rmue * Re)
        A[:, 1, 1] -= f * (g1lm / h ** 2 - rlm / h ** 3 * dhds)
        A[:, 1, 2] -= f * rlm / h ** 2 * dhdr
        A[:, 1, 4] -= f * dlm * divum / h
        B[:, 1, 2] -= f * (g1lm / h)
        C[:, 1, 3] -= f * (g1lm / h)
        D[:, 1, 2] -= f * (g1lm * dhdr / h ** 2 - rlm / h ** 3 * dhds * dhdr + rlm / h ** 2 * dhdsr)
        D[:, 1, 4] -= f * (g1dlm * divum / h + dlm * g1divum)
        Vxx[:, 1, 1] = f * rlm / h ** 2
        Vxy[:, 1, 2] = f * rlm / h
        Vxz[:, 1, 3] = f * rlm / h
        f = 1.0 / Re
        A[:, 1, 1] -= f * (2.0 * g1mu / h ** 2 - 2.0 * rmu * dhds / h ** 3)
        A[:, 1, 2] -= f * (g2mu / h + rmu * 3.0 * dhdr / h ** 2)
        A[:, 1, 3] -= f * g3mu / h
        A[:, 1, 4] -= f * dmu * 2.0 * S[:, 0, 0] / h
        B[:, 1, 1] -= f * (g2mu + rmu * dhdr / h)
        B[:, 1, 4] -= f * dmu * 2.0 * S[:, 0, 1]
        C[:, 1, 1] -= f * g3mu
        C[:, 1, 4] -= f * dmu * 2.0 * S[:, 0, 2]
        D[:, 1, 1] -= f * (g2mu / h * (-dhdr) - rmu * (dhdr ** 2 + dhdrr * h) / h ** 2)
        D[:, 1, 2] -= f * (2.0 * g1mu / h ** 2 * dhdr + 2.0 * rmu * (dhdsr * h - dhds * dhdr) / h ** 3)
        D[:, 1, 4] -= f * 2.0 * (g1dmu / h * S[:, 0, 0] + g2dmu * S[:, 0, 1] + g3dmu * S[:, 0, 2] + dmu * S1jj)
        Vxx[:, 1, 1] += f * 2.0 * rmu / h ** 2
        Vxy[:, 1, 2] += f * rmu / h
        Vyy[:, 1, 1] += f * rmu
        Vxz[:, 1, 3] += f * rmu / h
        Vzz[:, 1, 1] += f * rmu
    # x_2 momentum (spatial.f90:459-541)
    G[:, 2, 2] = rhom
    A[:, 2, 2] = rhom * u1m / h
    B[:, 2, 0] = tm / gM2; B[:, 2, 2] = rhom * u2m; B[:, 2, 4] = rhom / gM2
    C[:, 2, 2] = rhom * u3m
    D[:, 2, 0] = u1m / h * (gum[:, 1, 0] - u1m * dhdr) + u2m * gum[:, 1, 1] + u3m * gum[:, 1, 2] + gtm[:, 1] / gM2
    D[:, 2, 1] = rhom * (gum[:, 1, 0] - 2.0 * u1m * dhdr) / h
    D[:, 2, 2] = rhom * gum[:, 1, 1]
    D[:, 2, 3] = rhom * gum[:, 1, 2]
    D[:, 2, 4] = grhom[:, 1] / gM2
    if nav:
        f = rlme / (rmue * Re)
        A[:, 2, 1] -= f * (g2lm / h - rlm * dhdr / h ** 2)
        B[:, 2, 2] -= f * (g2lm + rlm * dhdr / h)
        B[:, 2, 4] -= f * dlm * divum
        C[:, 2, 3] -= f * g2lm
        D[:, 2, 2] -= f * (g2lm / h * dhdr - rlm * dhdr / h ** 2 * dhdr + rlm / h * dhdrr)
        D[:, 2, 4] -= f * (g2dlm * divum + dlm * g2divum)
        Vxy[:, 2, 1] = f * rlm / h
        Vyy[:, 2, 2] = f * rlm
        Vyz[:, 2, 3] = f * rlm
        f = 1.0 / Re
        A[:, 2, 1] += f * rmu * 3.0 * dhdr / h ** 2
        A[:, 2, 2] -= f * (g1mu / h ** 2 - rmu * dhds / h ** 3)
        A[:, 2, 4] -= f * dmu * 2.0 * S[:, 1, 0] / h
        B[:, 2, 1] -= f * g1mu / h
        B[:, 2, 2] -= f * (2.0 * g2mu + 2.0 * rmu * dhdr / h)
        B[:, 2, 3] -= f * g3mu
        B[:, 2, 4] -= f * dmu * 2.0 * S[:, 1, 1]
        C[:, 2, 2] -= f * g3mu
        C[:, 2, 4] -= f * dmu * 2.0 * S[:, 1, 2]
        D[:, 2, 1] -= f * (g1mu / h ** 2 * (-dhdr) + rmu * (dhds * dhdr - h * dhdsr) / h ** 3)
        D[:, 2, 2] += f * 2.0 * rmu * dhdr ** 2 / h ** 2
        D[:, 2, 4] -= f * 2.0 * (g1dmu / h * S[:, 1, 0] + g2dmu * S[:, 1, 1] + g3dmu * S[:, 1, 2] + dmu * S2jj)
        Vxx[:, 2, 2] += f * rmu / h ** 2
        Vxy[:, 2, 1] += f * rmu / h
        Vyy[:, 2, 2] += f * 2.0 * rmu
        Vyz[:, 2, 3] += f * rmu
        Vzz[:, 2, 2] += f * rmu
    # x_3 momentum (spatial.f90:545-597)
    G[:, 3, 3] = rhom
    A[:, 3, 3] = rhom * u1m / h
    B[:, 3, 3] = rhom * u2m
    C[:, 3, 0] = tm / gM2; C[:, 3, 3] = rhom * u3m; C[:, 3, 4] = rhom / gM2
    D[:, 3, 0] = u1m * gum[:, 2, 0] / h + u2m * gum[:, 2, 1] + u3m * gum[:, 2, 2] + gtm[:, 2] / gM2
    D[:, 3, 1] = rhom * gum[:, 2, 0] / h
    D[:, 3, 2] = rhom * gum[:, 2, 1]
    D[:, 3, 3] = rhom * gum[:, 2, 2]
    D[:, 3, 4] = grhom[:, 2] / gM2
    if nav:
        f = rlme / (rmue * Re)
        A[:, 3, 1] -= f * g3lm / h
        B[:, 3, 2] -= f * g3lm
        C[:, 3, 3] -= f * g3lm
        C[:, 3, 2] -= f * rlm / h * dhdr
        C[:, 3, 4] -= f * dlm * divum
        D[:, 3, 2] -= f * (g2lm / h * dhdr)
        D[:, 3, 4] -= f * (g3dlm * divum + dlm * g3divum)
        Vxz[:, 3, 1] = f * rlm / h
        Vyz[:, 3, 2] = f * rlm
        Vzz[:, 3, 3] = f * rlm
        f = 1.0 / Re
        A[:, 3, 3] -= f * (g1mu / h ** 2 - rmu * dhds / h ** 3)
        A[:, 3, 4] -= f * dmu * 2.0 * S[:, 2, 0] / h
        B[:, 3, 3] -= f * (g2mu + rmu * dhdr / h)
        B[:, 3, 4] -= f * dmu * 2.0 * S[:, 2, 1]
        C[:, 3, 1] -= f * g1mu / h
        C[:, 3, 2] -= f * (g2mu + rmu * dhdr / h)
        C[:, 3, 3] -= f * 2.0 * g3mu
        C[:, 3, 4] -= f * dmu * 2.0 * S[:, 2, 2]
        D[:, 3, 4] -= f * 2.0 * (g1dmu / h * S[:, 2, 0] + g2dmu * S[:, 2, 1] + g3dmu * S[:, 2, 2] + dmu * S3jj)
        Vxx[:, 3, 3] += f * rmu / h ** 2
        Vyy[:, 3, 3] += f * rmu
        Vxz[:, 3, 1] += f * rmu / h
        Vyz[:, 3, 2] += f * rmu
        Vzz[:, 3, 3] += f * 2.0 * rmu
    # energy (spatial.f90:601-673)
    G[:, 4, 4] = rhom
    A[:, 4, 1] = rhom * GAMMA1 * tm / h; A[:, 4, 4] = rhom * u1m / h
    B[:, 4, 2] = rhom * GAMMA1 * tm; B[:, 4, 4] = rhom * u2m
    C[:, 4, 3] = rhom * GAMMA1 * tm; C[:, 4, 4] = rhom * u3m
    D[:, 4, 0] = u1m / h * gtm[:, 0] + u2m * gtm[:, 1] + u3m * gtm[:, 2] + GAMMA1 * tm * divum
    D[:, 4, 1] = rhom * gtm[:, 0] / h
    D[:, 4, 2] = rhom * gtm[:, 1] + rhom * GAMMA1 * tm * dhdr / h
    D[:, 4, 3] = rhom * gtm[:, 2]
    D[:, 4, 4] = rhom * GAMMA1 * divum
    if nav:
        f = GAMMA / (Pr * Re)
        A[:, 4, 4] -= f * (g1con / h ** 2 + dcon * gtm[:, 0] / h ** 2 - con * dhds / h ** 3)
        B[:, 4, 4] -= f * (g2con + dcon * gtm[:, 1] + con * dhdr / h)
        C[:, 4, 4] -= f * (g3con + dcon * gtm[:, 2])
        D[:, 4, 4] -= f * (g1dcon * gtm[:, 0] / h ** 2 + g2dcon * gtm[:, 1] + g3dcon * gtm[:, 2] + dcon * LapT)
        Vxx[:, 4, 4] = f * con / h ** 2
        Vyy[:, 4, 4] = f * con
        Vzz[:, 4, 4] = f * con
        f = GAMMA * GAMMA1 * Ma ** 2 * rlme / (Re * rmue)
        A[:, 4, 1] -= f * 2.0 * rlm * divum / h
        B[:, 4, 2] -= f * 2.0 * rlm * divum
        C[:, 4, 3] -= f * 2.0 * rlm * divum
        D[:, 4, 2] -= f * 2.0 * rlm * divum * dhdr / h
        D[:, 4, 4] -= f * dlm * divum * divum
        f = GAMMA * GAMMA1 * Ma ** 2 / Re
        A[:, 4, 1] -= f * 4.0 * rmu * S[:, 0, 0] / h
        A[:, 4, 2] -= f * 4.0 * rmu * S[:, 1, 0] / h
        A[:, 4, 3] -= f * 4.0 * rmu * S[:, 2, 0] / h
        B[:, 4, 1] -= f * 4.0 * rmu * S[:, 0, 1]
        B[:, 4, 2] -= f * 4.0 * rmu * S[:, 1, 1]
        B[:, 4, 3] -= f * 4.0 * rmu * S[:, 2, 1]
        C[:, 4, 1] -= f * 4.0 * rmu * S[:, 0, 2]
        C[:, 4, 2] -= f * 4.0 * rmu * S[:, 1, 2]
        C[:, 4, 3] -= f * 4.0 * rmu * S[:, 2, 2]
        D[:, 4, 1] += f * 4.0 * rmu * S[:, 1, 0] * dhdr / h
        D[:, 4, 2] -= f * 4.0 * rmu * S[:, 0, 0] * dhdr / h
        D[:, 4, 4] -= f * 2.0 * dmu * (S ** 2).sum(axis=(1, 2))
    return bl


def spatial_blocks(p: StabParams, ms: MeanState):
    """Coefficient blocks of the spatial operator for a flat wall (curve=0,
    h=1), spatial.f90:138-673; curved walls (curve = 2) go through
    spatial_blocks_curved.  The spatial solver zeroes u2m
    (spatial.f90:147) and uses the gamma-multiplied energy equation
    (spatial.f90:599-673)."""
    if p.curve != 0:
        return spatial_blocks_curved(p, ms, wall_metrics(p, ms.y))
    ny = p.ny
    vm = ms.vm
    rhom, u1m, _, u3m, tm = (vm[:, k] for k in range(5))
    u2m = np.zeros(ny)
    g2vm, g22vm = ms.g2vm, ms.g22vm
    gum = np.zeros((ny, 3, 3))
    for i, k in enumerate((1, 2, 3)):
        gum[:, i, 1] = g2vm[:, k]
    # with h = 1 and no streamwise/spanwise derivatives of the mean:
    divum = gum[:, 0, 0] + gum[:, 1, 1] + gum[:, 2, 2]
    grhom = np.stack([np.zeros(ny), g2vm[:, 0], np.zeros(ny)], axis=1)
    gtm = np.stack([np.zeros(ny), g2vm[:, 4], np.zeros(ny)], axis=1)
    g1divum = np.zeros(ny)
    g2divum = g22vm[:, 2]          # g12vm(:,2) + g22vm(:,3) with h = 1
    g3divum = np.zeros(ny)
    S = np.zeros((ny, 3, 3))
    S[:, 0, 0] = gum[:, 0, 0]
    S[:, 0, 1] = 0.5 * (gum[:, 1, 0] + gum[:, 0, 1])
    S[:, 0, 2] = 0.5 * (gum[:, 2, 0] + gum[:, 0, 2])
    S[:, 1, 0] = S[:, 0, 1]
    S[:, 1, 1] = gum[:, 1, 1]
    S[:, 1, 2] = 0.5 * (gum[:, 2, 1] + gum[:, 1, 2])
    S[:, 2, 0] = S[:, 0, 2]
    S[:, 2, 1] = S[:, 1, 2]
    S[:, 2, 2] = gum[:, 2, 2]
    S1jj = 0.5 * g22vm[:, 1]
    S2jj = g22vm[:, 2]
    S3jj = 0.5 * g22vm[:, 3]
    LapT = g22vm[:, 4]
    m = _materials(p, tm)
    rmu, rlm, con = m["rmu"], m["rlm"], m["con"]
    dmu, d2mu, dlm, d2lm, dcon, d2con = m["dmu"], m["d2mu"], m["dlm"], m["d2lm"], m["dcon"], m["d2con"]
    g1mu, g2mu, g3mu = (dmu * gtm[:, k] for k in range(3))
    g1dmu, g2dmu, g3dmu = (d2mu * gtm[:, k] for k in range(3))
    g1con, g2con, g3con = (dcon * gtm[:, k] for k in range(3))
    g1dcon, g2dcon, g3dcon = (d2con * gtm[:, k] for k in range(3))
    g1lm, g2lm, g3lm = (dlm * gtm[:, k] for k in range(3))
    g1dlm, g2dlm, g3dlm = (d2lm * gtm[:, k] for k in range(3))
    rlme, rmue = m["rlme"], m["rmue"]
    ig = 1.0 / (GAMMA * p.Ma ** 2)
    nav = p.navier()
    Re, Pr, Ma = p.Re, p.Pr, p.Ma

    bl = _zero_blocks(ny)
    G, A, B, C, D = bl["G"], bl["A"], bl["B"], bl["C"], bl["D"]
    Vxx, Vxy, Vyy, Vxz, Vyz, Vzz = (bl[k] for k in ("Vxx", "Vxy", "Vyy", "Vxz", "Vyz", "Vzz"))

    # continuity (spatial.f90:356-371)
    G[:, 0, 0] = 1.0
    A[:, 0, 0] = u1m; A[:, 0, 1] = rhom
    B[:, 0, 0] = u2m; B[:, 0, 2] = rhom
    C[:, 0, 0] = u3m; C[:, 0, 3] = rhom
    D[:, 0, 0] = divum; D[:, 0, 1] = grhom[:, 0]; D[:, 0, 2] = grhom[:, 1]; D[:, 0, 3] = grhom[:, 2]
    # momentum, convective + pressure (spatial.f90:375-392, 459-476, 545-559)
    for e in (1, 2, 3):
        c = e - 1
        G[:, e, e] = rhom
        A[:, e, e] = rhom * u1m
        B[:, e, e] = rhom * u2m
        C[:, e, e] = rhom * u3m
        P = (A, B, C)[c]
        P[:, e, 0] = tm * ig
        P[:, e, 4] = rhom * ig
        D[:, e, 0] = u1m * gum[:, c, 0] + u2m * gum[:, c, 1] + u3m * gum[:, c, 2] + gtm[:, c] * ig
        D[:, e, 1] = rhom * gum[:, c, 0]
        D[:, e, 2] = rhom * gum[:, c, 1]
        D[:, e, 3] = rhom * gum[:, c, 2]
        D[:, e, 4] = grhom[:, c] * ig
    if nav:
        # x momentum (spatial.f90:396-455)
        f = rlme / (rmue * Re)
        A[:, 1, 1] -= f * g1lm
        A[:, 1, 4] -= f * dlm * divum
        B[:, 1, 2] -= f * g1lm
        C[:, 1, 3] -= f * g1lm
        D[:, 1, 4] -= f * (g1dlm * divum + dlm * g1divum)
        Vxx[:, 1, 1] = f * rlm
        Vxy[:, 1, 2] = f * rlm
        Vxz[:, 1, 3] = f * rlm
        f = 1.0 / Re
        A[:, 1, 1] -= f * 2.0 * g1mu
        A[:, 1, 2] -= f * g2mu
        A[:, 1, 3] -= f * g3mu
        A[:, 1, 4] -= f * dmu * 2.0 * S[:, 0, 0]
        B[:, 1, 1] -= f * g2mu
        B[:, 1, 4] -= f * dmu * 2.0 * S[:, 0, 1]
        C[:, 1, 1] -= f * g3mu
        C[:, 1, 4] -= f * dmu * 2.0 * S[:, 0, 2]
        D[:, 1, 4] -= f * 2.0 * (g1dmu * S[:, 0, 0] + g2dmu * S[:, 0, 1] + g3dmu * S[:, 0, 2] + dmu * S1jj)
        Vxx[:, 1, 1] += f * 2.0 * rmu
        Vxy[:, 1, 2] += f * rmu
        Vyy[:, 1, 1] += f * rmu
        Vxz[:, 1, 3] += f * rmu
        Vzz[:, 1, 1] += f * rmu
        # y momentum (spatial.f90:480-541)
        f = rlme / (rmue * Re)
        A[:, 2, 1] -= f * g2lm
        B[:, 2, 2] -= f * g2lm
        B[:, 2, 4] -= f * dlm * divum
        C[:, 2, 3] -= f * g2lm
        D[:, 2, 4] -= f * (g2dlm * divum + dlm * g2divum)
        Vxy[:, 2, 1] = f * rlm
        Vyy[:, 2, 2] = f * rlm
        Vyz[:, 2, 3] = f * rlm
        f = 1.0 / Re
        A[:, 2, 2] -= f * g1mu
        A[:, 2, 4] -= f * dmu * 2.0 * S[:, 1, 0]
        B[:, 2, 1] -= f * g1mu
        B[:, 2, 2] -= f * 2.0 * g2mu
        B[:, 2, 3] -= f * g3mu
        B[:, 2, 4] -= f * dmu * 2.0 * S[:, 1, 1]
        C[:, 2, 2] -= f * g3mu
        C[:, 2, 4] -= f * dmu * 2.0 * S[:, 1, 2]
        D[:, 2, 4] -= f * 2.0 * (g1dmu * S[:, 1, 0] + g2dmu * S[:, 1, 1] + g3dmu * S[:, 1, 2] + dmu * S2jj)
        Vxx[:, 2, 2] += f * rmu
        Vxy[:, 2, 1] += f * rmu
        Vyy[:, 2, 2] += f * 2.0 * rmu
        Vyz[:, 2, 3] += f * rmu
        Vzz[:, 2, 2] += f * rmu
        # z momentum (spatial.f90:563-597)
        f = rlme / (rmue * Re)
        A[:, 3, 1] -= f * g3lm
        B[:, 3, 2] -= f * g3lm
        C[:, 3, 3] -= f * g3lm
        C[:, 3, 4] -= f * dlm * divum
        D[:, 3, 4] -= f * (g3dlm * divum + dlm * g3divum)
        Vxz[:, 3, 1] = f * rlm
        Vyz[:, 3, 2] = f * rlm
        Vzz[:, 3, 3] = f * rlm
        f = 1.0 / Re
        A[:, 3, 3] -= f * g1mu
        A[:, 3, 4] -= f * dmu * 2.0 * S[:, 2, 0]
        B[:, 3, 3] -= f * g2mu
        B[:, 3, 4] -= f * dmu * 2.0 * S[:, 2, 1]
        C[:, 3, 1] -= f * g1mu
        C[:, 3, 2] -= f * g2mu
        C[:, 3, 3] -= f * 2.0 * g3mu
        C[:, 3, 4] -= f * dmu * 2.0 * S[:, 2, 2]
        D[:, 3, 4] -= f * 2.0 * (g1dmu * S[:, 2, 0] + g2dmu * S[:, 2, 1] + g3dmu * S[:, 2, 2] + dmu * S3jj)
        Vxx[:, 3, 3] += f * rmu
        Vyy[:, 3, 3] += f * rmu
        Vxz[:, 3, 1] += f * rmu
        Vyz[:, 3, 2] += f * rmu
        Vzz[:, 3, 3] += f * 2.0 * rmu
    # energy, gamma-multiplied form (spatial.f90:601-673)
    G[:, 4, 4] = rhom
    A[:, 4, 1] = rhom * GAMMA1 * tm
    A[:, 4, 4] = rhom * u1m
    B[:, 4, 2] = rhom * GAMMA1 * tm
    B[:, 4, 4] = rhom * u2m
    C[:, 4, 3] = rhom * GAMMA1 * tm
    C[:, 4, 4] = rhom * u3m
    D[:, 4, 0] = u1m * gtm[:, 0] + u2m * gtm[:, 1] + u3m * gtm[:, 2] + GAMMA1 * tm * divum
    D[:, 4, 1] = rhom * gtm[:, 0]
    D[:, 4, 2] = rhom * gtm[:, 1]
    D[:, 4, 3] = rhom * gtm[:, 2]
    D[:, 4, 4] = rhom * GAMMA1 * divum
    if nav:
        f = GAMMA / (Pr * Re)
        A[:, 4, 4] -= f * (g1con + dcon * gtm[:, 0])
        B[:, 4, 4] -= f * (g2con + dcon * gtm[:, 1])
        C[:, 4, 4] -= f * (g3con + dcon * gtm[:, 2])
        D[:, 4, 4] -= f * (g1dcon * gtm[:, 0] + g2dcon * gtm[:, 1] + g3dcon * gtm[:, 2] + dcon * LapT)
        Vxx[:, 4, 4] = f * con
        Vyy[:, 4, 4] = f * con
        Vzz[:, 4, 4] = f * con
        f = GAMMA * GAMMA1 * Ma ** 2 * rlme / (Re * rmue)
        A[:, 4, 1] -= f * 2.0 * rlm * divum
        B[:, 4, 2] -= f * 2.0 * rlm * divum
        C[:, 4, 3] -= f * 2.0 * rlm * divum
        D[:, 4, 4] -= f * dlm * divum * divum
        f = GAMMA * GAMMA1 * Ma ** 2 / Re
        for c in range(3):
            A[:, 4, 1 + c] -= f * 4.0 * rmu * S[:, c, 0]
            B[:, 4, 1 + c] -= f * 4.0 * rmu * S[:, c, 1]
            C[:, 4, 1 + c] -= f * 4.0 * rmu * S[:, c, 2]
        D[:, 4, 4] -= f * 2.0 * dmu * (S ** 2).sum(axis=(1, 2))
    return bl


# ---------------------------------------------------------------------------
# operator assembly
# ---------------------------------------------------------------------------
def _dense(rowblocks_D1, rowblocks_D2, rows_mask, D1, D2, diag):
    """Assemble M[(i,e),(j,v)] = P1[i,e,v] D1[i,j] - P2[i,e,v] D2[i,j]
    + delta_ij Q[i,e,v] on the equation rows selected by rows_mask[i,e]."""
    ny = D1.shape[0]
    M = (np.einsum("iev,ij->iejv", rowblocks_D1, D1)
         - np.einsum("iev,ij->iejv", rowblocks_D2, D2))
    idx = np.arange(ny)
    M[idx, :, idx, :] += diag
    M = M * rows_mask[:, :, None, None]
    return M.reshape(ny * NDOF, ny * NDOF)


def temporal_pencil(p: StabParams, ms: MeanState, bl=None):
    """A0, B0 of the temporal problem A0 x = omega B0 x, temporal.f90:604-752."""
    if bl is None:
        bl = temporal_blocks(p, ms)
    ny = p.ny
    a, b = p.alpha, p.beta
    im = 1j
    Dh = bl["D"] + im * a * bl["A"] + im * b * bl["C"] + a ** 2 * bl["Vxx"] + a * b * bl["Vxz"] + b ** 2 * bl["Vzz"]
    Bh = bl["B"] - im * a * bl["Vxy"] - im * b * bl["Vyz"]
    Bh = Bh * ms.deta[:, None, None] - bl["Vyy"] * ms.d2eta[:, None, None]
    Vyy = bl["Vyy"] * (ms.deta ** 2)[:, None, None]
    # interior rows, all equations: Bh D1 - Vyy D2 + Dh
    mask = np.zeros((ny, NDOF))
    mask[1:ny - 1, :] = 1.0
    A0 = _dense(Bh, Vyy, mask, ms.D1, ms.D2, Dh)
    # continuity rows at the free stream and the wall: Bh D1 + Dh
    mc = np.zeros((ny, NDOF))
    mc[0, 0] = 1.0
    mc[ny - 1, 0] = 1.0
    A0 += _dense(Bh, np.zeros_like(Vyy), mc, ms.D1, ms.D2, Dh)
    if p.wallt == 2:
        # wall energy row (temporal.f90:724-752); the reference multiplies
        # Vyy by D1 (not D2) in the jdof = 1..4 columns.
        i = ny - 1
        r = i * NDOF + 4
        A0[r, :] = 0.0
        for v in range(4):
            A0[r, v::NDOF] += Bh[i, 4, v] * ms.D1[i, :] - Vyy[i, 4, v] * ms.D1[i, :]
            A0[r, i * NDOF + v] += Dh[i, 4, v]
        A0[r, 4::NDOF] += Bh[i, 4, 4] * ms.Dt1[i, :] - Vyy[i, 4, 4] * ms.Dt2[i, :]
        A0[r, i * NDOF + 4] += Dh[i, 4, 4]
    n = ny * NDOF
    B0 = np.zeros((n, n), dtype=complex)
    B0[np.arange(NDOF), np.arange(NDOF)] = 1j
    for i in range(1, ny - 1):
        B0[i * NDOF:(i + 1) * NDOF, i * NDOF:(i + 1) * NDOF] = 1j * bl["G"][i]
    i = ny - 1
    for e in range(NDOF - 1):
        B0[i * NDOF + e, i * NDOF + e] = 1j
    if p.wallt == 0:
        B0[i * NDOF + 4, i * NDOF + 4] = 1j
    elif p.wallt == 2:
        B0[i * NDOF + 4, i * NDOF:(i + 1) * NDOF] = 1j * bl["G"][i, 4, :]
    else:
        raise ValueError(f"Illegal value of wallt: {p.wallt}")
    return A0, B0


def spatial_operators(p: StabParams, ms: MeanState, bl=None):
    """C0, C1, C2 of (C0 + alpha C1 + alpha^2 C2) phi = 0, spatial.f90:677-959."""
    if bl is None:
        bl = spatial_blocks(p, ms)
    ny = p.ny
    om, b = p.omega, p.beta
    im = 1j
    n = ny * NDOF
    Dh = bl["D"] + im * b * bl["C"] + b ** 2 * bl["Vzz"]
    Bh = (bl["B"] - im * b * bl["Vyz"]) * ms.deta[:, None, None] - bl["Vyy"] * ms.d2eta[:, None, None]
    Vyy = bl["Vyy"] * (ms.deta ** 2)[:, None, None]
    zero = np.zeros_like(Vyy)
    mask = np.zeros((ny, NDOF))
    mask[1:ny - 1, :] = 1.0
    C0 = _dense(Bh, Vyy, mask, ms.D1, ms.D2, Dh)
    mc = np.zeros((ny, NDOF))
    mc[ny - 1, 0] = 1.0
    if p.top == 1:
        mc[0, 0] = 1.0
    C0 = C0 + _dense(Bh, zero, mc, ms.D1, ms.D2, Dh)
    if p.wallt == 2:
        i = ny - 1
        r = i * NDOF + 4
        C0[r, :] = 0.0
        for v in range(4):
            C0[r, v::NDOF] += Bh[i, 4, v] * ms.D1[i, :] - Vyy[i, 4, v] * ms.D2[i, :]
            C0[r, i * NDOF + v] += Dh[i, 4, v]
        C0[r, 4::NDOF] += Bh[i, 4, 4] * ms.Dt1[i, :] - Vyy[i, 4, 4] * ms.Dt2[i, :]
        C0[r, i * NDOF + 4] += Dh[i, 4, 4]
    # time term and boundary rows (spatial.f90:786-835)
    if p.top == 1:
        C0[0, 0] = C0[0, 0] - im * om
    else:
        C0[0, 0] = -1.0
    for e in range(1, NDOF):
        C0[e, e] = -1.0
    for i in range(1, ny - 1):
        s = slice(i * NDOF, (i + 1) * NDOF)
        C0[s, s] = C0[s, s] - im * om * bl["G"][i]
    i = ny - 1
    i0 = i * NDOF
    C0[i0, i0] = C0[i0, i0] - im * om
    for e in (1, 2, 3):
        C0[i0 + e, i0 + e] = C0[i0 + e, i0 + e] - 1.0
    if p.wallt == 0:
        C0[i0 + 4, i0 + 4] = C0[i0 + 4, i0 + 4] - 1.0
    elif p.wallt == 2:
        C0[i0 + 4, i0:i0 + NDOF] = C0[i0 + 4, i0:i0 + NDOF] - im * om * bl["G"][i, 4, :]
    else:
        raise ValueError(f"Illegal value of wallt: {p.wallt}")
    # C1 (spatial.f90:839-938)
    Dh1 = im * bl["A"] + b * bl["Vxz"]
    Bh1 = (-im * bl["Vxy"]) * ms.deta[:, None, None]
    m1 = np.zeros((ny, NDOF))
    m1[1:ny - 1, :] = 1.0
    m1[ny - 1, 0] = 1.0
    if p.top == 1:
        m1[0, 0] = 1.0
    C1 = _dense(Bh1, zero, m1, ms.D1, ms.D2, Dh1)
    if p.wallt == 2:
        i = ny - 1
        r = i * NDOF + 4
        C1[r, :] = 0.0
        for v in range(4):
            C1[r, v::NDOF] += Bh1[i, 4, v] * ms.D1[i, :]
            C1[r, i * NDOF + v] += Dh1[i, 4, v]
        C1[r, 4::NDOF] += Bh1[i, 4, 4] * ms.Dt1[i, :]
        C1[r, i * NDOF + 4] += Dh1[i, 4, 4]
    # C2 (spatial.f90:942-959)
    C2 = np.zeros((n, n), dtype=complex)
    for i in range(1, ny - 1):
        s = slice(i * NDOF, (i + 1) * NDOF)
        C2[s, s] = bl["Vxx"][i]
    if p.wallt == 2:
        i = ny - 1
        C2[i * NDOF + 4, i * NDOF:(i + 1) * NDOF] = bl["Vxx"][i, 4, :]
    return C0, C1, C2


# ---------------------------------------------------------------------------
# eigensolves (the reference's LAPACK calls) and post-processing
# ---------------------------------------------------------------------------
def piksr2_order(keys: np.ndarray) -> np.ndarray:
    """PIKSR2 (Numerical Recipes straight insertion carrying an index): a
    stable ascending sort; returns the permutation."""
    return np.argsort(keys, kind="stable")


# ---------------------------------------------------------------------------
# finite-difference temporal solver (fd_temporal.f90, itype = 3)
# ---------------------------------------------------------------------------
# stencils.f90:9-120, the reference's coefficient table (values as written there)
FD_GA = (8.333333333333333333333E-02, -6.666666666666666666667E-01, 6.666666666666666666667E-01,
         -8.333333333333333333333E-02)
FD_GG = (-1.87603205562073772290017534999, 3.18538322557789286703668141674, -1.81454567943752757247830550034,
         0.59165824105260274421658150053, -0.101052068000505624644095417028, 0.0145883364282753087693133500917)
FD_GH = (-0.384254232677925402043233692192, -0.290638947767348681070279077173, 0.67176478451531541138011989728,
         0.071081659837399872713651693126, -0.073630718761724245070378308432, 0.0056774548542830440901194873933)
FD_GI = (0.182885278686826206583549109115, -1.08001475417455516433881053795, 0.65787289649662525818641772732,
         0.1776170486891931456381189546, 0.076779836395827558602005515075, -0.0151403060939170046712807681567)
FD_GJ = (-0.0341837103365291857798396404953, 0.224829025740103121729831613399, -0.89081233292845396245426338198,
         0.165299947710035014782196870489, 0.61343955208752529977826815383, -0.078572482272680288056193615249)
FD_DA = (-8.333333333333333333333E-02, 1.333333333333333333333E+00, -2.500000000000000000000E+00,
         1.333333333333333333333E+00, -8.333333333333333333333E-02)
FD_DB = (9.166666666666666666667E-01, -1.666666666666666666667E+00, 5.000000000000000000000E-01,
         3.333333333333333333333E-01, -8.333333333333333333333E-02)
FD_DD = (2.916666666666666666667E+00, -8.666666666666666666667E+00, 9.500000000000000000000E+00,
         -4.666666666666666666667E+00, 9.166666666666666666667E-01)


def ogengrid(ny: int, yi: float, ymax: float):
    """ogengrid.f90:14-44: uniform eta = (j-1)/(ny-1) on [0, 1], wall first,
    y = a eta / (b - eta) with a = ymax yi / (ymax - 2 yi), b = 1 + a / ymax.
    The Mahesh map (yi = 0) reads its parameters interactively and is not
    supported.  Returns y, eta, deta, d2eta and the eta spacing."""
    if yi == 0.0:
        raise ValueError("Mahesh map (Yi = 0) reads dymin, b, yc interactively; not supported")
    dy = 1.0 / float(ny - 1)
    aa = ymax * yi / (ymax - 2.0 * yi)
    bb = 1.0 + aa / ymax
    eta = np.arange(ny, dtype=np.float64) * dy
    y = aa * eta / (bb - eta)
    deta = (bb - eta) ** 2 / (aa * bb)
    d2eta = -2.0 * (bb - eta) ** 3 / (aa * bb) ** 2
    return y, eta, deta, d2eta, dy


def fd_grad_matrix(ny: int, dy: float) -> np.ndarray:
    """The y-gradient of grad.f90:62-86 as a matrix: fourth-order one-sided
    and biased five-point stencils at the two end rows on each side, the
    central stencil inside, each divided by 12 dy."""
    G = np.zeros((ny, ny))
    G[0, 0:5] = (-25.0, 48.0, -36.0, 16.0, -3.0)
    G[1, 0:5] = (-3.0, -10.0, 18.0, -6.0, 1.0)
    for i in range(2, ny - 2):
        G[i, i - 2:i + 3] = (1.0, -8.0, 0.0, 8.0, -1.0)
    G[ny - 2, ny - 5:ny] = -np.array((1.0, -6.0, 18.0, -10.0, -3.0))
    G[ny - 1, ny - 5:ny] = -np.array((-3.0, 16.0, -36.0, 48.0, -25.0))
    return G / (12.0 * dy)


def fd_operator_tables(ny: int, dy: float):
    """Per-row stencils of the finite-difference operator (fd_temporal.f90:
    636-895), as matrices multiplying Bh (first derivative, F1) and Vyy
    (second derivative, F2), with node 0 the wall:
      row 0        Carpenter's one-sided gg / the one-sided dd (wall rows);
      rows 1, 2, 3 Carpenter's biased gh, gi, gj / db, da, da;
      rows 4..ny-5 the central ga (no centre entry) / da;
      rows ny-4, ny-3, ny-2 the mirrored gj, gi, gh with a minus sign, and
                   the second-derivative signs exactly as the reference
                   writes them (+da4, +da5 on row ny-4; +da4 on row ny-3);
      row ny-1     zero (the free-stream rows are B0 = i I, A0 = 0)."""
    F1 = np.zeros((ny, ny))
    F2 = np.zeros((ny, ny))
    F1[0, 0:6] = FD_GG
    F2[0, 0:5] = FD_DD
    F1[1, 0:6] = FD_GH
    F2[1, 0:5] = FD_DB
    F1[2, 0:6] = FD_GI
    F2[2, 0:5] = FD_DA
    F1[3, 0:6] = FD_GJ
    F2[3, 1:6] = FD_DA
    for i in range(4, ny - 4):
        F1[i, i - 2] = FD_GA[0]
        F1[i, i - 1] = FD_GA[1]
        F1[i, i + 1] = FD_GA[2]
        F1[i, i + 2] = FD_GA[3]
        F2[i, i - 2:i + 3] = FD_DA
    i = ny - 4
    F1[i, i - 2:i + 4] = [-FD_GJ[5], -FD_GJ[4], -FD_GJ[3], -FD_GJ[2], -FD_GJ[1], -FD_GJ[0]]
    F2[i, i - 2:i + 3] = [FD_DA[0], FD_DA[1], FD_DA[2], -FD_DA[3], -FD_DA[4]]
    i = ny - 3
    F1[i, i - 3:i + 3] = [-FD_GI[5], -FD_GI[4], -FD_GI[3], -FD_GI[2], -FD_GI[1], -FD_GI[0]]
    F2[i, i - 2:i + 3] = [FD_DA[0], FD_DA[1], FD_DA[2], -FD_DA[3], FD_DA[4]]
    i = ny - 2
    F1[i, i - 4:i + 2] = [-FD_GH[5], -FD_GH[4], -FD_GH[3], -FD_GH[2], -FD_GH[1], -FD_GH[0]]
    F2[i, i - 3:i + 2] = [FD_DB[4], FD_DB[3], FD_DB[2], FD_DB[1], FD_DB[0]]
    return F1 / dy, F2 / (dy * dy)


def fd_spatial_tables(ny: int, dy: float):
    """Per-row stencils of the finite-difference spatial operator
    (fd_spatial.f90:668-960), node 0 the wall: rows 0-3 and the interior as
    in fd_operator_tables, the central rows running to ny-3, row ny-2 the
    fourth-order biased (-1, 6, -18, 10, 3)/12 with the mirrored db second
    derivative, and row ny-1 the one-sided (3, -16, 36, -48, 25)/12 first
    derivative that the free-stream continuity row uses when top = 1."""
    F1 = np.zeros((ny, ny))
    F2 = np.zeros((ny, ny))
    F1[0, 0:6] = FD_GG
    F2[0, 0:5] = FD_DD
    F1[1, 0:6] = FD_GH
    F2[1, 0:5] = FD_DB
    F1[2, 0:6] = FD_GI
    F2[2, 0:5] = FD_DA
    F1[3, 0:6] = FD_GJ
    F2[3, 1:6] = FD_DA
    for i in range(4, ny - 2):
        F1[i, i - 2] = FD_GA[0]
        F1[i, i - 1] = FD_GA[1]
        F1[i, i + 1] = FD_GA[2]
        F1[i, i + 2] = FD_GA[3]
        F2[i, i - 2:i + 3] = FD_DA
    i = ny - 2
    F1[i, i - 3:i + 2] = np.array([-1.0, 6.0, -18.0, 10.0, 3.0]) / 12.0
    F2[i, i - 3:i + 2] = [FD_DB[4], FD_DB[3], FD_DB[2], FD_DB[1], FD_DB[0]]
    i = ny - 1
    F1[i, i - 4:i + 1] = np.array([3.0, -16.0, 36.0, -48.0, 25.0]) / 12.0
    return F1 / dy, F2 / (dy * dy)


def fd_mean_state(p: StabParams, ym: np.ndarray, vt: np.ndarray, first=None, second=None) -> MeanState:
    """Grid, mean flow and mean derivatives of fd_temporal.f90:92-152: the
    ogengrid grid, getmean's spline at its nodes, then grad applied once and
    twice in eta and mapped (g22 = G(G v) deta^2 + (G v) d2eta, g2 = (G v)
    deta); with ider = 0 the derivatives come from getmean2's tables.  D1, D2
    hold the operator's stencil tables (fd_operator_tables)."""
    ny = p.ny
    y, eta, deta, d2eta, dy = ogengrid(ny, p.yi, p.ymax)
    if not p.ider:
        vm, g2, g22 = getmean2(ym, vt, first, second, y)
    else:
        vm = getmean(ym, vt, y)
        G = fd_grad_matrix(ny, dy)
        g2 = G @ vm
        g22 = G @ g2
        g22 = g22 * (deta ** 2)[:, None] + g2 * d2eta[:, None]
        g2 = g2 * deta[:, None]
    F1, F2 = fd_spatial_tables(ny, dy) if p.itype == 4 else fd_operator_tables(ny, dy)
    return MeanState(y, eta, deta, d2eta, F1, F2, F1, F2, vm, g2, g22)


def fd_temporal_pencil(p: StabParams, ms: MeanState, bl=None):
    """A0, B0 of the finite-difference temporal problem (fd_temporal.f90:
    581-895).  Node 0 is the wall: its continuity row is Dh + F1 Bh, its
    energy row Dh + F1 Bh - F2 Vyy with the temperature column's Bh term
    left out (the "adiabatic constraint", :693-708), and its momentum rows
    are B0 = i, A0 = 0; the free-stream node has B0 = i I, A0 = 0 (the
    zero-disturbance rows).  The wall temperature option is not read."""
    if bl is None:
        bl = temporal_blocks(p, ms)
    ny = p.ny
    a, b = p.alpha, p.beta
    im = 1j
    Dh = bl["D"] + im * a * bl["A"] + im * b * bl["C"] + a ** 2 * bl["Vxx"] + a * b * bl["Vxz"] + b ** 2 * bl["Vzz"]
    Bh = bl["B"] - im * a * bl["Vxy"] - im * b * bl["Vyz"]
    Bh = Bh * ms.deta[:, None, None] - bl["Vyy"] * ms.d2eta[:, None, None]
    Vyy = bl["Vyy"] * (ms.deta ** 2)[:, None, None]
    mask = np.zeros((ny, NDOF))
    mask[1:ny - 1, :] = 1.0
    A0 = _dense(Bh, Vyy, mask, ms.D1, ms.D2, Dh)
    # wall continuity row: Dh + F1 Bh
    mc = np.zeros((ny, NDOF))
    mc[0, 0] = 1.0
    A0 += _dense(Bh, np.zeros_like(Vyy), mc, ms.D1, ms.D2, Dh)
    # wall energy row: Dh + F1 Bh - F2 Vyy, no Bh term in the temperature column
    me = np.zeros((ny, NDOF))
    me[0, 4] = 1.0
    Bw = Bh.copy()
    Bw[0, 4, 4] = 0.0
    A0 += _dense(Bw, Vyy, me, ms.D1, ms.D2, Dh)
    n = ny * NDOF
    B0 = np.zeros((n, n), dtype=complex)
    for e in range(NDOF - 1):
        B0[e, e] = 1j
    B0[4, 0:NDOF] = 1j * bl["G"][0, 4, :]
    for i in range(1, ny - 1):
        B0[i * NDOF:(i + 1) * NDOF, i * NDOF:(i + 1) * NDOF] = 1j * bl["G"][i]
    i = ny - 1
    for e in range(NDOF):
        B0[i * NDOF + e, i * NDOF + e] = 1j
    return A0, B0


def fd_spatial_operators(p: StabParams, ms: MeanState):
    """C0, C1, C2 of the finite-difference spatial problem (fd_spatial.f90:
    106-1170), node 0 the wall.  The coefficient blocks are the spatial
    solver's; the wall metric is calch's for curve = 1 and flat otherwise
    (fd_spatial.f90:108-116 has no circle).  Rows as in spatial_operators
    with the finite-difference stencils, and two quirks kept: the wall
    energy row of wallt = 2 takes its -i omega G term from the G of node
    ny-1 (top = 1) or ny-2 (top = 0), the node index the assembly loops leave
    behind (fd_spatial.f90:917-921), and its temperature column has no
    first-derivative term in C0 and C1 (the "adiabatic constraint")."""
    q = p if (p.curve == 1 and p.x != -1.0) else dataclasses.replace(p, curve=0)
    bl = spatial_blocks(q, ms)
    ny = p.ny
    om, b = p.omega, p.beta
    im = 1j
    n = ny * NDOF
    Dh = bl["D"] + im * b * bl["C"] + b ** 2 * bl["Vzz"]
    Bh = (bl["B"] - im * b * bl["Vyz"]) * ms.deta[:, None, None] - bl["Vyy"] * ms.d2eta[:, None, None]
    Vyy = bl["Vyy"] * (ms.deta ** 2)[:, None, None]
    zero = np.zeros_like(Vyy)
    F1, F2 = ms.D1, ms.D2
    mask = np.zeros((ny, NDOF))
    mask[1:ny - 1, :] = 1.0
    C0 = _dense(Bh, Vyy, mask, F1, F2, Dh)
    mc = np.zeros((ny, NDOF))
    mc[0, 0] = 1.0
    if p.top == 1:
        mc[ny - 1, 0] = 1.0
    C0 = C0 + _dense(Bh, zero, mc, F1, F2, Dh)
    gq = ny - 1 if p.top == 1 else ny - 2
    if p.wallt == 2:
        me = np.zeros((ny, NDOF))
        me[0, 4] = 1.0
        Bw = Bh.copy()
        Bw[0, 4, 4] = 0.0
        C0 = C0 + _dense(Bw, Vyy, me, F1, F2, Dh)
    # time term and boundary rows (fd_spatial.f90:907-947)
    C0[0, 0] = C0[0, 0] - im * om
    for e in (1, 2, 3):
        C0[e, e] = -1.0
    if p.wallt == 0:
        C0[4, 4] = -1.0
    elif p.wallt == 2:
        C0[4, 0:NDOF] = C0[4, 0:NDOF] - im * om * bl["G"][gq, 4, :]
    else:
        raise ValueError(f"Illegal value of wallt: {p.wallt}")
    for i in range(1, ny - 1):
        sl = slice(i * NDOF, (i + 1) * NDOF)
        C0[sl, sl] = C0[sl, sl] - im * om * bl["G"][i]
    i0 = (ny - 1) * NDOF
    if p.top == 1:
        C0[i0, i0] = C0[i0, i0] - im * om
    else:
        C0[i0, i0] = -1.0
    for e in range(1, NDOF):
        C0[i0 + e, i0 + e] = -1.0
    # C1 (fd_spatial.f90:951-1160)
    Dh1 = im * bl["A"] + b * bl["Vxz"]
    Bh1 = (-im * bl["Vxy"]) * ms.deta[:, None, None]
    m1 = np.zeros((ny, NDOF))
    m1[1:ny - 1, :] = 1.0
    m1[0, 0] = 1.0
    if p.top == 1:
        m1[ny - 1, 0] = 1.0
    C1 = _dense(Bh1, zero, m1, F1, F2, Dh1)
    if p.wallt == 2:
        me = np.zeros((ny, NDOF))
        me[0, 4] = 1.0
        Bw1 = Bh1.copy()
        Bw1[0, 4, 4] = 0.0
        C1 = C1 + _dense(Bw1, zero, me, F1, F2, Dh1)
    # C2 (fd_spatial.f90:1164-1180)
    C2 = np.zeros((n, n), dtype=complex)
    if p.wallt == 2:
        C2[4, 0:NDOF] = bl["Vxx"][0, 4, :]
    for i in range(1, ny - 1):
        sl = slice(i * NDOF, (i + 1) * NDOF)
        C2[sl, sl] = bl["Vxx"][i]
    return C0, C1, C2


def fd_temporal_solve(p: StabParams, ms: MeanState, want_vectors=True) -> Eigensystem:
    """fd_temporal.f90:970-1042: ZGESV(B0, A0), ZGEEV('N','V'), PIKSR2 on
    Im(omega), columns scaled by their max-modulus entry."""
    lp = _lapack()
    A0, B0 = fd_temporal_pencil(p, ms)
    lu, piv, X, info = lp.zgesv(B0, A0)
    if info != 0:
        raise RuntimeError(f"ZGESV info={info}")
    w, vl, vr, info = lp.zgeev(X, compute_vl=0, compute_vr=1 if want_vectors else 0)
    if info != 0:
        raise RuntimeError(f"ZGEEV info={info}")
    order = piksr2_order(w.imag)
    w = w[order]
    evec = None
    if want_vectors:
        evec = vr[:, order]
        idx = np.argmax(np.abs(evec), axis=0)
        sc = evec[idx, np.arange(evec.shape[1])]
        nz = sc != 0
        evec[:, nz] = evec[:, nz] / sc[nz]
    return Eigensystem(p, ms, w, evec)


def _lapack():
    from scipy.linalg import lapack
    return lapack


@dataclasses.dataclass
class Eigensystem:
    params: StabParams
    ms: MeanState
    eig: np.ndarray          # sorted eigenvalues (omega or alpha)
    evec: Optional[np.ndarray]


def temporal_solve(p: StabParams, ms: MeanState, want_vectors=True) -> Eigensystem:
    """temporal.f90:771-880: ZGESV(B0, A0) then ZGEEV('N','V'), PIKSR2 on
    Im(omega), columns scaled by their max-modulus entry."""
    lp = _lapack()
    A0, B0 = temporal_pencil(p, ms)
    lu, piv, X, info = lp.zgesv(B0, A0)
    if info != 0:
        raise RuntimeError(f"ZGESV info={info}")
    w, vl, vr, info = lp.zgeev(X, compute_vl=0, compute_vr=1 if want_vectors else 0)
    if info != 0:
        raise RuntimeError(f"ZGEEV info={info}")
    order = piksr2_order(w.imag)
    w = w[order]
    evec = None
    if want_vectors:
        evec = vr[:, order]
        idx = np.argmax(np.abs(evec), axis=0)   # first max wins
        sc = evec[idx, np.arange(evec.shape[1])]
        nz = sc != 0
        evec[:, nz] = evec[:, nz] / sc[nz]
    return Eigensystem(p, ms, w, evec)


def spatial_companion(p: StabParams, ms: MeanState, ops=None):
    """spatial.f90:972-1016 (fd_spatial.f90:1194-1236): ZGETRF(C0),
    C1 := -C0^{-1} C1, C2 := -C0^{-1} C2, B0 = [[C1, C2], [I, 0]]."""
    lp = _lapack()
    C0, C1, C2 = spatial_operators(p, ms) if ops is None else ops
    lu, piv, info = lp.zgetrf(C0)
    if info < 0:
        raise RuntimeError(f"ZGETRF info={info}")
    X1, info1 = lp.zgetrs(lu, piv, -C1)
    X2, info2 = lp.zgetrs(lu, piv, -C2)
    n = C0.shape[0]
    B0 = np.zeros((2 * n, 2 * n), dtype=complex)
    B0[:n, :n] = X1
    B0[:n, n:] = X2
    B0[n + np.arange(n), np.arange(n)] = 1.0
    return B0


def spatial_solve(p: StabParams, ms: MeanState, want_vectors=True, ops=None) -> Eigensystem:
    """spatial.f90:1041-1084: ZGEEV on the companion matrix, alpha = 1/lambda
    (lambda = 0 -> 0), PIKSR2 on Im(alpha).  Eigenvectors are not rescaled."""
    lp = _lapack()
    B0 = spatial_companion(p, ms, ops)
    w, vl, vr, info = lp.zgeev(B0, compute_vl=0, compute_vr=1 if want_vectors else 0)
    alp = np.where(w != 0, 1.0 / np.where(w != 0, w, 1.0), 0.0)
    order = piksr2_order(alp.imag)
    alp = alp[order]
    evec = vr[:, order] if want_vectors else None
    return Eigensystem(p, ms, alp, evec)


def solve(p: StabParams, ym, vt, want_vectors=True, first=None, second=None) -> Eigensystem:
    if p.itype == 4:
        # stab.f90:61-67: itype becomes 2 before fd_spatial runs
        ms = fd_mean_state(p, ym, vt, first, second)
        es = spatial_solve(p, ms, want_vectors, fd_spatial_operators(p, ms))
        es.params = dataclasses.replace(p, itype=2)
        return es
    if p.itype == 3:
        # stab.f90:56-60: itype becomes 1 before fd_temporal runs, so evec.dat says 1
        es = fd_temporal_solve(p, fd_mean_state(p, ym, vt, first, second), want_vectors)
        es.params = dataclasses.replace(p, itype=1)
        return es
    ms = mean_state(p, ym, vt, first, second)
    if p.itype == 1:
        return temporal_solve(p, ms, want_vectors)
    if p.itype == 2:
        es = spatial_solve(p, ms, want_vectors)
        if p.curve == 2 and p.x != -1.0:
            # circh sets its argument, the module's x, to zero (circh.f90:60);
            # evec.dat records that x
            es.params = dataclasses.replace(p, x=0.0)
        return es
    raise ValueError("itype must be 1 or 2")


# ---------------------------------------------------------------------------
# getevec (selection, rescale quirk) and the ASCII / unformatted writers
# ---------------------------------------------------------------------------
def getevec_select(eig: np.ndarray, value: complex) -> int:
    """getevec.f90:161-172 (-v): nearest eigenvalue, first minimum wins."""
    d = np.abs(value - eig)
    return int(np.argmin(d))


def getevec_scale(vec: np.ndarray, ny: int) -> np.ndarray:
    """getevec.f90:179-189: `scale` is declared REAL, so only the real part
    of the running pick is kept; rows 1..5*ny divided by it."""
    v = vec[: ny * NDOF].copy()
    scale = 0.0
    for e in v:
        if abs(e) > abs(scale):
            scale = e.real
    if scale != 0.0:
        v = v / scale
    return v


def fortran_e(x: float, w: int, d: int, e: Optional[int]) -> str:
    """Fortran 1PEw.d[Ee] edit descriptor."""
    if not np.isfinite(x):
        return ("NaN" if np.isnan(x) else ("Infinity" if x > 0 else "-Infinity")).rjust(w)
    if x == 0.0:
        mant, ex = "0." + "0" * d, 0
        neg = math.copysign(1.0, x) < 0
    else:
        s = f"{abs(x):.{d}E}"
        m, ex_s = s.split("E")
        mant, ex = m, int(ex_s)
        neg = x < 0
    if e is None:
        if abs(ex) <= 99:
            exs = f"E{'-' if ex < 0 else '+'}{abs(ex):02d}"
        else:
            exs = f"{'-' if ex < 0 else '+'}{abs(ex):03d}"
    else:
        exs = f"E{'-' if ex < 0 else '+'}{abs(ex):0{e}d}"
    out = ("-" if neg else "") + mant + exs
    return out.rjust(w)


def e2113(x):
    return fortran_e(float(x), 21, 13, 3)


def e136(x):
    return fortran_e(float(x), 13, 6, None)


def eigfunction_text(es: Eigensystem, j: int) -> str:
    """The time.N / space.N file of getevec.f90:193-227 for eigenvalue j."""
    p, ms = es.params, es.ms
    ny = p.ny
    v = getevec_scale(es.evec[:, j], ny)
    ev = es.eig[j]
    lines = [f"# Re = {e136(p.Re)}, Ma = {e136(p.Ma)}, Pr = {e136(p.Pr)}"]

    def cx(z):
        return f"({e2113(z.real)},{e2113(z.imag)})"
    if p.itype == 1:
        lines.append(f"# Omega = {cx(ev)}")
        lines.append(f"# Alpha = {cx(p.alpha)}")
    else:
        lines.append(f"# Omega = {cx(p.omega)}")
        lines.append(f"# Alpha = {cx(ev)}")
    lines.append(f"# Beta  = {cx(p.beta)}")
    for i in range(ny - 1, -1, -1):
        vals = [ms.y[i]]
        for e in range(NDOF):
            z = v[i * NDOF + e]
            vals += [z.real, z.imag]
        # the trailing 1X of the format only positions; it writes no blank
        lines.append(" ".join(e2113(t) for t in vals))
    return "\n".join(lines) + "\n"


def parse_eigfunction(text: str):
    """Read a time.N / space.N file: (eigenvalue, rows[ny, 11])."""
    ev = None
    rows = []
    for ln in text.splitlines():
        if ln.startswith("#"):
            if "Omega" in ln or "Alpha" in ln:
                inner = ln.split("(")[1].split(")")[0]
                a, b = inner.split(",")
                key = "Omega" if "Omega" in ln else "Alpha"
                if ev is None:
                    ev = {}
                ev[key] = complex(float(a.replace("E", "e")), float(b))
            continue
        if ln.strip():
            rows.append([float(t) for t in ln.split()])
    return ev, np.asarray(rows)


def _record(payload: bytes) -> bytes:
    n = struct.pack("<i", len(payload))
    return n + payload + n


def evec_dat_bytes(es: Eigensystem) -> bytes:
    """gfortran sequential unformatted evec.dat (temporal.f90:883-890,
    spatial.f90:1120-1126): 4-byte little-endian record markers."""
    p, ms = es.params, es.ms
    r1 = struct.pack("<10i", p.ind, p.ny, NDOF, p.itype, p.ievec, p.curve, p.top, p.wall, p.wallt,
                     1 if p.ider else 0)
    r2 = np.array([p.omega, p.alpha, p.beta], dtype=np.complex128).tobytes() + \
        np.array([p.Re, p.Ma, p.Pr], dtype=np.float64).tobytes()
    r3 = np.concatenate([[p.x], ms.y, ms.eta, ms.deta, ms.d2eta, [p.yi, p.ymax]]).astype(np.float64).tobytes()
    r4 = np.asarray(es.eig, dtype=np.complex128).tobytes()
    out = _record(r1) + _record(r2) + _record(r3) + _record(r4)
    if p.itype == 1 or p.ievec == 1:
        out += _record(np.asfortranarray(es.evec, dtype=np.complex128).tobytes(order="F"))
    return out


# ---------------------------------------------------------------------------
# synthetic profiles with the shapes the benchmark configurations name
# ---------------------------------------------------------------------------
def synthetic_profile(M: float, ymax: float = 50.0, nym: int = 2000, erf_width: float = 2.0,
                      crossflow: bool = False):
    """Mean profile table in the profile.N layout (y rho u v w T):
    U = erf(y/s), V = 0, W = 0 or 0.08 y exp(1 - y/1.5)/1.5,
    Tw = 1 + 0.2 sqrt(0.72) M^2, T = Tw + (1-Tw) U + 0.2 M^2 U (1-U),
    rho = 1/T.  Uniform rows on [0, max(ymax, 60)]."""
    from scipy.special import erf
    y = np.linspace(0.0, max(ymax, 60.0), nym)
    U = erf(y / erf_width)
    W = 0.08 * y * np.exp(1.0 - y / 1.5) / 1.5 if crossflow else np.zeros_like(y)
    Tw = 1.0 + 0.2 * math.sqrt(0.72) * M ** 2
    T = Tw + (1.0 - Tw) * U + 0.2 * M ** 2 * U * (1.0 - U)
    rho = 1.0 / T
    vt = np.stack([rho, U, np.zeros_like(y), W, T], axis=1)
    return y, vt


# ---------------------------------------------------------------------------
# mode tracking across sweep files (getab / getax / getalpha)
# ---------------------------------------------------------------------------
def track_pick(spectra, param, start, rule):
    """Picks of the reference's post-processors over a sweep.

    spectra[j]: eigenvalues of point j; param[j]: swept value; start: the
    user's typed values for the first 1 ('nearest', getalpha.f90:120-146) or
    2 ('extrapolate', getab.f90:161-201, getax.f90:161-201) points.  Each pick
    is the first eigenvalue nearest the guess (strict '<' scan, as the
    reference's loops)."""
    picks = []
    for j, ev in enumerate(spectra):
        if j < len(start):
            g = complex(start[j])
        elif rule == "nearest" or j < 2:
            g = picks[j - 1]
        else:
            e1, p1 = picks[j - 1], param[j - 1]
            e2, p2 = picks[j - 2], param[j - 2]
            g = e1 + (e2 - e1) / (p2 - p1) * (param[j] - p1)
        d = np.abs(np.asarray(ev) - g)
        picks.append(complex(ev[int(np.argmin(d))]))
    return picks


def mtemporal_points(amin, amax, ainc, bmin, bmax, binc):
    """(alpha, beta) of the solves of the temporal driver, in loop order
    (mtemporal.f90:25-39): na = max(nint((amax-amin)/ainc), 1), beta inner."""
    na = max(_nint((amax - amin) / ainc), 1)
    nb = max(_nint((bmax - bmin) / binc), 1)
    return [(amin + float(ia - 1) * ainc, bmin + float(ib - 1) * binc)
            for ia in range(1, na + 1) for ib in range(1, nb + 1)]


def mspatial_points(omin, omax, oinc, bmin, bmax, binc, ind1, ind2, ind_inc, xb, delta):
    """(ind, x, Yi, omega, beta) of the spatial driver's solves in loop order
    (mspatial.f90:65-96): zero increments become one, nint(range/inc) + 1
    values each, x = xb(ind), Yi = 2 delta(ind)."""
    oinc = 1.0 if oinc == 0.0 else oinc
    binc = 1.0 if binc == 0.0 else binc
    ind_inc = 1 if ind_inc == 0 else ind_inc
    no = _nint((omax - omin) / oinc) + 1
    nb = _nint((bmax - bmin) / binc) + 1
    out = []
    for ind in range(ind1, ind2 + (1 if ind_inc > 0 else -1), ind_inc):
        for io in range(1, no + 1):
            for ib in range(1, nb + 1):
                out.append((ind, xb[ind - 1], 2.0 * delta[ind - 1], omin + float(io - 1) * oinc,
                            bmin + float(ib - 1) * binc))
    return out


def _nint(v: float) -> int:
    """Fortran NINT: nearest integer, halves away from zero."""
    return int(math.floor(abs(v) + 0.5)) * (1 if v >= 0 else -1)


def read_delta(text: str):
    """delta.dat (mspatial.f90:29-63): rows not starting with '#' hold xb, delta."""
    xb, de = [], []
    for ln in text.splitlines():
        if ln.startswith("#") or not ln.strip():
            continue
        f = ln.replace(",", " ").split()
        xb.append(float(f[0].replace("d", "e").replace("D", "e")))
        de.append(float(f[1].replace("d", "e").replace("D", "e")))
    return xb, de


def getab_picks(spectra, param, first):
    """getab / getax (getab.f90:161-201): the first two picks are the
    eigenvalues nearest the user's values `first` (the -v mode), then the
    eigenvalue nearest the linear extrapolation through the two previous
    picks; nearest = first minimum of a strict '<' scan."""
    picks = []
    for j, ev in enumerate(spectra):
        ev = np.asarray(ev)
        if j < 2:
            g = complex(first[j])
        else:
            e1, p1 = picks[j - 1], param[j - 1]
            e2, p2 = picks[j - 2], param[j - 2]
            g = e1 + (e2 - e1) / (p2 - p1) * (param[j] - p1)
        picks.append(complex(ev[int(np.argmin(np.abs(ev - g)))]))
    return picks


def getalpha_picks(spectra, jloc):
    """getalpha (getalpha.f90:120-146): the first pick by 1-based index jloc,
    then the eigenvalue nearest the previous pick."""
    picks = [complex(np.asarray(spectra[0])[jloc - 1])]
    for ev in spectra[1:]:
        ev = np.asarray(ev)
        picks.append(complex(ev[int(np.argmin(np.abs(ev - picks[-1])))]))
    return picks


def stab_out_text(param, values, ind=None):
    """stab.out of getab (format 60: 3(1x,1pe20.13)) or, with ind, of getax /
    parm.new of getalpha (format 50: i4,3(1x,1pe20.13))."""
    lines = []
    for j, (p, v) in enumerate(zip(param, values)):
        f = "".join(" " + fortran_e(float(t), 20, 13, None) for t in (p, v.real, v.imag))
        lines.append((f"{int(ind[j]):4d}" if ind is not None else "") + f)
    return "\n".join(lines) + "\n"
