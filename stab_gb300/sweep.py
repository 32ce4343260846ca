"""Mode tracking along parameter sweeps: the batched counterpart of the
reference's sweep drivers (mtemporal.f90:20-39, mspatial.f90:77-96) and of
the post-processors that follow one mode through their output files.

The reference solves every sweep point's full spectrum into eig.N files and
then picks a mode per file:
  - getab / getax (getab.f90:181-201, getax.f90:181-201): the first two
    points by the user (nearest eigenvalue to a typed value), then the
    eigenvalue nearest the linear extrapolation
    e1 + (e2 - e1) / (p2 - p1) * (p - p1) through the two previous points;
  - getalpha (getalpha.f90:132-146): the first point by the user, then the
    eigenvalue nearest the previous point's.
Here each sweep point is a polish from that guess (`MODE_TRACK`), started
from the previous point's eigenvector.  Where the polish fails, the library
takes the FP64 full spectrum and keeps the eigenvalue nearest the guess,
which is the reference's pick.  Many sweep lines run side by side: each
step solves one point of every line in one batch.

The output writers produce the reference's files: stab.out of getab (one
line per point, "p Re Im", 3(1x,1pe20.13)) and of getax / parm.new of
getalpha ("ind x Re Im", i4,3(1x,1pe20.13)).
"""
from __future__ import annotations

from typing import List, Optional, Sequence

import numpy as np

import stab_gb300 as sg
from stab_gb300.surrogate import chebyshev_coefficients


def _e2013(x: float) -> str:
    """Fortran 1PE20.13 (exponent E+dd up to 99)."""
    if x == 0.0:
        m, ex = "0." + "0" * 13, 0
    else:
        m, e = f"{abs(x):.13E}".split("E")
        ex = int(e)
    sign = "-" if np.signbit(x) else ""
    exs = f"E{'-' if ex < 0 else '+'}{abs(ex):02d}" if abs(ex) <= 99 else f"{'-' if ex < 0 else '+'}{abs(ex):03d}"
    return (sign + m + exs).rjust(20)


def guess(rule: str, j: int, param: np.ndarray, values: np.ndarray, start: Sequence[complex]) -> complex:
    """The reference's guess for point j of one line."""
    if j < len(start):
        return complex(start[j])
    if rule == "nearest":
        return complex(values[j - 1])
    if rule == "extrapolate":
        if j < 2:
            return complex(values[j - 1])
        e1, p1 = values[j - 1], param[j - 1]
        e2, p2 = values[j - 2], param[j - 2]
        return complex(e1 + (e2 - e1) / (p2 - p1) * (param[j] - p1))
    raise ValueError(f"unknown rule {rule!r}")


def track_lines(ctx: sg.Context, lines: List[List[sg.StabParams]], profiles: List[List[np.ndarray]],
                param: np.ndarray, start: List[Sequence[complex]], rule: str = "extrapolate",
                use_vectors: bool = True):
    """Follow one mode along each line.  lines[l][j] is point j of line l
    (all lines the same length K, same N per point index), param[j] the swept
    value, start[l] the user's values for the first one (nearest) or two
    (extrapolate) points.  Returns values (L, K) complex and status (L, K)."""
    L, K = len(lines), len(param)
    vals = np.zeros((L, K), dtype=np.complex128)
    stat = np.zeros((L, K), dtype=np.int32)
    prev_vecs = None
    for j in range(K):
        g = [guess(rule, j, param, vals[l], start[l]) for l in range(L)]
        b = ctx.batch([lines[l][j] for l in range(L)], [profiles[l][j] for l in range(L)])
        try:
            b.set_seeds(g)
            ny = lines[0][j].ny
            if use_vectors and prev_vecs is not None and all(p.itype == 1 and p.ny == ny for p in
                                                             (lines[l][j] for l in range(L))):
                b.set_start(np.stack([chebyshev_coefficients(v, ny, ncheb=ny) for v in prev_vecs]))
            b.run(sg.MODE_TRACK)
            eig, err, iters, st, vecs = b.results(want_vectors=True)
        finally:
            b.close()
        vals[:, j] = eig
        stat[:, j] = st
        prev_vecs = vecs
    return vals, stat


def stab_out_lines(param: np.ndarray, values: np.ndarray, ind: Optional[Sequence[int]] = None) -> str:
    """getab's stab.out (ind None) or getax's stab.out / getalpha's parm.new
    (ind given: "ind x Re Im")."""
    out = []
    for j, (p, v) in enumerate(zip(param, values)):
        cols = " " + " ".join(_e2013(t) for t in (float(p), v.real, v.imag))
        out.append((f"{int(ind[j]):4d}" if ind is not None else "") + cols)
    return "\n".join(out) + "\n"
