"""The oracle under grid refinement on an instance of the benchmark sweep
(index 180 of PCG64(20261203), N = 48) where the coarse-seeded path's trusted
result differs from the plain FP64 pick at the instance's own N.

At N = 48 the selection rule picks a growing mode with negative phase speed
(omega ~ -0.341 + 2.75e-3 i).  At N = 64 and N = 80 that mode is gone, and the
least-stable mode there is the same eigenvalue to 1e-9 relative
(0.374830 - 2.99e-4 i, the value the coarse path returns): the N = 48 pick is
a discretisation artifact, not the converged least-stable mode.
"""
import numpy as np

from oracle import baseline as bl
from oracle import stab_oracle as so


def _least(d, prof, ny):
    p = so.StabParams(mattyp=d["mattyp"], T0=d["T0"], Ma=d["Ma"], Re=d["Re"], Pr=d["Pr"], ny=ny, yi=d["yi"],
                      ymax=d["ymax"], ievec=0, ider=1, top=0, wall=0, wallt=0, curve=0, itype=1,
                      alpha=complex(*d["alpha"]), beta=complex(*d["beta"]), omega=0j)
    ym = prof[:, 0].copy()
    vt = prof[:, 1:6].copy()
    vt[:, 2] = 0.0
    es = so.solve(p, ym, vt, want_vectors=False)
    dd = dict(d)
    dd["ny"] = ny
    j = bl.select_least(es.eig, dd)
    return es.eig[j], es.eig


def test_plain_pick_at_n48_is_not_grid_converged():
    import bench
    params, prof = bench.workload(4096, 20261203)
    k = 180
    d = params[k]
    assert d["ny"] == 48
    w48, _ = _least(d, prof[k], 48)
    w64, e64 = _least(d, prof[k], 64)
    w80, _ = _least(d, prof[k], 80)
    assert w48.real < 0 and w48.imag > 0                      # upstream, growing
    assert np.min(np.abs(e64 - w48)) > 1e-3 * abs(w48)         # gone at N = 64
    assert abs(w64 - w80) <= 1e-9 * abs(w80)                   # converged pick
    assert abs(w80 - (0.374830 - 2.989e-4j)) <= 1e-6
