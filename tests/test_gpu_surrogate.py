"""What the trained network gains over the method without it.

Region: supersonic second modes (M in [1.5, 2], alpha in [0.2, 0.4],
Re in [1500, 3000], beta in [0, 0.1]).  Here the N = 32 seed spectrum does
not resolve the least-stable discrete mode, so the coarse-seeded method
(STAB_MODE_COARSE, the method without the network) can verify few instances
at its first level and sends the rest through the second seed level (N = 48 for these temporal
instances).  The
network, trained here by the library's BF16 kernels on plain FP64 solves at
N = 64, adds its prediction as one more candidate (STAB_MODE_SURROGATE);
where that candidate's converged pair is the least stable, the instance is
settled without the second level, with STAB_ST_UNVERIFIED.

Checks on 512 instances: the network's fit halves its loss; the surrogate
mode settles at least one instance from the network's seed and sends that
many fewer instances through the fallback chain; among its unverified
results at least half as many as the network settled equal the plain FP64
result within 1e-10; the count of instances
equal to the plain result (any status) drops by at most 8 against the
coarse mode; and no instance that either mode reports as STAB_ST_OK or
STAB_ST_FELLBACK differs from the plain result by more than 1e-10 in more
than 2 % of the instances.
"""
import math

import numpy as np
import pytest

import stab_gb300 as sg

pytestmark = pytest.mark.gpu
pytest.importorskip("torch")

REGION = {"M": (1.5, 2.0), "alpha": (0.2, 0.4), "log10Re": (math.log10(1500.0), math.log10(3000.0)),
          "beta": (0.0, 0.1)}


def test_network_gain_over_coarse_seeds(ctx):
    from stab_gb300 import surrogate as su
    ds = su.make_dataset(ctx, 4096, 21, REGION)
    P, v = ds["params"], ds["valid"]
    X = su.features(P["M"], P["Re"], P["alpha"], P["beta"], P["width"])[v]
    sur = su.Surrogate(ctx, max_batch=4096)
    fit = sur.fit(X, ds["omega"][v], P["alpha"][v], ds["coef"][v], steps=4000, batch=1024)
    assert fit["losses"][-1][1] < 0.5 * fit["losses"][0][1]
    n = 512
    Q = su.sample_params(n, 99, REGION)
    params = [su.stab_params(Q["M"][k], Q["Re"][k], Q["alpha"][k], Q["beta"][k], 64) for k in range(n)]
    profs = [su.erf_profile(Q["M"][k], Q["width"][k]) for k in range(n)]
    b = ctx.batch(params, profs)
    b.run(sg.MODE_PLAIN)
    truth, _, _, tst, _ = b.results()

    def right(eig, st):
        return (np.abs(eig - truth) / np.abs(truth) <= 1e-10) & np.isin(st, [sg.ST_OK, sg.ST_FELLBACK]) & (tst == 0)

    def any_right(eig):
        return (np.abs(eig - truth) / np.abs(truth) <= 1e-10) & (tst == 0)

    b.run(sg.MODE_COARSE)
    e_c, _, _, s_c, _ = b.results()
    counts_c = b.counts()
    sur.seed_batch(b, su.features(Q["M"], Q["Re"], Q["alpha"], Q["beta"], Q["width"]), Q["alpha"])
    b.run(sg.MODE_SURROGATE)
    e_s, _, _, s_s, _ = b.results()
    counts_s = b.counts()
    b.close()
    sur.close()
    trusted_c, trusted_s = np.isin(s_c, [sg.ST_OK, sg.ST_FELLBACK]), np.isin(s_s, [sg.ST_OK, sg.ST_FELLBACK])
    any_c, any_s = any_right(e_c), any_right(e_s)
    seed_picks = s_s == sg.ST_UNVERIFIED
    print(f"surrogate region: coarse any-right {int(any_c.sum())} counts {counts_c}; surrogate any-right "
          f"{int(any_s.sum())} counts {counts_s}; unverified {int(seed_picks.sum())}")
    assert counts_s["surrogate_seed"] >= 1
    assert counts_s["fp64_fallback"] <= counts_c["fp64_fallback"] - counts_s["surrogate_seed"]
    assert int(np.sum(any_s & seed_picks)) * 2 >= counts_s["surrogate_seed"]
    assert int(any_s.sum()) >= int(any_c.sum()) - 8
    assert np.sum(trusted_c & ~any_c) <= 0.02 * n and np.sum(trusted_s & ~any_s) <= 0.02 * n
