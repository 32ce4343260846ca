"""The LU panel-width autotuner: every variant it times is a correct
factorisation, and its choice is used afterwards (a polish through the tuned
width reproduces the oracle)."""
import numpy as np
import pytest

import stab_gb300 as sg
from tests import helpers as H

pytestmark = pytest.mark.gpu


def test_autotune_picks_a_feasible_width_and_keeps_results(ctx):
    table = ctx.autotune([160, 320])
    for n, row in table.items():
        for prec in ("c64", "c128"):
            nb, ms = row[prec]
            assert nb in (8, 16, 32) and ms > 0.0
    d, prof = H.synth_case(1, 48, 1.2, 800.0, a=0.25, b=0.05)
    es = H.oracle_solve(d, prof, want_vectors=False)
    w = es.eig[H.select_least(es.eig, d)]
    eig, err, iters, st, _ = ctx.solve_batch([H.stab_params(d)], [prof], sg.MODE_SEEDED, seeds=[w * (1 + 1e-7)])
    assert st[0] == sg.ST_OK and abs(eig[0] - w) / abs(w) < 1e-10


@pytest.mark.parametrize("n,z", [(240, True), (640, True), (320, False)])
def test_cluster_lu_matches_single_cta(ctx, n, z):
    md, pd = ctx.lu_cluster_check(n, 8, complex128=z)
    assert pd == 0 and md == 0.0


@pytest.mark.parametrize("tma", [1, 0])
@pytest.mark.parametrize("n", [40, 201, 320, 640])
def test_tensor_core_lu_backward_error(ctx, n, tma):
    """The complex64 LU with the trailing update on the tensor cores (TF32
    parts, six part products), with the A22 tiles moved by tensor (TMA)
    loads and stores or through the registers, against the CUDA-core LU on
    the same matrices: backward error max|PA - LU| / max|A| at most 4x the
    CUDA-core one and below 1e-5 (complex64 working accuracy, n up to 640;
    the odd order takes the register form in both settings)."""
    ctx.set_option(sg.OPT_POLISH_LU_TMA, tma)
    try:
        bt, bs, pd = ctx.lu_tc_check(n, 4)
    finally:
        ctx.set_option(sg.OPT_POLISH_LU_TMA, 1)
    assert np.isfinite(bt)
    assert bt < 1e-5, (bt, bs, pd)
    assert bt <= 4.0 * bs + 1e-7, (bt, bs, pd)


@pytest.mark.parametrize("n", [320, 640])
def test_tensor_core_lu_tma_form_identical_to_register_form(ctx, n):
    """The TMA form of the tensor-core LU moves each A22 tile through shared
    memory by tensor loads and stores; every tile takes the same MMAs in the
    same order and the same epilogue additions as the register form, so both
    factor the same matrices to the same bits: equal backward errors and
    pivots."""
    out = {}
    try:
        for tma in (1, 0):
            ctx.set_option(sg.OPT_POLISH_LU_TMA, tma)
            out[tma] = ctx.lu_tc_check(n, 4)
    finally:
        ctx.set_option(sg.OPT_POLISH_LU_TMA, 1)
    (bt1, bs1, pd1), (bt0, bs0, pd0) = out[1], out[0]
    assert bt1 == bt0, (bt1, bt0)
    assert pd1 == pd0 and bs1 == bs0
