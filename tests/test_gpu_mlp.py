"""The surrogate network's BF16 kernels against the CPU oracle
(oracle/mlp_oracle.py): forward pass, gradients and one Adam step, then a
short training run that must lower the loss.

Tolerances: outputs and gradients within 1e-3 of the oracle in relative
Frobenius norm per tensor (the kernels accumulate in float32 in another
order; a bf16 rounding that flips moves one element by one bf16 step);
parameters after one Adam step within 1e-5 absolute.
"""
import numpy as np
import pytest

import stab_gb300 as sg
from oracle import mlp_oracle as mo

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

SIZES = (6, 256, 256, 256, 256, 162)


def _init(sizes, seed):
    rng = np.random.default_rng(seed)
    flat = []
    for k, n in zip(sizes[:-1], sizes[1:]):
        flat.append((rng.uniform(-1, 1, size=(k, n)) * np.sqrt(6.0 / k)).astype(np.float32).ravel())
        flat.append((0.05 * rng.normal(size=n)).astype(np.float32))
    return np.concatenate(flat)


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def _data(B, seed):
    rng = np.random.default_rng(seed)
    X = rng.uniform(-1.5, 1.5, size=(B, SIZES[0])).astype(np.float32)
    T = rng.normal(size=(B, SIZES[-1])).astype(np.float32)
    w = np.where(np.arange(SIZES[-1]) < 2, 4.0, 0.25).astype(np.float32)
    return X, T, w


@pytest.mark.parametrize("B", [37, 512])
def test_forward_and_gradients_match_oracle(ctx, B):
    net = sg.Network(ctx, SIZES, 1024)
    flat = _init(SIZES, 3)
    net.set_params(flat)
    X, T, w = _data(B, 4)
    dev = "cuda:0"
    x, t, wd = (torch.from_numpy(a).to(dev) for a in (X, T, w))
    y = torch.empty((B, SIZES[-1]), dtype=torch.float32, device=dev)
    net.forward(B, x.data_ptr(), y.data_ptr())
    ctx.sync()
    params = net.split(flat)
    Yo, cache = mo.forward(params, X)
    assert _rel(y.cpu().numpy(), Yo) < 1e-3
    loss = net.gradients(B, x.data_ptr(), t.data_ptr(), wd.data_ptr())
    Lo, dY = mo.loss_grad(Yo, T, w)
    assert abs(loss - Lo) <= 1e-3 * Lo
    go = mo.backward(params, cache, dY)
    _, g = net.get_params(grads=True)
    for (gW, gb), (oW, ob) in zip(net.split(g), go):
        assert _rel(gW, oW) < 1e-3
        assert _rel(gb, ob) < 1e-3
    net.close()


def test_adam_step_matches_oracle(ctx):
    net = sg.Network(ctx, SIZES, 256)
    flat = _init(SIZES, 5)
    net.set_params(flat)
    X, T, w = _data(256, 6)
    x, t, wd = (torch.from_numpy(a).cuda() for a in (X, T, w))
    net.train_step(256, x.data_ptr(), t.data_ptr(), wd.data_ptr(), 1e-3)
    p1, g = net.get_params(grads=True)
    params = net.split(flat)
    new = mo.adam(params, net.split(g), mo.adam_state(params), 1, 1e-3)
    ref = np.concatenate([np.concatenate([W.ravel(), b]) for W, b in new])
    assert np.max(np.abs(p1 - ref)) < 1e-5
    net.close()


def test_training_lowers_the_loss(ctx):
    """A smooth 6 -> 162 target learned by the library's own training loop."""
    net = sg.Network(ctx, SIZES, 2048)
    net.set_params(_init(SIZES, 7))
    rng = np.random.default_rng(8)
    X = rng.uniform(-1, 1, size=(2048, 6)).astype(np.float32)
    A = rng.normal(size=(6, 162)).astype(np.float32) / 3
    T = np.sin(X @ A).astype(np.float32)
    w = np.ones(162, np.float32)
    x, t, wd = (torch.from_numpy(a).cuda() for a in (X, T, w))
    first = net.train_step(2048, x.data_ptr(), t.data_ptr(), wd.data_ptr(), 1e-3, want_loss=True)
    for _ in range(300):
        net.train_step(2048, x.data_ptr(), t.data_ptr(), wd.data_ptr(), 1e-3)
    last = net.gradients(2048, x.data_ptr(), t.data_ptr(), wd.data_ptr())
    assert last < 0.05 * first
    net.close()


@pytest.mark.parametrize("B", [37, 300])
def test_tcgen05_and_mma_sync_forms_agree(ctx, B):
    """The network's GEMMs on tcgen05 (STAB_OPT_MLP_TCGEN05, default) and on
    mma.sync multiply the same bf16 operands and accumulate in float32 in
    another order: outputs agree within 2e-4 and gradients within 1e-3
    relative (a bf16 rounding of a hidden activation that flips between them
    moves one element by one bf16 step), and the tcgen05 outputs match the
    oracle within 1e-3."""
    flat = _init(SIZES, 5)
    X, T, w = _data(B, 6)
    dev = "cuda:0"
    x, t, wd = (torch.from_numpy(a).to(dev) for a in (X, T, w))
    out = {}
    try:
        for tc5 in (1, 0):
            ctx.set_option(sg.OPT_MLP_TCGEN05, tc5)
            net = sg.Network(ctx, SIZES, 1024)
            net.set_params(flat)
            y = torch.empty((B, SIZES[-1]), dtype=torch.float32, device=dev)
            net.forward(B, x.data_ptr(), y.data_ptr())
            ctx.sync()
            loss = net.gradients(B, x.data_ptr(), t.data_ptr(), wd.data_ptr())
            _, g = net.get_params(grads=True)
            out[tc5] = (y.cpu().numpy(), loss, g.copy(), net.split(flat))
            net.close()
    finally:
        ctx.set_option(sg.OPT_MLP_TCGEN05, 1)
    (y1, l1, g1, params), (y0, l0, g0, _) = out[1], out[0]
    assert _rel(y1, y0) < 2e-4, _rel(y1, y0)
    assert abs(l1 - l0) <= 2e-4 * abs(l0), (l1, l0)
    assert _rel(g1, g0) < 1e-3, _rel(g1, g0)
    Yo, _ = mo.forward(params, X)
    assert _rel(y1, Yo) < 1e-3


def test_inference_batch_8192_both_forms(ctx):
    """Inference at the surrogate's full batch (8192 rows, the 6 -> 4 x 256 ->
    162 network): the tcgen05 and mma.sync forms agree within 2e-4 and the
    tcgen05 output matches the oracle within 1e-3 on the first 256 rows."""
    B = 8192
    flat = _init(SIZES, 7)
    X, _, _ = _data(B, 8)
    dev = "cuda:0"
    x = torch.from_numpy(X).to(dev)
    out = {}
    try:
        for tc5 in (1, 0):
            ctx.set_option(sg.OPT_MLP_TCGEN05, tc5)
            net = sg.Network(ctx, SIZES, B)
            net.set_params(flat)
            y = torch.empty((B, SIZES[-1]), dtype=torch.float32, device=dev)
            net.forward(B, x.data_ptr(), y.data_ptr())
            ctx.sync()
            out[tc5] = (y.cpu().numpy(), net.split(flat))
            net.close()
    finally:
        ctx.set_option(sg.OPT_MLP_TCGEN05, 1)
    (y1, params), (y0, _) = out[1], out[0]
    assert _rel(y1, y0) < 2e-4, _rel(y1, y0)
    Yo, _ = mo.forward(params, X[:256])
    assert _rel(y1[:256], Yo) < 1e-3
