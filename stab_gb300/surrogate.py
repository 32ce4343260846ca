"""Surrogate seeding of the shift-invert polish (no counterpart in the reference).

A BF16 multilayer perceptron, 6 inputs -> 4 hidden layers of 256 (GELU) ->
162 outputs, maps the flow parameters of a temporal instance of the profile
family U = erf(y/s), T by Crocco-Busemann with the adiabatic wall temperature
Tw = 1 + 0.2 sqrt(0.72) M^2, rho = 1/T, to its least-stable omega and the
first 16 Chebyshev coefficients of each of the five eigenvector fields.

Inputs:  (M, Re, alpha, beta, Tw, s), shifted and scaled by `features`.
Outputs: Re(omega)/alpha, 100 Im(omega)/alpha, then Re and Im of the
         coefficients c[e][q] (field e in rho, u, v, w, T; q < 16), each
         standardised by the training set's mean and deviation.

The network is trained on the GPU by the library's own kernels (the
``stab_mlp_*`` entry points, tensor-core BF16 GEMMs with float32
accumulation), on solves of the plain FP64 batched path at N = 64, and it
seeds ``MODE_SURROGATE``: after the coarse N = 32 candidates, the instances
that are not yet final polish the predicted omega from the start vector
evaluated from the predicted coefficients, and the least-stable converged
pair wins.  That recovers discrete modes N = 32 does not resolve (the
supersonic second modes), whose coarse candidates are spurious.  PyTorch
only holds device buffers here.
"""
from __future__ import annotations

import math
import time
from typing import Optional

import numpy as np

import stab_gb300 as sg

SIZES = (6, 256, 256, 256, 256, 162)
NCHEB = 16
TRAIN_NY = 64
T0_SUTHERLAND = 110.4 / 0.3815      # S / T_inf = 0.3815 with S = 110.4 K
LOSS_WEIGHTS = np.concatenate([[4.0, 4.0], np.full(160, 0.1)]).astype(np.float32)

# the parameter ranges of the sweep the network is trained for
RANGES = {"alpha": (0.05, 0.4), "beta": (0.0, 0.3), "log10Re": (math.log10(300.0), math.log10(3000.0)),
          "M": (0.0, 2.0), "width": (1.5, 3.0)}


def adiabatic_tw(M):
    return 1.0 + 0.2 * math.sqrt(0.72) * np.asarray(M, dtype=np.float64) ** 2


def features(M, Re, alpha, beta, width) -> np.ndarray:
    """Network inputs, each scaled to roughly unit range."""
    M, Re, a, b, s = (np.asarray(v, dtype=np.float64) for v in (M, Re, alpha, beta, width))
    return np.stack([M - 1.0, (np.log10(Re) - 2.9) / 0.5, (a - 0.225) / 0.1, (b - 0.15) / 0.087,
                     (adiabatic_tw(M) - 1.34) / 0.2, (s - 2.25) / 0.43], axis=1).astype(np.float32)


def erf_profile(M: float, width: float = 2.0, nym: int = 2000, ymax: float = 60.0) -> np.ndarray:
    """profile.<ind> rows (y rho u v w T) of the erf family on [0, ymax]."""
    from scipy.special import erf
    y = np.linspace(0.0, ymax, nym)
    U = erf(y / width)
    Tw = float(adiabatic_tw(M))
    T = Tw + (1.0 - Tw) * U + 0.2 * M * M * U * (1.0 - U)
    return np.stack([y, 1.0 / T, U, np.zeros_like(y), np.zeros_like(y), T], axis=1)


def sample_params(count: int, seed: int, ranges: Optional[dict] = None) -> dict:
    """Uniform draws over `ranges` (M >= 1e-3: the pressure scales as 1/M^2)."""
    r = dict(RANGES, **(ranges or {}))
    rng = np.random.Generator(np.random.PCG64(seed))
    out = {k: rng.uniform(*r[k], count) for k in ("alpha", "beta", "log10Re", "M", "width")}
    out["M"] = np.maximum(out["M"], 1e-3)
    out["Re"] = 10.0 ** out.pop("log10Re")
    return out


def stab_params(M, Re, alpha, beta, ny: int) -> sg.StabParams:
    return sg.StabParams.make(itype=1, ny=int(ny), Ma=float(M), Re=float(Re), Pr=0.72, mattyp=1, T0=T0_SUTHERLAND,
                              yi=1.0 / 23.0, ymax=50.0, alpha=complex(alpha), beta=complex(beta))


def chebyshev_coefficients(vec: np.ndarray, ny: int, ncheb: int = NCHEB) -> np.ndarray:
    """(5, ncheb) coefficients of the fields of a temporal eigenvector given
    at the Gauss-Lobatto points eta_i = cos(pi i/(ny-1)) (row 5 i + e),
    after dividing it by its first max-modulus entry."""
    v = np.asarray(vec, dtype=np.complex128)[: 5 * ny]
    p = int(np.argmax(np.abs(v)))
    v = v / v[p] if v[p] != 0 else v
    f = v.reshape(ny, 5).T                       # (5, ny)
    i = np.arange(ny)
    q = np.arange(ncheb)[:, None]
    C = np.cos(np.pi * q * i[None, :] / (ny - 1))  # (ncheb, ny)
    wgt = np.ones(ny)
    wgt[0] = wgt[-1] = 0.5
    c = (2.0 / (ny - 1)) * (f * wgt) @ C.T       # (5, ncheb)
    c[:, 0] *= 0.5
    if ncheb >= ny:
        c[:, ny - 1] *= 0.5
    return c


def chebyshev_eval(coef: np.ndarray, ny: int) -> np.ndarray:
    """The start vector the library builds from `coef` (5 x ncheb)."""
    i = np.arange(ny)
    q = np.arange(coef.shape[1])
    T = np.cos(np.pi * np.outer(i, q) / (ny - 1))  # (ny, ncheb)
    return (T @ coef.T).reshape(-1)                # node-major: 5 i + e


def make_dataset(ctx: sg.Context, count: int, seed: int, ranges: Optional[dict] = None, chunk: int = 4096,
                 ny: int = TRAIN_NY) -> dict:
    """Least-stable omega and eigenvector coefficients from the plain FP64
    batched path at N = ny (default 64, where the supersonic discrete modes
    are resolved; N = 32 still carries unresolved modes above them) on
    `count` sampled instances."""
    P = sample_params(count, seed, ranges)
    w = np.zeros(count, dtype=np.complex128)
    coef = np.zeros((count, 5, NCHEB), dtype=np.complex128)
    ok = np.zeros(count, dtype=bool)
    t0 = time.perf_counter()
    for k0 in range(0, count, chunk):
        idx = range(k0, min(count, k0 + chunk))
        params = [stab_params(P["M"][k], P["Re"][k], P["alpha"][k], P["beta"][k], ny) for k in idx]
        profs = [erf_profile(P["M"][k], P["width"][k]) for k in idx]
        eig, err, iters, st, vecs = ctx.solve_batch(params, profs, sg.MODE_PLAIN, want_vectors=True)
        for j, k in enumerate(idx):
            c = eig[j] / P["alpha"][k]
            # phase speeds outside (0, 3) are the unresolved acoustic modes of
            # the near-incompressible end (|c| up to 10 (1 + 1/M) passes the
            # selection filter): kept out of the training targets
            if st[j] == sg.ST_OK and np.all(np.isfinite(vecs[j])) and 0.0 < c.real < 3.0 and abs(c.imag) < 0.2:
                ok[k] = True
                w[k] = eig[j]
                coef[k] = chebyshev_coefficients(vecs[j], ny)
    return {"params": P, "omega": w, "coef": coef, "valid": ok, "seconds": time.perf_counter() - t0}


def init_params(sizes=SIZES, seed: int = 0) -> np.ndarray:
    """He-uniform weights, zero biases, packed [W_0, b_0, ...]."""
    rng = np.random.default_rng(seed)
    out = []
    for k, n in zip(sizes[:-1], sizes[1:]):
        out.append((rng.uniform(-1.0, 1.0, size=(k, n)) * math.sqrt(6.0 / k)).astype(np.float32).ravel())
        out.append(np.zeros(n, dtype=np.float32))
    return np.concatenate(out)


class Surrogate:
    """The seeding network plus its target standardisation."""

    def __init__(self, ctx: sg.Context, max_batch: int = 8192, seed: int = 0):
        import torch
        self.torch = torch
        self.ctx = ctx
        self.max_batch = int(max_batch)
        self.net = sg.Network(ctx, SIZES, self.max_batch)
        self.net.set_params(init_params(SIZES, seed))
        self.mean = np.zeros(SIZES[-1], dtype=np.float64)
        self.std = np.ones(SIZES[-1], dtype=np.float64)

    # -- encoding -------------------------------------------------------------
    @staticmethod
    def raw_targets(omega, alpha, coef) -> np.ndarray:
        a = np.asarray(alpha, dtype=np.float64)
        w = np.asarray(omega, dtype=np.complex128)
        c = np.asarray(coef, dtype=np.complex128).reshape(len(w), -1)
        t = np.empty((len(w), SIZES[-1]), dtype=np.float64)
        t[:, 0] = w.real / a
        t[:, 1] = 100.0 * w.imag / a
        t[:, 2::2] = c.real
        t[:, 3::2] = c.imag
        return t

    def decode(self, y: np.ndarray, alpha) -> tuple:
        t = y.astype(np.float64) * self.std + self.mean
        a = np.asarray(alpha, dtype=np.float64)
        w = a * t[:, 0] + 1j * a * t[:, 1] / 100.0
        coef = (t[:, 2::2] + 1j * t[:, 3::2]).reshape(len(t), 5, NCHEB)
        return w, coef

    # -- training -------------------------------------------------------------
    def fit(self, X: np.ndarray, omega, alpha, coef, steps: int = 2000, batch: int = 1024, lr: float = 1e-3,
            lr_min: float = 2e-5, seed: int = 0) -> dict:
        """Adam with a cosine learning rate, minibatches drawn per epoch from a
        host permutation and read as contiguous slices of device arrays."""
        torch = self.torch
        T = self.raw_targets(omega, alpha, coef)
        self.mean = T.mean(axis=0)
        self.std = np.maximum(T.std(axis=0), 1e-6)
        Tn = ((T - self.mean) / self.std).astype(np.float32)
        X = np.ascontiguousarray(X, dtype=np.float32)
        n = len(X)
        batch = min(batch, n, self.max_batch)
        dev = torch.device("cuda", torch.cuda.current_device())
        w = torch.from_numpy(LOSS_WEIGHTS).to(dev)
        rng = np.random.default_rng(seed)
        per_epoch = max(1, n // batch)
        losses = []
        t0 = time.perf_counter()
        xs = ts = None
        for step in range(steps):
            e, j = divmod(step, per_epoch)
            if j == 0:
                perm = rng.permutation(n)
                xs = torch.from_numpy(X[perm]).to(dev)
                ts = torch.from_numpy(Tn[perm]).to(dev)
            rate = lr_min + 0.5 * (lr - lr_min) * (1.0 + math.cos(math.pi * step / max(1, steps - 1)))
            xp = xs.data_ptr() + j * batch * X.shape[1] * 4
            tp = ts.data_ptr() + j * batch * Tn.shape[1] * 4
            want = (step % 100 == 0) or step == steps - 1
            loss = self.net.train_step(batch, xp, tp, w.data_ptr(), rate, want_loss=want)
            if want:
                losses.append((step, loss))
        torch.cuda.synchronize()
        return {"losses": losses, "seconds": time.perf_counter() - t0, "steps": steps, "batch": batch}

    # -- inference ------------------------------------------------------------
    def predict(self, X: np.ndarray, alpha) -> tuple:
        torch = self.torch
        X = np.ascontiguousarray(X, dtype=np.float32)
        n = len(X)
        dev = torch.device("cuda", torch.cuda.current_device())
        out = np.empty((n, SIZES[-1]), dtype=np.float32)
        y = torch.empty((self.max_batch, SIZES[-1]), dtype=torch.float32, device=dev)
        for k0 in range(0, n, self.max_batch):
            b = min(self.max_batch, n - k0)
            x = torch.from_numpy(X[k0:k0 + b]).to(dev)
            self.net.forward(b, x.data_ptr(), y.data_ptr())
            self.ctx.sync()
            out[k0:k0 + b] = y[:b].cpu().numpy()
        return self.decode(out, alpha)

    def seed_batch(self, batch: "sg.Batch", X: np.ndarray, alpha) -> np.ndarray:
        """Predicted seeds and start vectors onto a batch; returns the seeds."""
        w, coef = self.predict(X, alpha)
        batch.set_seeds(w)
        batch.set_start(coef)
        return w

    def save(self, path: str) -> None:
        np.savez(path, params=self.net.get_params(), mean=self.mean, std=self.std, sizes=np.asarray(SIZES))

    def load(self, path: str) -> None:
        z = np.load(path)
        if tuple(z["sizes"]) != SIZES:
            raise ValueError("network shape mismatch")
        self.net.set_params(z["params"])
        self.mean, self.std = z["mean"], z["std"]

    def close(self) -> None:
        self.net.close()
