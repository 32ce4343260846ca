"""stab_gb300: GB300 (sm_103a) implementation of stab's Chebyshev
linear-stability hot path, behind the C ABI of ``include/stab_gb300.h``.

This module is a thin ctypes mirror of that ABI.  It loads the in-tree
``libstab_gb300.so`` (built by ``stab_gb300/build.py``) and raises if the
library is missing: there is no CPU fallback.

The reference's own entry points are Fortran subroutines (``temporal(name,
ind)``, ``spatial(name, ind)`` in temporal.f90:2 and spatial.f90:2) fed from
module ``stuff``; here the same run parameters travel in ``StabParams`` and
the mean profile as an (nym, 6) array of ``y rho u v w T`` rows.
"""
from __future__ import annotations

import ctypes
import os
import weakref
from typing import Optional, Sequence

import numpy as np

__all__ = ["StabParams", "Sweep", "parse_sweep_input", "read_delta", "read_body", "eig_name", "stab_out_line",
           "sweep_points", "EvecHeader", "Context", "Network", "load", "LIB_PATH", "parse_input", "profile_name",
           "read_profile", "grid", "write_evec", "read_evec", "getevec_select", "eigfunction_text", "MODE_PLAIN", "MODE_SEEDED", "MODE_COARSE", "MODE_SURROGATE", "MODE_TRACK",
           "ST_OK", "ST_SINGULAR", "ST_NOCONV", "ST_NAN", "ST_FELLBACK", "ST_NOMODE", "ST_UNVERIFIED",
           "StabError"]

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libstab_gb300.so")

MODE_PLAIN, MODE_SEEDED, MODE_COARSE, MODE_SURROGATE, MODE_TRACK = 0, 1, 2, 3, 4
# arithmetic per stage (stab_set_arithmetic)
STAGE_SEED_EIG, STAGE_PLAIN_EIG, STAGE_RETRY_LU, STAGE_POLISH_LU = 0, 1, 2, 3
ARITH_FP64, ARITH_DOUBLE_WORD, ARITH_FP32, ARITH_TF32_SPLIT = 0, 1, 2, 3
OPT_SEED_QR_SHARED, OPT_POLISH_LU_TMA, OPT_EIG_RESIDENT, OPT_EIG_THREADS, OPT_EIG_MID, OPT_SEED_VECTORS = 1, 2, 3, 4, 5, 6
OPT_PARALLEL_CANDIDATES, OPT_MEDIUM_NY, OPT_FIRST_RETRY, OPT_LEVEL_CONSISTENCY = 7, 8, 9, 10
OPT_MEDIUM_NY_SPATIAL, OPT_MLP_TCGEN05 = 11, 12
ST_OK, ST_SINGULAR, ST_NOCONV, ST_NAN, ST_FELLBACK, ST_NOMODE, ST_UNVERIFIED = 0, 1, 2, 3, 4, 5, 6

EXPORTED = (
    "stab_abi_version", "stab_create", "stab_destroy", "stab_last_error", "stab_set_stream", "stab_sync",
    "stab_set_profiling", "stab_kernel_stats", "stab_reset_kernel_stats", "stab_assemble",
    "stab_full_spectrum", "stab_batch_create", "stab_batch_set_seeds", "stab_batch_run",
    "stab_batch_results", "stab_batch_work", "stab_batch_destroy", "stab_solve_batch",
    "stab_eigvals_noalloc", "stab_eigenvectors", "stab_parse_input", "stab_parse_sweep_input",
    "stab_read_delta", "stab_read_body", "stab_eig_name", "stab_stab_out_line", "stab_sweep_points", "stab_profile_name", "stab_read_profile",
    "stab_grid", "stab_fd_grid", "stab_write_evec", "stab_read_evec", "stab_getevec_select", "stab_eigfunction_text",
    "stab_mlp_create", "stab_mlp_param_count", "stab_mlp_set_params", "stab_mlp_get_params", "stab_mlp_forward",
    "stab_mlp_gradients", "stab_mlp_train_step", "stab_mlp_destroy", "stab_batch_set_start", "stab_batch_counts",
    "stab_batch_spectra", "stab_autotune", "stab_eig_phases", "stab_lu_cluster_check", "stab_lu_tc_check", "stab_peak_rates", "stab_set_option", "stab_set_arithmetic", "stab_set_seed_size",
)


class StabError(RuntimeError):
    pass


class EvecHeader(ctypes.Structure):
    """Mirror of ``stab_evec_header``: records R1-R3 of evec.dat."""

    _fields_ = [(k, ctypes.c_int32) for k in ("ind", "ny", "ndof", "itype", "ievec", "curve", "top", "wall",
                                              "wallt", "ider", "nmax", "has_vectors")] + [
        ("omega", ctypes.c_double * 2), ("alpha", ctypes.c_double * 2), ("beta", ctypes.c_double * 2)] + [
        (k, ctypes.c_double) for k in ("Re", "Ma", "Pr", "x", "yi", "ymax")]


class StabParams(ctypes.Structure):
    """Mirror of ``stab_params`` (module ``stuff``, stuff.f90:11-55)."""

    _fields_ = [
        ("mattyp", ctypes.c_int32), ("ny", ctypes.c_int32), ("ievec", ctypes.c_int32),
        ("ider", ctypes.c_int32), ("top", ctypes.c_int32), ("wall", ctypes.c_int32),
        ("wallt", ctypes.c_int32), ("curve", ctypes.c_int32), ("itype", ctypes.c_int32),
        ("ind", ctypes.c_int32),
        ("T0", ctypes.c_double), ("Ma", ctypes.c_double), ("Re", ctypes.c_double),
        ("Pr", ctypes.c_double), ("yi", ctypes.c_double), ("ymax", ctypes.c_double),
        ("x", ctypes.c_double),
        ("alpha", ctypes.c_double * 2), ("beta", ctypes.c_double * 2), ("omega", ctypes.c_double * 2),
    ]

    @classmethod
    def make(cls, *, itype=1, ny=64, Ma=0.5, Re=1000.0, Pr=0.72, mattyp=1, T0=110.4 / 0.3815,
             yi=1.0 / 23.0, ymax=50.0, alpha=0j, beta=0j, omega=0j, top=0, wall=0, wallt=0,
             ievec=1, ind=0, x=0.0):
        p = cls()
        p.mattyp, p.ny, p.ievec, p.ider = mattyp, ny, ievec, 1
        p.top, p.wall, p.wallt, p.curve, p.itype, p.ind = top, wall, wallt, 0, itype, ind
        p.T0, p.Ma, p.Re, p.Pr, p.yi, p.ymax, p.x = T0, Ma, Re, Pr, yi, ymax, x
        a, b, w = complex(alpha), complex(beta), complex(omega)
        p.alpha[0], p.alpha[1] = a.real, a.imag
        p.beta[0], p.beta[1] = b.real, b.imag
        p.omega[0], p.omega[1] = w.real, w.imag
        return p

    def n(self) -> int:
        return 5 * self.ny

    def m(self) -> int:
        return 2 * self.n() if self.itype in (2, 4) else self.n()


class Sweep(ctypes.Structure):
    """Mirror of ``stab_sweep``: the ranges of the multi-point drivers
    (itype 7: mtemporal.f90:20-23; itype 8: mspatial.f90:20-27)."""

    _fields_ = [("itype", ctypes.c_int32), ("dtype", ctypes.c_int32), ("ind1", ctypes.c_int32),
                ("ind2", ctypes.c_int32), ("ind_inc", ctypes.c_int32), ("p_min", ctypes.c_double),
                ("p_max", ctypes.c_double), ("p_inc", ctypes.c_double), ("b_min", ctypes.c_double),
                ("b_max", ctypes.c_double), ("b_inc", ctypes.c_double)]


_lib = None


def load(path: str = LIB_PATH):
    """Load the in-tree shared library (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise StabError(f"{path} is missing: run `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = ctypes.CDLL(path)
    P = ctypes.POINTER
    vp = ctypes.c_void_p
    i32, i64, dbl = ctypes.c_int32, ctypes.c_int64, ctypes.c_double
    lib.stab_abi_version.restype = ctypes.c_int
    lib.stab_create.argtypes = [P(vp), ctypes.c_int]
    lib.stab_destroy.argtypes = [vp]
    lib.stab_last_error.argtypes = [vp]
    lib.stab_last_error.restype = ctypes.c_char_p
    lib.stab_set_stream.argtypes = [vp, vp]
    lib.stab_sync.argtypes = [vp]
    lib.stab_set_profiling.argtypes = [vp, ctypes.c_int]
    lib.stab_kernel_stats.argtypes = [vp, i32, P(ctypes.c_char_p), P(i64), P(dbl), P(i32)]
    lib.stab_reset_kernel_stats.argtypes = [vp]
    lib.stab_assemble.argtypes = [vp, P(StabParams), i32, P(dbl), P(dbl)]
    lib.stab_full_spectrum.argtypes = [vp, P(StabParams), i32, P(dbl), P(dbl), P(dbl), P(i32), P(i32)]
    lib.stab_batch_create.argtypes = [vp, i32, P(StabParams), P(i32), P(P(dbl)), P(vp)]
    lib.stab_batch_set_seeds.argtypes = [vp, P(dbl)]
    lib.stab_batch_run.argtypes = [vp, i32]
    lib.stab_batch_results.argtypes = [vp, P(dbl), P(dbl), P(i32), P(i32), P(P(dbl))]
    lib.stab_batch_destroy.argtypes = [vp]
    lib.stab_batch_work.argtypes = [vp, P(dbl)]
    lib.stab_eigvals_noalloc.argtypes = [vp, i32, vp, vp, vp]
    lib.stab_solve_batch.argtypes = [vp, i32, P(StabParams), P(i32), P(P(dbl)), i32, P(dbl), P(dbl), P(dbl),
                                     P(i32), P(P(dbl))]
    lib.stab_eigenvectors.argtypes = [vp, P(StabParams), i32, P(dbl), i32, P(dbl), P(dbl), P(i32)]
    lib.stab_parse_input.argtypes = [ctypes.c_char_p, P(StabParams), ctypes.c_char_p, ctypes.c_size_t]
    lib.stab_parse_sweep_input.argtypes = [ctypes.c_char_p, P(StabParams), P(Sweep), ctypes.c_char_p,
                                           ctypes.c_size_t]
    lib.stab_read_delta.argtypes = [ctypes.c_char_p, i32, P(dbl), P(dbl), P(i32)]
    lib.stab_read_body.argtypes = [ctypes.c_char_p, i32, P(dbl), P(i32)]
    lib.stab_eig_name.argtypes = [i32, ctypes.c_char_p, ctypes.c_size_t]
    lib.stab_stab_out_line.argtypes = [i32, i32, dbl, dbl, dbl, ctypes.c_char_p, ctypes.c_size_t]
    lib.stab_sweep_points.argtypes = [P(StabParams), P(Sweep), i32, P(dbl), P(dbl), i32, P(StabParams), P(i32)]
    lib.stab_profile_name.argtypes = [i32, ctypes.c_char_p, ctypes.c_size_t]
    lib.stab_read_profile.argtypes = [ctypes.c_char_p, i32, P(dbl), P(i32)]
    lib.stab_grid.argtypes = [i32, dbl, dbl, P(dbl), P(dbl), P(dbl), P(dbl)]
    lib.stab_fd_grid.argtypes = [i32, dbl, dbl, P(dbl), P(dbl), P(dbl), P(dbl)]
    lib.stab_write_evec.argtypes = [ctypes.c_char_p, P(StabParams), P(dbl), P(dbl)]
    lib.stab_read_evec.argtypes = [ctypes.c_char_p, P(EvecHeader), P(dbl), P(dbl), P(dbl)]
    lib.stab_getevec_select.argtypes = [P(dbl), i32, dbl, dbl]
    lib.stab_getevec_select.restype = i32
    lib.stab_eigfunction_text.argtypes = [P(EvecHeader), P(dbl), P(dbl), P(dbl), ctypes.c_char_p, i64]
    lib.stab_eigfunction_text.restype = i64
    f32p = P(ctypes.c_float)
    lib.stab_mlp_create.argtypes = [vp, i32, P(i32), i32, P(vp)]
    lib.stab_mlp_param_count.argtypes = [vp]
    lib.stab_mlp_param_count.restype = i64
    lib.stab_mlp_set_params.argtypes = [vp, f32p]
    lib.stab_mlp_get_params.argtypes = [vp, f32p, f32p]
    lib.stab_mlp_forward.argtypes = [vp, i32, vp, vp]
    lib.stab_mlp_gradients.argtypes = [vp, i32, vp, vp, vp, P(dbl)]
    lib.stab_mlp_train_step.argtypes = [vp, i32, vp, vp, vp, ctypes.c_float, P(dbl)]
    lib.stab_mlp_destroy.argtypes = [vp]
    lib.stab_batch_set_start.argtypes = [vp, P(dbl), i32]
    lib.stab_batch_counts.argtypes = [vp, P(i32)]
    lib.stab_batch_spectra.argtypes = [vp, P(P(dbl))]
    lib.stab_autotune.argtypes = [vp, P(i32), i32, P(i32), P(ctypes.c_float)]
    lib.stab_eig_phases.argtypes = [vp, P(ctypes.c_uint64), i32]
    lib.stab_set_arithmetic.argtypes = [vp, i32, i32]
    lib.stab_set_seed_size.argtypes = [vp, i32]
    lib.stab_lu_cluster_check.argtypes = [vp, i32, i32, i32, P(dbl), P(i32)]
    lib.stab_lu_tc_check.argtypes = [vp, i32, i32, P(dbl), P(dbl), P(i32)]
    lib.stab_peak_rates.argtypes = [vp, P(dbl)]
    lib.stab_set_option.argtypes = [vp, i32, i32]
    _lib = lib
    return lib


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _iptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


def _prof(profile) -> np.ndarray:
    a = np.ascontiguousarray(profile, dtype=np.float64)
    if a.ndim != 2 or a.shape[1] not in (6, 18):
        raise ValueError("profile must be (nym, 6): y rho u v w T, or (nym, 18) with the derivative tables "
                         "(ider = 0)")
    return a


class Batch:
    """A device-resident batch (``stab_batch_*``)."""

    def __init__(self, ctx: "Context", params: Sequence[StabParams], profiles: Sequence[np.ndarray]):
        self.ctx = ctx
        self.lib = ctx.lib
        self.count = len(params)
        self.params = (StabParams * self.count)(*params)
        self._profiles = [_prof(p) for p in profiles]
        # identical arrays share one upload
        ptrs = (ctypes.POINTER(ctypes.c_double) * self.count)(*[_dptr(p) for p in self._profiles])
        nym = np.array([p.shape[0] for p in self._profiles], dtype=np.int32)
        h = ctypes.c_void_p()
        ctx._check(self.lib.stab_batch_create(ctx.h, self.count, self.params, _iptr(nym), ptrs, ctypes.byref(h)))
        self.h = h
        ctx._batches.add(self)

    def set_seeds(self, seeds) -> None:
        s = np.ascontiguousarray(np.asarray(seeds, dtype=np.complex128)).view(np.float64)
        self.ctx._check(self.lib.stab_batch_set_seeds(self.h, _dptr(s)))

    def set_start(self, coef) -> None:
        """Chebyshev coefficients of start vectors: (count, 5, ncheb) complex."""
        a = np.ascontiguousarray(np.asarray(coef, dtype=np.complex128))
        if a.ndim != 3 or a.shape[0] != self.count or a.shape[1] != 5:
            raise ValueError("coef must be (count, 5, ncheb)")
        self._start = a
        self.ctx._check(self.lib.stab_batch_set_start(self.h, _dptr(a.view(np.float64)), a.shape[2]))

    def run(self, mode: int) -> None:
        self.ctx._check(self.lib.stab_batch_run(self.h, int(mode)))

    def spectra(self) -> list:
        """Sorted full spectra after a MODE_PLAIN run (stab_batch_spectra)."""
        out = [np.zeros(p.m(), dtype=np.complex128) for p in self.params]
        ptrs = (ctypes.POINTER(ctypes.c_double) * self.count)(*[_dptr(v.view(np.float64)) for v in out])
        self.ctx._check(self.lib.stab_batch_spectra(self.h, ptrs))
        return out

    def counts(self) -> dict:
        """Where the last run resolved its instances (stab_batch_counts)."""
        c = np.zeros(3, dtype=np.int32)
        self.ctx._check(self.lib.stab_batch_counts(self.h, _iptr(c)))
        return {"first_stage": int(c[0]), "surrogate_seed": int(c[1]), "fp64_fallback": int(c[2])}

    def results(self, want_vectors: bool = False):
        n = self.count
        eig = np.zeros(n, dtype=np.complex128)
        err = np.zeros(n)
        iters = np.zeros(n, dtype=np.int32)
        status = np.zeros(n, dtype=np.int32)
        vecs = None
        vptr = None
        if want_vectors:
            vecs = [np.zeros(p.m(), dtype=np.complex128) for p in self.params]
            vptr = (ctypes.POINTER(ctypes.c_double) * n)(*[_dptr(v.view(np.float64)) for v in vecs])
        self.ctx._check(self.lib.stab_batch_results(self.h, _dptr(eig.view(np.float64)), _dptr(err), _iptr(iters),
                                                    _iptr(status), vptr))
        return eig, err, iters, status, vecs

    def work(self) -> dict:
        """Algorithmic flops of the last run (see stab_batch_work)."""
        w = np.zeros(4)
        self.ctx._check(self.lib.stab_batch_work(self.h, _dptr(w)))
        return {"eig_fp64": w[0], "eig_fp64_coarse": w[1], "lu_c64": w[2], "lu_c128": w[3]}

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.stab_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Network:
    """A ``stab_mlp``: BF16 MLP trained and run by the library's kernels.

    Device arrays are passed as raw device addresses (``tensor.data_ptr()``
    of contiguous float32 CUDA tensors): row-major batch x width."""

    def __init__(self, ctx: "Context", sizes: Sequence[int], max_batch: int):
        self.ctx = ctx
        self.lib = ctx.lib
        self.sizes = tuple(int(v) for v in sizes)
        arr = np.asarray(self.sizes, dtype=np.int32)
        h = ctypes.c_void_p()
        ctx._check(self.lib.stab_mlp_create(ctx.h, len(arr) - 1, _iptr(arr), int(max_batch), ctypes.byref(h)))
        self.h = h
        self.max_batch = int(max_batch)
        self.count = int(self.lib.stab_mlp_param_count(self.h))
        ctx._nets.add(self)

    def set_params(self, params: np.ndarray) -> None:
        a = np.ascontiguousarray(params, dtype=np.float32)
        if a.size != self.count:
            raise ValueError(f"expected {self.count} parameters")
        self.ctx._check(self.lib.stab_mlp_set_params(self.h, a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))

    def get_params(self, grads: bool = False):
        p = np.zeros(self.count, dtype=np.float32)
        g = np.zeros(self.count, dtype=np.float32) if grads else None
        fp = ctypes.POINTER(ctypes.c_float)
        self.ctx._check(self.lib.stab_mlp_get_params(self.h, p.ctypes.data_as(fp),
                                                     g.ctypes.data_as(fp) if grads else None))
        return (p, g) if grads else p

    def forward(self, batch: int, x_ptr: int, y_ptr: int) -> None:
        self.ctx._check(self.lib.stab_mlp_forward(self.h, int(batch), ctypes.c_void_p(x_ptr), ctypes.c_void_p(y_ptr)))

    def gradients(self, batch: int, x_ptr: int, t_ptr: int, w_ptr: int) -> float:
        loss = ctypes.c_double(0.0)
        self.ctx._check(self.lib.stab_mlp_gradients(self.h, int(batch), ctypes.c_void_p(x_ptr), ctypes.c_void_p(t_ptr),
                                                    ctypes.c_void_p(w_ptr), ctypes.byref(loss)))
        return loss.value

    def train_step(self, batch: int, x_ptr: int, t_ptr: int, w_ptr: int, lr: float, want_loss: bool = False):
        loss = ctypes.c_double(0.0)
        self.ctx._check(self.lib.stab_mlp_train_step(self.h, int(batch), ctypes.c_void_p(x_ptr), ctypes.c_void_p(t_ptr),
                                                     ctypes.c_void_p(w_ptr), float(lr),
                                                     ctypes.byref(loss) if want_loss else None))
        return loss.value if want_loss else None

    def split(self, flat: np.ndarray) -> list:
        """Packed parameters -> [(W_l, b_l)] views."""
        out, o = [], 0
        for k, n in zip(self.sizes[:-1], self.sizes[1:]):
            W = flat[o:o + k * n].reshape(k, n)
            o += k * n
            out.append((W, flat[o:o + n]))
            o += n
        return out

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.stab_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Context:
    """A ``stab_ctx`` on one CUDA device."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = ctypes.c_void_p()
        self._batches = weakref.WeakSet()
        self._nets = weakref.WeakSet()
        rc = self.lib.stab_create(ctypes.byref(h), int(device))
        if rc != 0:
            raise StabError(f"stab_create failed ({rc}): no usable CUDA device {device}")
        self.h = h
        self.device = int(device)

    def close(self) -> None:
        if getattr(self, "h", None):
            for b in list(self._batches):
                b.close()
            for m in list(self._nets):
                m.close()
            self.lib.stab_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int) -> None:
        if rc != 0:
            msg = self.lib.stab_last_error(self.h)
            raise StabError(f"stab call failed ({rc}): {msg.decode() if msg else ''}")

    # -- profiling ---------------------------------------------------------
    def set_stream(self, stream_handle: Optional[int]) -> None:
        self._check(self.lib.stab_set_stream(self.h, ctypes.c_void_p(stream_handle or 0)))

    def sync(self) -> None:
        self._check(self.lib.stab_sync(self.h))

    def set_profiling(self, on: bool) -> None:
        self._check(self.lib.stab_set_profiling(self.h, 1 if on else 0))

    def kernel_stats(self) -> dict:
        cnt = ctypes.c_int32(0)
        self._check(self.lib.stab_kernel_stats(self.h, -1, None, None, None, ctypes.byref(cnt)))
        out = {}
        for k in range(cnt.value):
            name = ctypes.c_char_p()
            la = ctypes.c_int64()
            ms = ctypes.c_double()
            self._check(self.lib.stab_kernel_stats(self.h, k, ctypes.byref(name), ctypes.byref(la),
                                                   ctypes.byref(ms), None))
            out[name.value.decode()] = (la.value, ms.value)
        return out

    def autotune(self, orders: Sequence[int]) -> dict:
        """Tune the LU panel width per order (stab_autotune): {n: {"c64": (nb, ms), "c128": (nb, ms)}}."""
        o = np.asarray(orders, dtype=np.int32)
        nb = np.zeros(2 * len(o), dtype=np.int32)
        ms = np.zeros(2 * len(o), dtype=np.float32)
        self._check(self.lib.stab_autotune(self.h, _iptr(o), len(o), _iptr(nb),
                                           ms.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
        return {int(n): {"c64": (int(nb[2 * q]), float(ms[2 * q])), "c128": (int(nb[2 * q + 1]), float(ms[2 * q + 1]))}
                for q, n in enumerate(o)}

    def lu_cluster_check(self, n: int, count: int, complex128: bool = True):
        """(max |difference|, differing pivots) of one-CTA vs four-CTA-cluster LU."""
        md = ctypes.c_double(0.0)
        pd = ctypes.c_int32(0)
        self._check(self.lib.stab_lu_cluster_check(self.h, n, count, 1 if complex128 else 0, ctypes.byref(md),
                                                   ctypes.byref(pd)))
        return md.value, pd.value

    def peak_rates(self) -> dict:
        """stab_peak_rates: measured FP32 / FP64 FMA and double-word complex
        multiply-add throughput of this device, TFLOP/s."""
        out = np.zeros(3)
        self._check(self.lib.stab_peak_rates(self.h, _dptr(out)))
        return {"fp32": float(out[0]), "fp64": float(out[1]), "double_word_complex": float(out[2])}

    def set_option(self, option: int, value: int) -> None:
        """stab_set_option: OPT_SEED_QR_SHARED (0 default, 1 on), OPT_POLISH_LU_TMA (1 default, 0 off),
        OPT_EIG_RESIDENT (0 default: occupancy; k: k instances per SM)."""
        self._check(self.lib.stab_set_option(self.h, int(option), int(value)))

    def lu_tc_check(self, n: int, count: int):
        """(backward error with the tensor-core update, backward error on the
        CUDA cores, differing pivots) of count complex64 test LUs of order n
        (stab_lu_tc_check)."""
        bt, bs, pd = ctypes.c_double(), ctypes.c_double(), ctypes.c_int32()
        self._check(self.lib.stab_lu_tc_check(self.h, n, count, ctypes.byref(bt), ctypes.byref(bs),
                                              ctypes.byref(pd)))
        return bt.value, bs.value, pd.value

    DEFAULT_ARITHMETIC = {STAGE_SEED_EIG: ARITH_DOUBLE_WORD, STAGE_PLAIN_EIG: ARITH_FP64,
                          STAGE_RETRY_LU: ARITH_DOUBLE_WORD, STAGE_POLISH_LU: ARITH_TF32_SPLIT}

    def set_arithmetic(self, stage: int, arithmetic: int) -> None:
        """Arithmetic of one stage (stab_set_arithmetic): STAGE_SEED_EIG,
        STAGE_PLAIN_EIG or STAGE_RETRY_LU with ARITH_FP64 or ARITH_DOUBLE_WORD;
        STAGE_POLISH_LU with ARITH_FP32 or ARITH_TF32_SPLIT."""
        self._check(self.lib.stab_set_arithmetic(self.h, int(stage), int(arithmetic)))

    def set_seed_size(self, ny: int = 32) -> None:
        """N of the coarse seed spectrum for batches created afterwards (stab_set_seed_size)."""
        self._check(self.lib.stab_set_seed_size(self.h, int(ny)))

    def reset_arithmetic(self) -> None:
        for st, ar in self.DEFAULT_ARITHMETIC.items():
            self.set_arithmetic(st, ar)

    def eig_phases(self, reset: bool = True) -> dict:
        """SM cycles per phase of the eigensolver (stab_eig_phases)."""
        v = (ctypes.c_uint64 * 6)()
        self._check(self.lib.stab_eig_phases(self.h, v, 1 if reset else 0))
        names = ("isolation", "compaction", "balancing", "hessenberg", "repack", "qr")
        return {k: int(x) for k, x in zip(names, v)}

    def reset_kernel_stats(self) -> None:
        self._check(self.lib.stab_reset_kernel_stats(self.h))

    # -- single instance -------------------------------------------------------
    def assemble(self, p: StabParams, profile) -> list:
        """Dense operators: [A0, B0] (temporal) or [C0, C1, C2] (spatial)."""
        prof = _prof(profile)
        n = p.n()
        k = 3 if p.itype in (2, 4) else 2
        out = np.zeros(k * n * n, dtype=np.complex128)
        self._check(self.lib.stab_assemble(self.h, ctypes.byref(p), prof.shape[0], _dptr(prof),
                                           _dptr(out.view(np.float64))))
        return [out[q * n * n:(q + 1) * n * n].reshape(n, n, order="F") for q in range(k)]

    def full_spectrum(self, p: StabParams, profile, want_vector: bool = True):
        """Sorted spectrum, least-stable eigenvector, its index, status."""
        prof = _prof(profile)
        m = p.m()
        eig = np.zeros(m, dtype=np.complex128)
        vec = np.zeros(m, dtype=np.complex128) if want_vector else None
        li = ctypes.c_int32(-1)
        st = ctypes.c_int32(0)
        self._check(self.lib.stab_full_spectrum(self.h, ctypes.byref(p), prof.shape[0], _dptr(prof),
                                                _dptr(eig.view(np.float64)),
                                                _dptr(vec.view(np.float64)) if want_vector else None,
                                                ctypes.byref(li), ctypes.byref(st)))
        return eig, vec, li.value, st.value

    def eigenvectors(self, p: StabParams, profile, eig) -> tuple:
        """Eigenvectors at the given eigenvalues (columns) and their status."""
        prof = _prof(profile)
        ev = np.ascontiguousarray(eig, dtype=np.complex128)
        m = p.m()
        vec = np.zeros((len(ev), m), dtype=np.complex128)
        st = np.zeros(len(ev), dtype=np.int32)
        self._check(self.lib.stab_eigenvectors(self.h, ctypes.byref(p), prof.shape[0], _dptr(prof), len(ev),
                                               _dptr(ev.view(np.float64)), _dptr(vec.view(np.float64)),
                                               _iptr(st)))
        return vec.T.copy(), st

    # -- batches -------------------------------------------------------------
    def batch(self, params: Sequence[StabParams], profiles: Sequence[np.ndarray]) -> Batch:
        return Batch(self, params, profiles)

    def solve_batch(self, params: Sequence[StabParams], profiles: Sequence[np.ndarray], mode: int,
                    seeds=None, want_vectors: bool = False):
        b = Batch(self, params, profiles)
        try:
            if seeds is not None:
                b.set_seeds(seeds)
            b.run(mode)
            return b.results(want_vectors)
        finally:
            b.close()


# -- the reference's file interface (host only) ---------------------------------
def parse_input(text: str) -> StabParams:
    """``stab < input.dat`` stdin protocol (input.f90:15-123, stab.f90:46-55)."""
    lib = load()
    p = StabParams()
    msg = ctypes.create_string_buffer(256)
    rc = lib.stab_parse_input(text.encode(), ctypes.byref(p), msg, 256)
    if rc:
        raise StabError(f"input: {msg.value.decode()}")
    return p


def parse_sweep_input(text: str):
    """The stdin protocol including the multi-point drivers (itypes 7, 8):
    (StabParams, Sweep) (stab_parse_sweep_input)."""
    lib = load()
    p, sw = StabParams(), Sweep()
    msg = ctypes.create_string_buffer(256)
    rc = lib.stab_parse_sweep_input(text.encode(), ctypes.byref(p), ctypes.byref(sw), msg, 256)
    if rc:
        raise StabError(f"input: {msg.value.decode()}")
    return p, sw


def read_delta(path: str):
    """delta.dat rows (xb, delta) (mspatial.f90:29-63)."""
    lib = load()
    n = ctypes.c_int32()
    if lib.stab_read_delta(path.encode(), 0, None, None, ctypes.byref(n)):
        raise StabError(f"cannot read {path}")
    xb, de = np.zeros(n.value), np.zeros(n.value)
    if lib.stab_read_delta(path.encode(), n.value, _dptr(xb), _dptr(de), ctypes.byref(n)):
        raise StabError(f"cannot read {path}")
    return xb, de


def read_body(path: str) -> np.ndarray:
    """body.dat stations xb (getab.f90:73-86)."""
    lib = load()
    n = ctypes.c_int32()
    if lib.stab_read_body(path.encode(), 0, None, ctypes.byref(n)):
        raise StabError(f"cannot read {path}")
    xb = np.zeros(n.value)
    if lib.stab_read_body(path.encode(), n.value, _dptr(xb), ctypes.byref(n)):
        raise StabError(f"cannot read {path}")
    return xb


def eig_name(iver: int) -> str:
    buf = ctypes.create_string_buffer(64)
    if load().stab_eig_name(iver, buf, 64):
        raise StabError("iver out of range")
    return buf.value.decode()


def stab_out_line(p: float, value: complex, ind=None) -> str:
    """One stab.out / parm.new line (stab_stab_out_line)."""
    buf = ctypes.create_string_buffer(160)
    v = complex(value)
    rc = load().stab_stab_out_line(0 if ind is None else 1, 0 if ind is None else int(ind), float(p), v.real, v.imag,
                                   buf, 160)
    if rc < 0:
        raise StabError("line does not fit")
    return buf.value.decode()


def sweep_points(base: StabParams, sw: Sweep, xb=None, delta=None):
    """The solves of a sweep in the reference's loop order (stab_sweep_points)."""
    lib = load()
    nb = 0 if xb is None else len(xb)
    xa = None if xb is None else np.ascontiguousarray(xb, dtype=np.float64)
    da = None if delta is None else np.ascontiguousarray(delta, dtype=np.float64)
    n = ctypes.c_int32()
    if lib.stab_sweep_points(ctypes.byref(base), ctypes.byref(sw), nb, _dptr(xa) if xa is not None else None,
                             _dptr(da) if da is not None else None, 0, None, ctypes.byref(n)):
        raise StabError("invalid sweep")
    pts = (StabParams * max(n.value, 1))()
    if lib.stab_sweep_points(ctypes.byref(base), ctypes.byref(sw), nb, _dptr(xa) if xa is not None else None,
                             _dptr(da) if da is not None else None, n.value, pts, ctypes.byref(n)):
        raise StabError("invalid sweep")
    return [pts[k] for k in range(n.value)]


def profile_name(ind: int) -> str:
    buf = ctypes.create_string_buffer(64)
    if load().stab_profile_name(ind, buf, 64):
        raise StabError("profile index out of range")
    return buf.value.decode()


def read_profile(path: str) -> np.ndarray:
    """profile.<ind> rows (nym, 6): y rho u v w T (getmean.f90:27-80)."""
    lib = load()
    n = ctypes.c_int32(0)
    rc = lib.stab_read_profile(path.encode(), 0, None, ctypes.byref(n))
    if rc:
        raise StabError(f"cannot read {path} ({rc})")
    rows = np.zeros((n.value, 6), dtype=np.float64)
    rc = lib.stab_read_profile(path.encode(), n.value, _dptr(rows), ctypes.byref(n))
    if rc:
        raise StabError(f"cannot read {path} ({rc})")
    return rows


def grid(ny: int, yi: float, ymax: float):
    """y, eta, deta, d2eta of the collocation grid (sgengrid.f90:18-45)."""
    out = [np.zeros(ny) for _ in range(4)]
    if load().stab_grid(ny, yi, ymax, *[_dptr(a) for a in out]):
        raise StabError("bad grid arguments")
    return tuple(out)


def fd_grid(ny: int, yi: float, ymax: float):
    """y, eta, deta, d2eta of the finite-difference grid (ogengrid.f90:20-44),
    wall first."""
    out = [np.zeros(ny) for _ in range(4)]
    if load().stab_fd_grid(ny, yi, ymax, *[_dptr(a) for a in out]):
        raise StabError("bad grid arguments")
    return tuple(out)


def write_evec(path: str, p: StabParams, eig, vecs=None) -> None:
    """evec.dat (temporal.f90:883-890, spatial.f90:1120-1126); vecs (m, m)."""
    ev = np.ascontiguousarray(eig, dtype=np.complex128)
    vp = None
    if vecs is not None:
        va = np.asfortranarray(vecs, dtype=np.complex128)
        vp = va.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    rc = load().stab_write_evec(path.encode(), ctypes.byref(p), _dptr(ev.view(np.float64)), vp)
    if rc:
        raise StabError(f"cannot write {path} ({rc})")


def read_evec(path: str):
    """(header, y, eigenvalues, eigenvectors or None) of an evec.dat."""
    lib = load()
    h = EvecHeader()
    if lib.stab_read_evec(path.encode(), ctypes.byref(h), None, None, None):
        raise StabError(f"cannot read {path}")
    y = np.zeros(h.ny)
    eig = np.zeros(h.nmax, dtype=np.complex128)
    vec = np.zeros((h.nmax, h.nmax), dtype=np.complex128, order="F") if h.has_vectors else None
    rc = lib.stab_read_evec(path.encode(), ctypes.byref(h), _dptr(y), _dptr(eig.view(np.float64)),
                            vec.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) if vec is not None else None)
    if rc:
        raise StabError(f"cannot read {path}")
    return h, y, eig, vec


def getevec_select(eig, value: complex) -> int:
    """getevec -v: 0-based index of the nearest eigenvalue (first wins)."""
    ev = np.ascontiguousarray(eig, dtype=np.complex128)
    return int(load().stab_getevec_select(_dptr(ev.view(np.float64)), len(ev), value.real, value.imag))


def eigfunction_text(h: EvecHeader, y, eig_j: complex, vec_j) -> str:
    """time.N / space.N text of one eigenpair (getevec.f90:176-227)."""
    lib = load()
    ya = np.ascontiguousarray(y, dtype=np.float64)
    e = np.array([eig_j], dtype=np.complex128)
    v = np.ascontiguousarray(vec_j, dtype=np.complex128)
    args = (ctypes.byref(h), _dptr(ya), _dptr(e.view(np.float64)), _dptr(v.view(np.float64)))
    n = lib.stab_eigfunction_text(*args, None, 0)
    if n < 0:
        raise StabError("bad eigenfunction arguments")
    buf = ctypes.create_string_buffer(n + 1)
    lib.stab_eigfunction_text(*args, buf, n + 1)
    return buf.value.decode()
