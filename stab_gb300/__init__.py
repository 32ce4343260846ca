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

__all__ = ["StabParams", "Context", "load", "LIB_PATH", "MODE_PLAIN", "MODE_SEEDED", "MODE_COARSE",
           "ST_OK", "ST_SINGULAR", "ST_NOCONV", "ST_NAN", "ST_FELLBACK", "ST_NOMODE", "StabError"]

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libstab_gb300.so")

MODE_PLAIN, MODE_SEEDED, MODE_COARSE = 0, 1, 2
ST_OK, ST_SINGULAR, ST_NOCONV, ST_NAN, ST_FELLBACK, ST_NOMODE = 0, 1, 2, 3, 4, 5

EXPORTED = (
    "stab_abi_version", "stab_create", "stab_destroy", "stab_last_error", "stab_set_stream", "stab_sync",
    "stab_set_profiling", "stab_kernel_stats", "stab_reset_kernel_stats", "stab_assemble",
    "stab_full_spectrum", "stab_batch_create", "stab_batch_set_seeds", "stab_batch_run",
    "stab_batch_results", "stab_batch_work", "stab_batch_destroy", "stab_solve_batch",
    "stab_eigvals_noalloc",
)


class StabError(RuntimeError):
    pass


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
        return self.n() if self.itype == 1 else 2 * self.n()


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
    _lib = lib
    return lib


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _iptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


def _prof(profile) -> np.ndarray:
    a = np.ascontiguousarray(profile, dtype=np.float64)
    if a.ndim != 2 or a.shape[1] != 6:
        raise ValueError("profile must be (nym, 6): y rho u v w T")
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

    def run(self, mode: int) -> None:
        self.ctx._check(self.lib.stab_batch_run(self.h, int(mode)))

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


class Context:
    """A ``stab_ctx`` on one CUDA device."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = ctypes.c_void_p()
        self._batches = weakref.WeakSet()
        rc = self.lib.stab_create(ctypes.byref(h), int(device))
        if rc != 0:
            raise StabError(f"stab_create failed ({rc}): no usable CUDA device {device}")
        self.h = h

    def close(self) -> None:
        if getattr(self, "h", None):
            for b in list(self._batches):
                b.close()
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

    def reset_kernel_stats(self) -> None:
        self._check(self.lib.stab_reset_kernel_stats(self.h))

    # -- single instance -------------------------------------------------------
    def assemble(self, p: StabParams, profile) -> list:
        """Dense operators: [A0, B0] (temporal) or [C0, C1, C2] (spatial)."""
        prof = _prof(profile)
        n = p.n()
        k = 2 if p.itype == 1 else 3
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
