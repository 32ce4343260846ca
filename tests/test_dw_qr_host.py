"""Double-word eigensolver of the seed spectra, built for the CPU.

tests/host/dw_qr_host.cpp compiles the per-instance eigensolver
(stab_gb300/csrc/qr.cuh, eig_body.cuh) with g++, the 32 threads of a warp run
as std::threads.  Two entry points: the QR iteration alone on a Hessenberg
matrix, and the whole kernel body (isolation, compaction, balancing,
Hessenberg reduction, QR) on a standard-form matrix.  The input is the balanced, power-of-two scaled Hessenberg form
of a temporal operator X = B0^-1 A0 (temporal.f90:771-803) or of a spatial
companion matrix (spatial.f90:972-1016) at small N, which the test builds
with the oracle and scipy; the reference spectrum is numpy's.

Tolerances:
  complex128 QR     each of the 8 least-stable eigenvalues within 1e-12
                    relative of numpy's
  double-word QR    the same 8 within 1e-11 relative (about 48 significant
                    bits against 53; the seeds need 1e-9), and every
                    eigenvalue within 1e-9 absolute (the matrix is scaled to
                    a largest entry near 1)
  both converge, and the double-word QR in no more than 1.5x the 2-element
  reflector applications of the complex128 one
Whole body (one warp, and the batch kernel's four warps): both converge;
the 8 least-stable finite eigenvalues within 1e-12 (complex128) and 1e-11
(double-word) relative of numpy's.
"""
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest
import scipy.linalg as sl

from oracle import stab_oracle as so
from tests import helpers as H

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA_INC = os.environ.get("CUDA_HOME", "/usr/local/cuda") + "/include"


@pytest.fixture(scope="module")
def harness():
    if not shutil.which("g++") or not os.path.exists(os.path.join(CUDA_INC, "cuda_runtime.h")):
        pytest.skip("needs g++ and the CUDA headers")
    d = tempfile.mkdtemp(prefix="dwqr")
    exe = os.path.join(d, "dw_qr_host")
    subprocess.run(["g++", "-std=c++20", "-O2", "-ffp-contract=off", "-pthread", "-I" + CUDA_INC,
                    os.path.join(ROOT, "tests", "host", "dw_qr_host.cpp"), "-o", exe], check=True)
    yield exe, d
    shutil.rmtree(d, ignore_errors=True)


def _operator(itype: int, seed: int, N: int, M=None) -> np.ndarray:
    """Standard-form operator: B0^-1 A0 (temporal) or the companion matrix."""
    rng = np.random.default_rng(seed)
    if itype == 1:
        M = float(rng.uniform(0.0, 2.0)) if M is None else M
        Re = float(10 ** rng.uniform(np.log10(300.0), np.log10(3000.0)))
        a, b = float(rng.uniform(0.05, 0.4)), float(rng.uniform(0.0, 0.3))
        d, prof = H.synth_case(1, N, max(M, 1e-3), Re, a=a, b=b)
    else:
        M, Re = (float(rng.uniform(0.3, 1.5)) if M is None else M), float(rng.uniform(500, 2500))
        d, prof = H.synth_case(2, N, M, Re, w=0.05, b=float(rng.uniform(0, 0.2)), crossflow=True)
    p = H.oracle_params(d)
    ms = so.mean_state(p, prof[:, 0], prof[:, 1:])
    if itype == 1:
        A0, B0 = so.temporal_pencil(p, ms)
        return np.linalg.solve(B0, A0)
    return so.spatial_companion(p, ms)       # spatial.f90:972-1016


def _hessenberg(itype: int, seed: int, N: int) -> np.ndarray:
    X = _operator(itype, seed, N)
    Xb, _ = sl.matrix_balance(X, permute=True, separate=True)
    n = Xb.shape[0]
    lo, hi = 0, n - 1   # active block between the isolated rows / columns
    while lo < n and np.all(Xb[lo + 1:, lo] == 0):
        lo += 1
    while hi > lo and np.all(Xb[hi, :hi] == 0):
        hi -= 1
    Bk = Xb[lo:hi + 1, lo:hi + 1]
    Bk = Bk * 2.0 ** (-int(np.frexp(np.max(np.abs(Bk)))[1]))
    return sl.hessenberg(Bk)


# the spatial companion case at N = 20 is where complex64 shift formulas took
# 6x the reflector applications (and failed outright at N = 32)
@pytest.mark.parametrize("itype,seed,N", [(1, 0, 8), (1, 2, 12), (1, 5, 12), (2, 1, 20)])
def test_double_word_qr_matches_numpy(harness, itype, seed, N):
    exe, d = harness
    Hm = _hessenberg(itype, seed, N)
    mp = Hm.shape[0]
    fin, fout = os.path.join(d, f"h{seed}.bin"), os.path.join(d, f"o{seed}.bin")
    with open(fin, "wb") as f:
        f.write(np.int32(mp).tobytes())
        f.write(np.asfortranarray(Hm).astype(np.complex128).tobytes(order="F"))
    subprocess.run([exe, "qr", fin, fout], check=True, timeout=600)
    raw = open(fout, "rb").read()
    st64, stdw = np.frombuffer(raw[:8], np.int32)
    up64, updw = np.frombuffer(raw[8:24], np.int64)
    ev = np.frombuffer(raw[24:], np.complex128)
    e64, edw = ev[:mp], ev[mp:]
    assert st64 == 0 and stdw == 0
    assert updw <= 1.5 * up64
    ref = np.linalg.eigvals(Hm)
    top = ref[np.argsort(-ref.imag)[:8]]
    for r in top:
        assert np.min(np.abs(e64 - r)) / abs(r) < 1e-12
        assert np.min(np.abs(edw - r)) / abs(r) < 1e-11
    assert max(np.min(np.abs(edw - r)) for r in ref) < 1e-9


def _run(exe, d, tag, X, threads=32, mode="body"):
    """Whole kernel body on X with a block of `threads` (32: one warp; 128:
    the four warps of the batch kernel); mode "bodyq" runs the QR phase on
    the packed copy in the shared-memory scratch (k_eig_plain_sq)."""
    m = X.shape[0]
    fin, fout = os.path.join(d, f"b{tag}.bin"), os.path.join(d, f"bo{tag}{mode}.bin")
    with open(fin, "wb") as f:
        f.write(np.int32(m).tobytes())
        f.write(np.asfortranarray(X).astype(np.complex128).tobytes(order="F"))
    env = dict(os.environ, HOST_BLOCK_THREADS=str(threads))
    subprocess.run([exe, mode, fin, fout], check=True, timeout=600, env=env)
    raw = open(fout, "rb").read()
    st64, stdw = np.frombuffer(raw[:8], np.int32)
    ev = np.frombuffer(raw[24:], np.complex128)
    return st64, stdw, ev[:m], ev[m:]


# low Mach numbers give the operator entries over ~30 decades (the
# 1/(gamma M^2) pressure terms): the float exponent range and the squares of
# tiny entries are what the double-word form has to survive
@pytest.mark.parametrize("itype,seed,N,M,threads", [(1, 4, 12, 0.01, 32), (2, 0, 12, 0.5, 32), (2, 0, 12, 0.001, 32),
                                                    (1, 4, 12, 0.01, 128), (2, 0, 12, 0.001, 128)])
def test_double_word_eigensolver_body_matches_numpy(harness, itype, seed, N, M, threads):
    exe, d = harness
    X = _operator(itype, seed, N, M)
    st64, stdw, e64, edw = _run(exe, d, f"{itype}_{seed}_{N}_{M}_{threads}", X, threads)
    assert st64 == 0 and stdw == 0
    ref = np.linalg.eigvals(X)
    fin = ref[np.isfinite(ref) & (np.abs(ref) < 1e10)]
    for r in fin[np.argsort(-fin.imag)[:8]]:
        assert np.min(np.abs(e64 - r)) <= 1e-12 * abs(r)
        assert np.min(np.abs(edw - r)) <= 1e-11 * abs(r)


def test_double_word_eigensolver_low_mach_spatial_seed(harness):
    """A spatial request of the serving mix at the seed size N = 32 (M = 0.045,
    Re = 426): bulge entries of its QR fall below the float normal range,
    where an unclamped power-of-two scale factor overflowed to infinity and
    turned the matrix into NaN."""
    from stab_gb300 import serve as sv
    from stab_gb300.surrogate import erf_profile
    exe, d = harness
    r = [q for q in sv.make_requests(2000.0, 1.0, 20261205) if q.itype == 2][178]
    p = so.StabParams(mattyp=1, T0=sv.T0_SUTHERLAND, Ma=r.M, Re=r.Re, Pr=0.72, ny=32, yi=1.0 / 23.0, ymax=50.0,
                      ievec=1, ider=1, top=0, wall=0, wallt=0, curve=0, itype=2, alpha=0j, beta=complex(r.beta),
                      omega=complex(r.omega))
    prof = erf_profile(r.M)
    X = so.spatial_companion(p, so.mean_state(p, prof[:, 0], prof[:, 1:]))
    st64, stdw, e64, edw = _run(exe, d, "serve178", X)
    assert st64 == 0 and stdw == 0
    ref = np.linalg.eigvals(X)
    fin = ref[np.isfinite(ref) & (np.abs(ref) < 1e10)]
    for q in fin[np.argsort(-fin.imag)[:8]]:
        assert np.min(np.abs(edw - q)) <= 1e-11 * abs(q)


def test_kernel_body_memory_safe_under_asan():
    """The same host build with AddressSanitizer (compute-sanitizer is not
    available): every index of the kernel body stays inside its buffers on a
    temporal and a spatial operator, in both working precisions."""
    if not shutil.which("g++") or not os.path.exists(os.path.join(CUDA_INC, "cuda_runtime.h")):
        pytest.skip("needs g++ and the CUDA headers")
    d = tempfile.mkdtemp(prefix="dwasan")
    try:
        exe = os.path.join(d, "dw_qr_asan")
        r = subprocess.run(["g++", "-std=c++20", "-O1", "-g", "-fsanitize=address", "-fno-omit-frame-pointer",
                            "-ffp-contract=off", "-pthread", "-I" + CUDA_INC,
                            os.path.join(ROOT, "tests", "host", "dw_qr_host.cpp"), "-o", exe],
                           capture_output=True, text=True)
        if r.returncode != 0 and "asan" in (r.stderr + r.stdout).lower():
            pytest.skip("AddressSanitizer runtime not available")
        assert r.returncode == 0, r.stderr
        for itype, N, M, threads in ((1, 8, 0.5, 32), (2, 8, 0.01, 128)):
            X = _operator(itype, 3, N, M)
            st64, stdw, _, _ = _run(exe, d, f"asan{itype}", X, threads)
            assert st64 == 0 and stdw == 0
    finally:
        shutil.rmtree(d, ignore_errors=True)


@pytest.mark.parametrize("itype,N,M,threads", [(1, 12, 0.5, 32), (2, 10, 0.01, 128)])
def test_shared_memory_qr_variant_is_bit_identical(harness, itype, N, M, threads):
    """The variant with the QR phase on a packed copy in shared memory (the
    seed kernel k_eig_plain_sq) computes the same operations on the same
    values as the in-place repack: eigenvalues equal bit for bit, in FP64 and
    double-word form."""
    exe, d = harness
    X = _operator(itype, 0, N, M)
    a = _run(exe, d, f"q{itype}_{N}_{threads}", X, threads, "body")
    b = _run(exe, d, f"q{itype}_{N}_{threads}", X, threads, "bodyq")
    assert a[0] == b[0] == 0 and a[1] == b[1] == 0
    assert np.array_equal(a[2], b[2]) and np.array_equal(a[3], b[3])
