"""Double-word QR of the seed spectra, built for the CPU.

tests/host/dw_qr_host.cpp compiles the eigensolver's QR iteration
(stab_gb300/csrc/qr.cuh) with g++, the 32 threads of a warp run as
std::threads.  The input is the balanced, power-of-two scaled Hessenberg form
of a temporal operator X = B0^-1 A0 (temporal.f90:771-803) at small N, which
the test builds with the oracle and scipy; the reference spectrum is numpy's.

Tolerances:
  complex128 QR     each of the 8 least-stable eigenvalues within 1e-12
                    relative of numpy's
  double-word QR    the same 8 within 1e-11 relative (about 48 significant
                    bits against 53; the seeds need 1e-9), and every
                    eigenvalue within 1e-9 absolute (the matrix is scaled to
                    a largest entry near 1)
  both converge, and the double-word QR in no more than 1.5x the 2-element
  reflector applications of the complex128 one
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


def _hessenberg(seed: int, N: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    M = float(rng.uniform(0.0, 2.0))
    Re = float(10 ** rng.uniform(np.log10(300.0), np.log10(3000.0)))
    a, b = float(rng.uniform(0.05, 0.4)), float(rng.uniform(0.0, 0.3))
    d, prof = H.synth_case(1, N, max(M, 1e-3), Re, a=a, b=b)
    p = H.oracle_params(d)
    ms = so.mean_state(p, prof[:, 0], prof[:, 1:])
    A0, B0 = so.temporal_pencil(p, ms)
    Xb, _ = sl.matrix_balance(np.linalg.solve(B0, A0), permute=True, separate=True)
    n = Xb.shape[0]
    lo, hi = 0, n - 1   # active block between the isolated rows / columns
    while lo < n and np.all(Xb[lo + 1:, lo] == 0):
        lo += 1
    while hi > lo and np.all(Xb[hi, :hi] == 0):
        hi -= 1
    Bk = Xb[lo:hi + 1, lo:hi + 1]
    Bk = Bk * 2.0 ** (-int(np.frexp(np.max(np.abs(Bk)))[1]))
    return sl.hessenberg(Bk)


@pytest.mark.parametrize("seed,N", [(0, 8), (2, 12), (5, 12)])
def test_double_word_qr_matches_numpy(harness, seed, N):
    exe, d = harness
    Hm = _hessenberg(seed, N)
    mp = Hm.shape[0]
    fin, fout = os.path.join(d, f"h{seed}.bin"), os.path.join(d, f"o{seed}.bin")
    with open(fin, "wb") as f:
        f.write(np.int32(mp).tobytes())
        f.write(np.asfortranarray(Hm).astype(np.complex128).tobytes(order="F"))
    subprocess.run([exe, fin, fout], check=True, timeout=600)
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
