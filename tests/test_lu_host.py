"""Batched LU body (stab_gb300/csrc/lu_body.cuh), built for the CPU.

tests/host/lu_host.cpp runs the factorisation of one matrix by a 256-thread
CTA (std::threads, cuda_host_shim.h) with panel width 16, in complex64,
double-word and complex128: the three LUs of the polish (complex64), of its
inverse-iteration retry (double-word) and of the plain path's eigenvectors
(complex128).  Inputs are the polish's matrices: A0 - s B0 of a temporal
operator (temporal.f90:604-752) and the spatial C0 that ZGETRF factors
(spatial.f90:978).  Tolerance on the backward error ||P A - L U|| / ||A||:
complex64 1e-6, double-word 1e-13, complex128 1e-14.
"""
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

from oracle import stab_oracle as so
from tests import helpers as H

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA_INC = os.environ.get("CUDA_HOME", "/usr/local/cuda") + "/include"
TOL = {"c64": 1e-6, "dw": 1e-13, "c128": 1e-14}


@pytest.fixture(scope="module")
def lu_exe():
    if not shutil.which("g++") or not os.path.exists(os.path.join(CUDA_INC, "cuda_runtime.h")):
        pytest.skip("needs g++ and the CUDA headers")
    d = tempfile.mkdtemp(prefix="luhost")
    exe = os.path.join(d, "lu_host")
    subprocess.run(["g++", "-std=c++20", "-O2", "-ffp-contract=off", "-pthread", "-I" + CUDA_INC,
                    os.path.join(ROOT, "tests", "host", "lu_host.cpp"), "-o", exe], check=True)
    yield exe, d
    shutil.rmtree(d, ignore_errors=True)


def _matrix(kind: str, N: int) -> np.ndarray:
    if kind == "temporal":
        d, prof = H.synth_case(1, N, 0.5, 1000.0, a=0.2)
        p = H.oracle_params(d)
        A0, B0 = so.temporal_pencil(p, so.mean_state(p, prof[:, 0], prof[:, 1:]))
        return A0 - (0.2 - 4e-5j) * B0
    d, prof = H.synth_case(2, N, 0.8, 1500.0, w=0.06, b=0.1)
    p = H.oracle_params(d)
    C0, _, _ = so.spatial_operators(p, so.mean_state(p, prof[:, 0], prof[:, 1:]))
    return C0


@pytest.mark.parametrize("kind,N", [("temporal", 16), ("spatial", 12), ("temporal", 24)])
def test_lu_body_backward_error(lu_exe, kind, N):
    exe, d = lu_exe
    A = _matrix(kind, N)
    n = A.shape[0]
    fin, fout = os.path.join(d, f"in_{kind}_{N}.bin"), os.path.join(d, f"out_{kind}_{N}.bin")
    with open(fin, "wb") as f:
        f.write(np.int32(n).tobytes())
        f.write(np.asfortranarray(A).astype(np.complex128).tobytes(order="F"))
    subprocess.run([exe, fin, fout], check=True, timeout=300)
    raw, o = open(fout, "rb").read(), 0
    for name in ("c64", "dw", "c128"):
        info = int(np.frombuffer(raw[o:o + 4], np.int32)[0])
        o += 4
        ip = np.frombuffer(raw[o:o + 4 * n], np.int32)
        o += 4 * n
        F = np.frombuffer(raw[o:o + 16 * n * n], np.complex128).reshape((n, n), order="F")
        o += 16 * n * n
        assert info == 0, name
        L, U = np.tril(F, -1) + np.eye(n), np.triu(F)
        PA = A.copy()
        for j in range(n):   # row swaps in order, as ZGETRF's ipiv
            if ip[j] != j:
                PA[[j, ip[j]], :] = PA[[ip[j], j], :]
        assert np.linalg.norm(PA - L @ U) / np.linalg.norm(A) <= TOL[name], name
