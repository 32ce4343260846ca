"""Double-word primitives (stab_gb300/csrc/dw.cuh), built for the CPU.

tests/host/dw_prims_host.cpp runs 200000 random operand sets (signs and
binary exponents in [-20, 20]) through each primitive and measures the error
against long double.  With u = 2^-24 the bounds checked here are a little
above the published ones (Joldes, Muller, Popescu, ACM TOMS 44, 2017) and
the measured values:

  dw_add          4 u^2 of |x| + |y|   (sloppy sum: no bound relative to the
                                        result under cancellation)
  dw_mul          6 u^2 relative       (DWTimesDW: 5 u^2)
  dw_fma          8 u^2 of |xy| + |c|
  dw_rcp          6 u^2 relative       (one Newton step from a correctly
                                        rounded float reciprocal)
  dw_rsqrt        8 u^2 on r^2 s - 1   (two Newton steps)
  complex fma     8 u^2 of |a||b| + |c|
  complex divide 10 u^2 relative
and every sum normalised: |l| <= ulp(h) / 2.
"""
import os
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA_INC = os.environ.get("CUDA_HOME", "/usr/local/cuda") + "/include"
U2 = 2.0 ** -48

BOUNDS = {"dw_add": 4 * U2, "dw_mul": 6 * U2, "dw_fma": 8 * U2, "dw_rcp": 6 * U2, "dw_rsqrt": 8 * U2,
          "zfma": 8 * U2, "zdiv": 10 * U2}


def test_double_word_primitive_error_bounds():
    if not shutil.which("g++") or not os.path.exists(os.path.join(CUDA_INC, "cuda_runtime.h")):
        pytest.skip("needs g++ and the CUDA headers")
    d = tempfile.mkdtemp(prefix="dwprims")
    try:
        exe = os.path.join(d, "dw_prims_host")
        subprocess.run(["g++", "-std=c++20", "-O2", "-ffp-contract=off", "-pthread", "-I" + CUDA_INC,
                        os.path.join(ROOT, "tests", "host", "dw_prims_host.cpp"), "-o", exe], check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True, timeout=120).stdout
    finally:
        shutil.rmtree(d, ignore_errors=True)
    got = {ln.split()[0]: float(ln.split()[1]) for ln in out.strip().splitlines()}
    for name, bound in BOUNDS.items():
        assert got[name] <= bound, (name, got[name], bound)
    assert got["dw_add_norm"] <= 0.5 + 1e-6
