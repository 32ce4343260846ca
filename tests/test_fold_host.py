"""The second candidate level's fold decision (stab_gb300/csrc/fold.cuh, the
per-instance code of k_fold_copies) built for the CPU and run on crafted
copies (tests/host/fold_host.cpp): the sequential fold order, ties, quick
accepts, and each condition of the agreement of the two seed levels, in
both orders of their N."""
import os
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA_INC = os.environ.get("CUDA_HOME", "/usr/local/cuda") + "/include"


def test_fold_decision_cases():
    if not shutil.which("g++") or not os.path.exists(os.path.join(CUDA_INC, "cuda_runtime.h")):
        pytest.skip("needs g++ and the CUDA headers")
    d = tempfile.mkdtemp(prefix="fold")
    try:
        exe = os.path.join(d, "fold_host")
        subprocess.run(["g++", "-std=c++17", "-O1", "-I" + CUDA_INC, os.path.join(ROOT, "tests", "host", "fold_host.cpp"),
                        "-o", exe], check=True)
        r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
        assert r.returncode == 0, r.stdout
        assert r.stdout.count(" ok") == 14, r.stdout
    finally:
        shutil.rmtree(d, ignore_errors=True)
