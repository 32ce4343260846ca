"""Host-side checks of the C ABI library (no GPU needed)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_functions():
    names = []
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            src = open(os.path.join(ROOT, "include", f)).read()
            names += re.findall(r"^\s*(?:int|int32_t|int64_t|const char\*)\s+(stab_\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    import stab_gb300
    if not os.path.exists(stab_gb300.LIB_PATH):
        from stab_gb300 import build
        build.build()
    return stab_gb300.load()


def test_header_declares_entry_points():
    names = _declared_functions()
    assert "stab_full_spectrum" in names and "stab_batch_run" in names


def test_library_exports_every_declared_symbol(lib):
    import stab_gb300
    missing = [n for n in _declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    assert set(stab_gb300.EXPORTED) <= set(_declared_functions())


def test_abi_version(lib):
    assert lib.stab_abi_version() == 1


def test_params_struct_layout():
    import stab_gb300
    # 10 int32 then 7 doubles then 3 complex pairs
    assert ctypes.sizeof(stab_gb300.StabParams) == 10 * 4 + 7 * 8 + 6 * 8
    assert stab_gb300.StabParams.T0.offset == 40


def test_create_without_gpu_reports_error(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    rc = lib.stab_create(ctypes.byref(h), 0)
    assert rc != 0


def test_settings_reject_null_context(lib):
    """The per-stage arithmetic, seed-size and tuning setters check their
    arguments before touching a device: a null context is STAB_ERR_ARG."""
    import stab_gb300 as sg
    assert lib.stab_set_arithmetic(None, sg.STAGE_SEED_EIG, sg.ARITH_FP64) != 0
    assert lib.stab_set_seed_size(None, 32) != 0
    assert lib.stab_set_profiling(None, 1) != 0

