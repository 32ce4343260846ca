"""The allocation-free eigenvalue entry point against the regular one.

stab_eigvals_noalloc serves callers that cannot allocate device memory when
they call (their GPU memory belongs to another allocator, or a cudaFree's
device-wide synchronisation is not acceptable on their path).  This file is
named to be collected last, so a run that stops at the first failure has run
every other test before it; it also passes alone in a fresh process.

Check: for the temporal operator C = B0^-1 A0 of an N = 32 instance (m = 160),
two calls in a row through the C ABI give the eigenvalues of
stab_full_spectrum: every eigenvalue with |omega| < 2 within 1e-8 (absolute,
or relative above 1), the least-stable one within 1e-10 relative.  The
second call changes the device's free memory by nothing and leaves the input
matrix bit for bit as it was.  The edge sizes m = 1 (isolation leaves no QR
window) and m = 256 (the largest the fixed array holds) give numpy's
eigenvalues within 1e-10 * max(1, |A|).
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _least(eig, d):
    from tests import helpers as H
    j = H.select_least(eig, d)
    return eig[j]


def test_noalloc_eigenvalues_match_full_spectrum_twice():
    import torch
    import stab_gb300 as sg
    from tests import helpers as H

    d, prof = H.synth_case(1, 32, 0.5, 1000.0, a=0.2, b=0.05)
    p = H.stab_params(d)
    ctx = sg.Context(0)
    try:
        ref, _, _, st = ctx.full_spectrum(p, prof, want_vector=False)
        assert st == sg.ST_OK
        A0, B0 = ctx.assemble(p, prof)
    finally:
        ctx.close()
    C = np.linalg.solve(B0, A0)
    m = C.shape[0]
    assert m <= 256
    lib = sg.load()
    dev = torch.device("cuda:0")
    a_dev = torch.from_numpy(np.asfortranarray(C).ravel(order="F").view(np.float64).copy()).to(dev)
    eig_dev = torch.zeros(2 * m, dtype=torch.float64, device=dev)
    st_dev = torch.full((1,), -1, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)
    ref_least = _least(ref, d)
    a_before = a_dev.clone()
    prev = None
    for call in range(2):
        eig_dev.fill_(float("nan"))
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info(dev)
        rc = lib.stab_eigvals_noalloc(ctypes.c_void_p(a_dev.data_ptr()), m, ctypes.c_void_p(eig_dev.data_ptr()),
                                      ctypes.c_void_p(st_dev.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0
        torch.cuda.synchronize()
        if call == 1:   # the first call may load the module (lazy loading); later ones allocate nothing
            assert torch.cuda.mem_get_info(dev) == free0
        assert torch.equal(a_dev, a_before)
        assert int(st_dev.item()) == sg.ST_OK
        got = eig_dev.cpu().numpy().view(np.complex128)
        assert np.all(np.isfinite(got))
        for w in ref[(np.abs(ref) < 2.0)]:
            assert np.min(np.abs(got - w)) <= 1e-8 * max(1.0, abs(w))
        g = _least(got, d)
        assert abs(g - ref_least) / abs(ref_least) < 1e-10
        if prev is not None:
            assert np.array_equal(np.sort_complex(got), np.sort_complex(prev))
        prev = got


def test_noalloc_rejects_sizes_beyond_the_fixed_array():
    import torch
    import stab_gb300 as sg
    lib = sg.load()
    dev = torch.device("cuda:0")
    buf = torch.zeros(8, dtype=torch.float64, device=dev)
    st = torch.zeros(1, dtype=torch.int32, device=dev)
    rc = lib.stab_eigvals_noalloc(ctypes.c_void_p(buf.data_ptr()), 257, ctypes.c_void_p(buf.data_ptr()),
                                  ctypes.c_void_p(st.data_ptr()), None)
    assert rc == -1   # STAB_ERR_ARG


@pytest.mark.parametrize("m", [1, 256])
def test_noalloc_edge_sizes_match_numpy(m):
    import torch
    import stab_gb300 as sg
    lib = sg.load()
    dev = torch.device("cuda:0")
    rng = np.random.Generator(np.random.PCG64(5 + m))
    if m == 1:
        A = np.array([[2.5 - 0.75j]])
    else:
        A = rng.standard_normal((m, m)) + 1j * rng.standard_normal((m, m))
    ref = np.linalg.eigvals(A)
    a_dev = torch.from_numpy(np.asfortranarray(A).ravel(order="F").view(np.float64).copy()).to(dev)
    eig_dev = torch.full((2 * m,), float("nan"), dtype=torch.float64, device=dev)
    st_dev = torch.full((1,), -1, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)
    for _ in range(2):
        rc = lib.stab_eigvals_noalloc(ctypes.c_void_p(a_dev.data_ptr()), m, ctypes.c_void_p(eig_dev.data_ptr()),
                                      ctypes.c_void_p(st_dev.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0
        torch.cuda.synchronize()
        assert int(st_dev.item()) == sg.ST_OK
        got = eig_dev.cpu().numpy().view(np.complex128)
        scale = max(1.0, float(np.max(np.abs(A))))
        for w in ref:
            assert np.min(np.abs(got - w)) <= 1e-10 * scale * max(1.0, abs(w)), w
