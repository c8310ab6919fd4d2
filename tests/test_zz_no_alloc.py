"""The allocation-free integrate entry point against the workspace one.

gdft_integrate_noalloc is for callers that cannot allocate device memory at
the point of the call (a JAX/XLA custom-call handler must not allocate
outside XLA's allocator; a service may have reserved all device memory at
start-up).  It keeps its scratch in a fixed array inside the library, so this
test checks it gives the same energy as gdft_integrate, called through the C
ABI, on two calls in a row with different data (the array keeps the previous
call's contents, which must not leak into the next result).  The file sorts
last so that a run that stops at the first failure has run everything else.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def _energy(lib, fn_name, dens, w, coeffs, clip, ws=None):
    from graddft_gb300 import _lib

    out = torch.empty((), dtype=torch.float64, device="cuda")
    c = (ctypes.c_double * len(coeffs))(*coeffs)
    n_grid, n_cols = dens.shape
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    if fn_name == "gdft_integrate":
        rc = lib.gdft_integrate(n_grid, n_cols, c, len(coeffs), ctypes.c_void_p(dens.data_ptr()),
                                ctypes.c_void_p(w.data_ptr()), clip, ctypes.c_void_p(out.data_ptr()),
                                ctypes.c_void_p(ws.data_ptr()), ws.numel(), stream)
    else:
        rc = lib.gdft_integrate_noalloc(n_grid, n_cols, c, len(coeffs), ctypes.c_void_p(dens.data_ptr()),
                                        ctypes.c_void_p(w.data_ptr()), clip, ctypes.c_void_p(out.data_ptr()), stream)
    _lib.check(rc)
    torch.cuda.synchronize()
    return float(out)


def test_integrate_noalloc_matches_workspace_entry(built_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from graddft_gb300 import _lib

    lib = _lib.load()
    rng = np.random.default_rng(2024)
    for call, (n_grid, n_cols, coeffs) in enumerate([(1_000_003, 3, [1.0]), (257_000, 5, [0.8, 0.72, 0.19, 0.81, 0.2])]):
        dens = torch.as_tensor(-np.abs(rng.lognormal(-4, 2, (n_grid, n_cols))), device="cuda")
        w = torch.as_tensor(rng.lognormal(-6, 1, n_grid), device="cuda")
        nbytes = ctypes.c_size_t()
        _lib.check(lib.gdft_integrate_workspace_bytes(n_grid, ctypes.byref(nbytes)))
        ws = torch.empty(nbytes.value, dtype=torch.uint8, device="cuda")
        ref = _energy(lib, "gdft_integrate", dens, w, coeffs, 1e-30, ws)
        got = _energy(lib, "gdft_integrate_noalloc", dens, w, coeffs, 1e-30)
        assert abs(got - ref) <= RTOL * abs(ref), (call, got, ref)


def test_integrate_noalloc_rejects_oversized_grid(built_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from graddft_gb300 import _lib

    lib = _lib.load()
    dummy = torch.zeros(1, dtype=torch.float64, device="cuda")
    c = (ctypes.c_double * 1)(1.0)
    rc = lib.gdft_integrate_noalloc((1 << 25) + 1, 1, c, 1, ctypes.c_void_p(dummy.data_ptr()),
                                    ctypes.c_void_p(dummy.data_ptr()), 1e-30, ctypes.c_void_p(dummy.data_ptr()), None)
    assert rc == _lib.GDFT_ERR_INVALID
    assert b"scratch limit" in lib.gdft_last_error()
