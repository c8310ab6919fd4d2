"""The packed TF32x3 tensor-core GEMM (network mixed form) against FP64 numpy."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib(built_lib):
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from graddft_gb300 import _lib

    return _lib


def _run(lib, a, b, nsplit):
    m, k = a.shape
    n = b.shape[0]
    d = np.zeros((m, n))
    p = lambda x: x.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    lib.check(lib.load().gdft_tc_gemm_probe(m, n, k, nsplit, p(a), p(b), p(d)))
    return d


@pytest.mark.parametrize("m,n,k,nsplit", [(128, 128, 32, 1), (256, 256, 256, 1), (200, 130, 70, 1),
                                          (256, 256, 8192, 7), (11, 256, 4096, 3), (384, 128, 96, 5)])
def test_tc_gemm_vs_numpy(lib, m, n, k, nsplit):
    rng = np.random.default_rng(m + n + k)
    a = rng.standard_normal((m, k))
    b = rng.standard_normal((n, k))
    ref = a @ b.T
    got = _run(lib, a, b, nsplit)
    scale = np.sqrt(k)  # typical magnitude of the sums
    err = np.max(np.abs(got - ref)) / scale
    # ~22-bit operands, FP32 Kahan-folded sums: a few 1e-7 of the sum scale.
    assert err <= 2e-6, err
