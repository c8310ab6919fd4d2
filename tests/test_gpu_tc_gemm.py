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


def _run3(lib, a, b, nsplit):
    m, k = a.shape
    n = b.shape[0]
    d = np.zeros((m, n))
    p = lambda x: x.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    lib.check(lib.load().gdft_tc_gemm3_probe(m, n, k, nsplit, p(a), p(b), p(d)))
    return d


@pytest.mark.parametrize("m,n,k,nsplit", [(128, 128, 32, 1), (200, 130, 70, 1), (256, 256, 8192, 7),
                                          (11, 256, 4096, 3), (384, 128, 96, 5)])
def test_tc_gemm3_integers_exact(lib, m, n, k, nsplit):
    """Small integers: every hi*hi chunk sum is exact and the corrections vanish."""
    rng = np.random.default_rng(7 * m + n + k)
    a = rng.integers(-100, 101, (m, k)).astype(np.float64)
    b = rng.integers(-100, 101, (n, k)).astype(np.float64)
    got = _run3(lib, a, b, nsplit)
    np.testing.assert_array_equal(got, a @ b.T)


@pytest.mark.parametrize("m,n,k,nsplit", [(128, 128, 32, 1), (256, 256, 256, 1), (200, 130, 70, 1),
                                          (256, 256, 8192, 7), (11, 256, 4096, 3), (384, 128, 96, 5)])
def test_tc_gemm3_vs_numpy(lib, m, n, k, nsplit):
    rng = np.random.default_rng(m + n + k)
    a = rng.standard_normal((m, k))
    b = rng.standard_normal((n, k))
    ref = a @ b.T
    got = _run3(lib, a, b, nsplit)
    # Operands to about 2^-33 of each row chunk's largest value, hi*hi chunk
    # sums exact, the fold into the running sum error-free: what is left (the
    # residuals, the truncating correction accumulator, the products left out)
    # stays near 2^-31 of the sum of |terms|.
    bound = 2.0 ** -26 * (np.abs(a) @ np.abs(b).T)
    assert np.all(np.abs(got - ref) <= bound), np.max(np.abs(got - ref) / bound)


def test_tc_gemm3_no_drift_on_same_sign_sums(lib):
    """Long contraction of positive terms, where a truncating accumulator drifts by ~2^-23 relative."""
    rng = np.random.default_rng(3)
    k = 1 << 16
    a = rng.uniform(0.5, 1.5, (128, k)) * np.exp(rng.uniform(-3, 3, (128, 1)))
    b = rng.uniform(0.5, 1.5, (128, k))
    ref = a @ b.T
    got = _run3(lib, a, b, 1)
    rel = np.max(np.abs(got - ref) / np.abs(ref))
    assert rel <= 5e-9, rel
