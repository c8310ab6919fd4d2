"""Characterise the FP32 accumulation rounding of the kind::tf32 tensor-core path.

Runs gdft_umma_probe on random TF32 operands (K = 32: four chained MMAs) and
compares with exact FP64 sums: reports the mean and spread of the error in
units of the FP32 ulp of the exact result.  Round-to-nearest gives a mean
near 0 and |err| <= ~0.5 ulp per rounding; truncation gives a mean of the
opposite sign to the result.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def tf32(x):
    x = np.asarray(x, dtype=np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    u = (u + 0x0FFF + ((u >> 13) & 1)) & 0xFFFFE000
    return u.astype(np.uint32).view(np.float32)


def test_umma_accumulation_rounding(built_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from graddft_gb300 import _lib

    lib = _lib.load()
    rng = np.random.default_rng(0)
    for name, gen in (("uniform(0,1)", lambda s: rng.uniform(0, 1, s)),
                      ("normal", lambda s: rng.standard_normal(s)),
                      ("lognormal", lambda s: rng.lognormal(0, 3, s) * rng.choice([-1, 1], s))):
        a = tf32(gen((128, 32)))
        b = tf32(gen((128, 32)))
        d = np.zeros((128, 128), np.float32)
        _lib.check(lib.gdft_umma_probe(a.ctypes.data_as(ctypes.c_void_p), b.ctypes.data_as(ctypes.c_void_p),
                                       d.ctypes.data_as(ctypes.c_void_p)))
        exact = a.astype(np.float64) @ b.astype(np.float64).T
        ulp = np.spacing(np.abs(exact).astype(np.float32)).astype(np.float64)
        err = (d.astype(np.float64) - exact) / ulp
        signed = err * np.sign(exact)
        rn = np.float32(exact)
        print(f"{name:14s} err/ulp mean {err.mean():+.3f} |max| {np.abs(err).max():.2f} "
              f"toward-zero frac {(signed < -0.01).mean():.3f} away frac {(signed > 0.01).mean():.3f} "
              f"equals RN(exact) {(d == rn).mean():.3f}")
        if name == "uniform(0,1)":
            # same-sign sums of four chained MMAs: a few ulp, all toward zero (truncation)
            assert np.abs(err).max() <= 8.0
