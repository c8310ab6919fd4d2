"""The three-slice split the mixed form's exchange packers use (hf.cu, store_row3_scaled), restated in
numpy: per row of 32 values, hi on the quantum 2^(E-8) of the row maximum (E its binary exponent), lo and
lo2 TF32 roundings of the remainders taken in FP32 with the FP64 remainder x - float(x) carried alongside.
The claims the kernels and the tensor-core GEMM rely on: hi is an integer multiple k q with |k| <= 512 (so
a 32-term hi.hi chunk sum stays on the q_a q_b grid), lo and lo2 are TF32 values, and hi + lo + lo2
reproduces scale * x to 2^-31 of the row maximum."""
import numpy as np
import pytest


def _tf32(x):
    b = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x0FFF + ((b >> 13) & 1)) & ~np.uint64(0x1FFF)
    return b.astype(np.uint32).view(np.float32)


def _split(rows, scale):
    f = rows.astype(np.float32)
    xl = (rows - f.astype(np.float64)).astype(np.float32) * np.float32(scale)
    xf = f * np.float32(scale)
    m = np.abs(xf).max(-1)
    eb = ((m.view(np.uint32) >> 23) & 0xFF).astype(np.int64)
    assert np.all((eb >= 9) & (eb < 255)), "rows of normal magnitude only"
    q = np.ldexp(np.float32(1), eb - 135).astype(np.float32)[:, None]
    inv = np.ldexp(np.float32(1), 135 - eb).astype(np.float32)[:, None]
    hi = (np.rint(xf * inv) * q).astype(np.float32)
    r = (xf - hi).astype(np.float32)
    lo = _tf32(r)
    lo2 = _tf32((r - lo).astype(np.float32) + xl)
    return hi, lo, lo2, q


@pytest.mark.parametrize("scale", [1.0, -0.5])
def test_three_slice_split_bounds(scale):
    rng = np.random.default_rng(7)
    rows = rng.standard_normal((4096, 32)) * np.exp(rng.uniform(-60, 60, (4096, 1)))
    rows[::7, ::3] *= 1e-9  # small entries beside large ones
    rows[::11, 5] = 0.0
    hi, lo, lo2, q = _split(rows, scale)
    k = hi.astype(np.float64) / q
    assert np.all(k == np.rint(k)) and np.abs(k).max() <= 512
    for s in (lo, lo2):
        assert np.all((s.view(np.uint32) & 0x1FFF) == 0)
    target = scale * rows
    err = np.abs(hi.astype(np.float64) + lo + lo2 - target).max(-1) / np.abs(target).max(-1)
    assert err.max() <= 2.0 ** -31, err.max()
