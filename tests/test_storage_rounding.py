"""Stochastic rounding of the 16-bit population storage
(mf-lbm-cuda_gb300/csrc/common.cuh, PopCodec<float, __half / __nv_bfloat16>
::enc_dither), restated in numpy on the FP32 bit patterns: for every 16-bit
variate the stored value is one of the two 16-bit neighbours of x, and over
all 65536 variates the mean is x itself (unbiased rounding), across the
half-normal and half-subnormal ranges, binade edges, negative values and
exactly representable values (stored exactly, whatever the variate)."""
import numpy as np

R16 = np.arange(65536, dtype=np.uint32)


def half_sr(x, r16):
    """enc_dither for __half: x float32 scalar, r16 uint32 array."""
    b = np.float32(x).view(np.uint32)
    mag = b & np.uint32(0x7FFFFFFF)
    if mag < 0x38800000:
        t = np.uint32(np.float32(np.uint32(mag).view(np.float32)) * np.float32(1099511627776.0))
        bits = ((b >> np.uint32(16)) & np.uint32(0x8000)) | ((t + r16) >> np.uint32(16))
        return bits.astype(np.uint16).view(np.float16)
    b2 = (b + (r16 >> np.uint32(3))) & np.uint32(0xFFFFE000)      # rz: drop the 13 low bits
    with np.errstate(over="ignore"):
        h = b2.view(np.float32).astype(np.float16)                 # exactly representable below 65520
    return np.where(np.isinf(h), np.copysign(np.float16(65504), h), h)   # rz saturates


def bf16_sr(x, r16):
    """enc_dither for __nv_bfloat16, as the FP32 value of the stored BF16."""
    b = np.float32(x).view(np.uint32)
    top = (b + r16) >> np.uint32(16)
    return (top << np.uint32(16)).astype(np.uint32).view(np.float32)


def _neighbours16(x):
    h = np.float16(x)
    if np.float32(h) == np.float32(x):
        return h, h
    lo = h if np.float32(h) < x else np.nextafter(h, np.float16(-np.inf))
    hi = np.nextafter(lo, np.float16(np.inf))
    return lo, hi


def _xs(rng):
    xs = [0.0, -0.0, 1.0, -1.0, 2.0 ** -14, -(2.0 ** -14), 2.0 ** -24, 1.5e-5, -3.1e-6, 6.0e-8, 1e-9,
          np.float32(2.0 ** -14) * np.float32(1 - 2 ** -20), 0.9999999, 1.0000001, -0.5000001, 3.14159, 100.3]
    xs += list(rng.uniform(-1, 1, 40)) + list(rng.uniform(-1, 1, 40) * 1e-4) + list(rng.uniform(-1, 1, 20) * 1e-6)
    return [np.float32(x) for x in xs]


def test_half_rounding_is_unbiased_between_neighbours():
    rng = np.random.default_rng(3)
    for x in _xs(rng):
        out = half_sr(x, R16).astype(np.float64)
        lo, hi = _neighbours16(x)
        assert set(np.unique(out)) <= {float(lo), float(hi)}, x
        if lo == hi:
            assert np.all(out == float(lo)), x
        else:
            assert abs(out.mean() - float(x)) <= 2.0 ** -16 * (float(hi) - float(lo)), x


def test_bf16_rounding_is_unbiased_between_neighbours():
    rng = np.random.default_rng(4)
    for x in _xs(rng):
        out = bf16_sr(x, R16).astype(np.float64)
        b = np.float32(x).view(np.uint32)
        lo = float((b & np.uint32(0xFFFF0000)).view(np.float32))
        hi = float(((b & np.uint32(0xFFFF0000)) + np.uint32(0x10000)).view(np.float32))
        if b & 0xFFFF == 0:
            assert np.all(out == float(x)), x
        else:
            assert set(np.unique(out)) <= {lo, hi}, x
            assert abs(out.mean() - float(x)) <= 2.0 ** -16 * abs(hi - lo), x
