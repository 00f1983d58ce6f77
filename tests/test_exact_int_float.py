"""The FP32 identities the TUNED kernels use in place of conversion
instructions (tuned_core.cuh small_int_to_float / small_float_to_int),
checked on the host with the same IEEE-754 single-precision operations,
exhaustively over the range the kernels use them on.

* (float)k == bits(0x4B400000 + k) - 1.5 * 2^23 for |k| < 2^22: 1.5 * 2^23 + k
  lies in [2^23, 2^24), where floats are exactly the integers and their bit
  patterns are consecutive.
* the inverse, bits(f + 1.5 * 2^23) - 0x4B400000 == (int)f for every
  integer-valued f with |f| < 2^22 (the addition is exact there).
"""
import numpy as np

BIAS_BITS = np.int32(0x4B400000)
BIAS = np.float32(12582912.0)  # 1.5 * 2^23


def test_small_int_to_float_is_exact():
    k = np.arange(-(1 << 22), 1 << 22, dtype=np.int32)
    f = (BIAS_BITS + k).view(np.float32) - BIAS
    assert f.dtype == np.float32
    assert np.array_equal(f, k.astype(np.float32))


def test_small_float_to_int_is_exact():
    k = np.arange(-(1 << 22), 1 << 22, dtype=np.int32)
    f = k.astype(np.float32)
    back = (f + BIAS).view(np.int32) - BIAS_BITS
    assert np.array_equal(back, k)


def test_the_bias_fails_outside_the_range():
    """Just outside |k| < 2^22 the sum leaves [2^23, 2^24) and the identity
    breaks, which is why the kernels only use it on ring-pixel offsets
    (|k| <= 2 nside <= 16384)."""
    k = np.array([-(1 << 22) - 1], dtype=np.int32)
    f = (BIAS_BITS + k).view(np.float32) - BIAS
    assert f[0] != np.float32(k[0])
