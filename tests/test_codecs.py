"""The GSLC sample codecs' oracle (oracle/codecs.py) against known answers
of python/packages/isce3/core/types.py's semantics, and the argument checks
of isce3_gb300.types.truncate_mantissa.  No GPU is used."""
import numpy as np
import pytest

from oracle import codecs


def _h(x):
    with np.errstate(over="ignore"):
        return np.array([x], np.float32).astype(np.float16).view(np.uint16)[0]


def test_float16_rounding_known_answers():
    # round to nearest even, overflow to infinity, subnormals, signed zero
    assert _h(1.0) == 0x3C00
    assert _h(1.0 + 2.0 ** -11) == 0x3C00            # tie -> even
    assert _h(1.0 + 3 * 2.0 ** -11) == 0x3C02        # tie -> even (up)
    assert _h(65504.0) == 0x7BFF
    assert _h(65519.99) == 0x7BFF
    assert _h(65520.0) == 0x7C00                     # rounds to infinity
    assert _h(-0.0) == 0x8000
    assert _h(2.0 ** -24) == 0x0001                  # smallest subnormal
    assert _h(2.0 ** -26) == 0x0000
    assert _h(np.float32(np.nan)) == 0x7E00


def test_to_complex32_and_back():
    z = np.array([1 + 2j, -3.5 - 0.25j, 7e4 + 1e-9j, np.nan + 1j], np.complex64)
    c = codecs.to_complex32(z)
    assert c.dtype == codecs.complex32 and c.itemsize == 4
    np.testing.assert_array_equal(c["r"][:2], np.array([1.0, -3.5], np.float16))
    assert np.isinf(c["r"][2]) and c["i"][2] == np.float16(1e-9)
    back = codecs.read_c4_as_c8(c)
    assert back.dtype == np.complex64
    np.testing.assert_array_equal(back[:2], z[:2])
    assert np.isnan(back[3].real) and back[3].imag == 1.0


def test_truncate_mantissa_known_answers():
    z = np.array([1.0 + 2.0 ** -10 + 2.0 ** -11, -np.pi], np.float32)
    codecs.truncate_mantissa(z, 10)
    assert z[0] == np.float32(1.0 + 2.0 ** -10)
    assert z.view(np.uint32)[1] & 0x1FFF == 0
    c = np.array([np.pi + 1j * np.e], np.complex64)
    codecs.truncate_mantissa(c, 3)
    assert c[0].real == np.float32(3.0) and c[0].imag == np.float32(2.5)
    d = np.array([1.0 / 3.0])
    codecs.truncate_mantissa(d, 52)                  # all bits kept
    assert d[0] == 1.0 / 3.0
    with pytest.raises(ValueError):
        codecs.truncate_mantissa(np.zeros(2, np.int32))
    with pytest.raises(ValueError):
        codecs.truncate_mantissa(np.zeros(2, np.float32), 24)


def test_product_truncate_mantissa_argument_errors():
    """isce3_gb300.types raises the reference's errors before any GPU work."""
    from isce3_gb300 import types
    with pytest.raises(ValueError):
        types.truncate_mantissa([1.0, 2.0])
    with pytest.raises(ValueError):
        types.truncate_mantissa(np.zeros(4, np.int16))
    with pytest.raises(ValueError):
        types.truncate_mantissa(np.zeros(4, np.float32), 0)
    with pytest.raises(ValueError):
        types.truncate_mantissa(np.zeros(4, np.float16), 11)
    z = np.ones(3, np.float32)
    types.truncate_mantissa(z, 23)                   # no-op, no GPU needed
    assert np.all(z == 1.0)
    assert types.complex32 == codecs.complex32
