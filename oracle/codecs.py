"""NumPy restatement of the GSLC sample codecs (the checker for them).

TEST INFRASTRUCTURE ONLY: tests/ use it to check isce3_gb300.types and the
geocoder's complex32 / truncated-mantissa loads and stores.  It follows
python/packages/isce3/core/types.py:
  complex32            types.py:12      pairs of float16
  to_complex32         types.py:38-42   part-wise float32 -> float16 cast
  read_c4_as_c8        types.py:45-72   float16 -> float32 cast (exact)
  truncate_mantissa    types.py:116-165 AND with a mask of the leading bits
numpy's float32 -> float16 cast rounds to nearest even and overflows to
infinity; a NaN keeps its sign and the top ten mantissa bits (never the
infinity pattern).
"""
from __future__ import annotations

import numpy as np

complex32 = np.dtype([("r", np.float16), ("i", np.float16)])


def to_complex32(z: np.ndarray) -> np.ndarray:
    """types.py:38-42."""
    zf = np.zeros(z.shape, dtype=complex32)
    with np.errstate(over="ignore"):
        zf["r"] = z.real
        zf["i"] = z.imag
    return zf


def read_c4_as_c8(z: np.ndarray) -> np.ndarray:
    """types.py:45-72 on an in-memory complex32 array."""
    c64 = np.dtype([("r", np.float32), ("i", np.float32)])
    return np.ascontiguousarray(z).astype(c64).view(np.complex64)


def truncate_mantissa(z: np.ndarray, significant_bits: int = 10) -> None:
    """types.py:116-165, in place."""
    if not isinstance(z, np.ndarray):
        raise ValueError("argument z is not of type np.ndarray")
    if np.iscomplexobj(z):
        truncate_mantissa(z.real, significant_bits)
        truncate_mantissa(z.imag, significant_bits)
        return
    if not issubclass(z.dtype.type, np.floating):
        raise ValueError("argument z is not complex float or float type")
    mant_bits = np.finfo(z.dtype).nmant
    float_bytes = z.dtype.itemsize
    if significant_bits == mant_bits:
        return
    if not 0 < significant_bits <= mant_bits:
        raise ValueError(f"Require 0 < {significant_bits=} <= {mant_bits}")
    allbits = (1 << (float_bytes * 8)) - 1
    bitmask = (allbits << (mant_bits - significant_bits)) & allbits
    u = z.view(np.dtype(f"u{float_bytes}"))
    u &= np.array(bitmask, dtype=u.dtype)
