"""The integer forms the kernels use in place of FP64 conversions
(isce3_gb300/csrc/gslc_math.cuh: split_bits, fixed64_to_float,
dbl_to_float, floor_int, small_int_to_float), compiled for the host from
the same header and checked against the FP64 operations they replace:
trunc(x), x - trunc(x) (exact) and its rounding to float, the FP64 -> FP32
conversion, floor."""
import shutil
import subprocess
from fractions import Fraction
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]

HARNESS = r"""
#include "gslc_math.cuh"
#include <cstdio>
#include <cstring>
using namespace gslc;
int main() {
    unsigned long long b;
    while (scanf("%llx", &b) == 1) {
        double x;
        memcpy(&x, &b, 8);
        uint64_t f;
        const int32_t i = split_bits(x, f);
        const float r = fixed64_to_float(f);
        uint32_t rb;
        memcpy(&rb, &r, 4);
        printf("%d %llx %x\n", i, (unsigned long long)f, rb);
    }
    return 0;
}
"""


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("needs nvcc")
    d = tmp_path_factory.mktemp("bits")
    (d / "h.cu").write_text(HARNESS)
    subprocess.run([nvcc, "-std=c++17", "-O2", "-I", str(ROOT / "isce3_gb300" / "csrc"), str(d / "h.cu"),
                    "-o", str(d / "h")], check=True, capture_output=True)

    def run(xs):
        inp = "\n".join(f"{int(np.float64(x).view(np.uint64)):x}" for x in xs) + "\n"
        out = subprocess.run([str(d / "h")], input=inp, capture_output=True, text=True, check=True).stdout
        rows = [line.split() for line in out.splitlines()]
        return [(int(a), int(b, 16), int(c, 16)) for a, b, c in rows]
    return run


def _samples():
    rng = np.random.default_rng(7)
    xs = [1.0, 1.5, 2.0, 4.0 + 2.0 ** -50, 7.999999999999999, 2.0 ** 31 - 2.0 ** -22, 10000.0 + 2.0 ** -39]
    xs += list(rng.uniform(1.0, 16.0, 3000))
    xs += list(rng.uniform(4.0, 20000.0, 3000))
    xs += list(np.exp(rng.uniform(0.0, np.log(2.0 ** 31), 3000)))
    xs += list(np.floor(rng.uniform(1, 1e6, 500)) + 0.5)          # exact halves
    # fractions whose float rounding is a tie (to even, down and up) or just beside one
    base = np.floor(rng.uniform(2, 4000, 500))
    xs += list(base + (1 + 2 * rng.integers(0, 2 ** 20, 500)) * 2.0 ** -25)
    for k in (1, 3, 5):
        xs += list(base[:100] + 0.5 + k * 2.0 ** -25)
        xs += list(base[:100] + 0.25 + k * 2.0 ** -26)
        xs += list(base[:100] + 0.5 + k * 2.0 ** -25 + 2.0 ** -38)
    return [float(x) for x in xs if 1.0 <= x < 2.0 ** 31]


def test_split_and_float_match_fp64_operations(harness):
    xs = _samples()
    got = harness(xs)
    assert len(got) == len(xs)
    for x, (i, f, rb) in zip(xs, got):
        t = int(x)                                   # (int)x: truncation
        frac = x - t                                 # exact for x >= 1
        assert i == t, x
        assert Fraction(f, 2 ** 64) == Fraction(frac), x
        assert rb == int(np.float32(frac).view(np.uint32)), x   # (float)(x - trunc(x)), ties to even


def test_out_of_range_inputs(harness):
    xs = [0.0, 0.25, 0.999999, -0.0, -1.5, -3e9, 2.0 ** 31, 1e300, float("inf"), float("nan"), -float("nan")]
    got = harness(xs)
    want_int = [0, 0, 0, 2 ** 31 - 1, 2 ** 31 - 1, 2 ** 31 - 1, 2 ** 31 - 1, 2 ** 31 - 1, 2 ** 31 - 1,
                2 ** 31 - 1, 2 ** 31 - 1]
    assert [g[0] for g in got] == want_int
    assert all(g[1] == 0 and g[2] == 0 for g in got)


HARNESS2 = r"""
#include "gslc_math.cuh"
#include <cstdio>
#include <cstring>
using namespace gslc;
int main() {
    unsigned long long b;
    while (scanf("%llx", &b) == 1) {
        double x;
        memcpy(&x, &b, 8);
        const float r = dbl_to_float(x);
        uint32_t rb;
        memcpy(&rb, &r, 4);
        const int fl = (x > -2147483648.0 && x < 2147483648.0) ? floor_int(x) : 0;
        printf("%x %d\n", rb, fl);
    }
    return 0;
}
"""


@pytest.fixture(scope="module")
def harness2(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("needs nvcc")
    d = tmp_path_factory.mktemp("bits2")
    (d / "h.cu").write_text(HARNESS2)
    subprocess.run([nvcc, "-std=c++17", "-O2", "-I", str(ROOT / "isce3_gb300" / "csrc"), str(d / "h.cu"),
                    "-o", str(d / "h")], check=True, capture_output=True)

    def run(xs):
        inp = "\n".join(f"{int(np.float64(x).view(np.uint64)):x}" for x in xs) + "\n"
        out = subprocess.run([str(d / "h")], input=inp, capture_output=True, text=True, check=True).stdout
        rows = [line.split() for line in out.splitlines()]
        return [(int(a, 16), int(b)) for a, b in rows]
    return run


def test_double_to_float_from_bits(harness2):
    """dbl_to_float (the LUT values of the chip Doppler) equals the FP64 ->
    FP32 conversion, ties to even, over normal, tie, overflow, subnormal and
    special inputs."""
    rng = np.random.default_rng(11)
    xs = list(rng.standard_normal(3000) * 10.0 ** rng.uniform(-30, 30, 3000))
    m = rng.integers(1, 2 ** 23, 500)
    tie = (m.astype(np.float64) * 2 + 1) * 2.0 ** -24 + 1.0           # halfway between two floats near 1
    xs += list(tie) + list(-tie) + list(np.nextafter(tie, 2.0)) + list(np.nextafter(tie, 0.0))
    xs += [0.0, -0.0, 1e-40, -1e-45, 1e-50, 3.4028235677973366e38, 3.5e38, -1e39, float("inf"), -float("inf"),
           1.1754943508222875e-38, 1.1754942106924411e-38]
    got = harness2(xs)
    for x, (rb, *_rest) in zip(xs, got):
        with np.errstate(over="ignore"):
            want = int(np.float32(x).view(np.uint32))
        assert rb == want, (x, hex(rb), hex(want))
    nan = harness2([float("nan")])[0][0]
    assert (nan & 0x7f800000) == 0x7f800000 and (nan & 0x7fffff) != 0


def test_floor_from_bits(harness2):
    """floor_int (the corner test's integer positions) equals (int)floor(x):
    from the bits in [0, 2^31), the FP64 floor below zero."""
    rng = np.random.default_rng(12)
    xs = list(np.exp(rng.uniform(np.log(1e-25), np.log(2.0 ** 31), 4000)))
    xs += [0.0, 2.0 ** -70, 0.5, 0.999999, 1.0, 2.0 ** 31 - 2.0 ** -21, 7e6 + 0.123456789]
    xs += [-0.25, -1.0, -1.5, -2.0 ** 30, -1e-300]
    got = harness2(xs)
    for x, (_rb, fl) in zip(xs, got):
        assert fl == int(np.floor(x)), x


def test_small_int_to_float_identity():
    """The device form of small_int_to_float: the bits of 1.5 * 2^23 plus n,
    less 1.5 * 2^23, is n for |n| < 2^22 (checked on the identity; the
    host form is the conversion)."""
    n = np.concatenate([np.arange(-5000, 5000), np.array([-(2 ** 22) + 1, 2 ** 22 - 1, 123456, -987654])])
    bits = (np.uint64(0x4B400000) + n.astype(np.int64).astype(np.uint64)) & np.uint64(0xFFFFFFFF)
    v = bits.astype(np.uint32).view(np.float32) - np.float32(12582912.0)
    np.testing.assert_array_equal(v, n.astype(np.float32))
