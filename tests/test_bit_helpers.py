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


HARNESS3 = r"""
#include "gslc_math.cuh"
#include <cstdio>
#include <cstring>
using namespace gslc;
static double d(unsigned long long b) { double x; memcpy(&x, &b, 8); return x; }
int main() {
    int mode, n;
    unsigned long long a, b, c, e, x;
    while (scanf("%d %d %llx %llx %llx %llx %llx", &mode, &n, &a, &b, &c, &e, &x) == 7) {
        int64_t lo, hi;
        if (mode == 1) {
            lut_axis_keys(d(a), d(b), n, lo, hi);
        } else {
            const double t0 = d(a), prf = d(b), y0 = d(c), dy = d(e);
            key_interval([&](double azc) { return ((t0 + azc / prf) - y0) / dy; }, (prf > 0) == (dy > 0), n - 1.0,
                         lo, hi);
        }
        const int64_t k = dkey(d(x));
        printf("%d\n", (k >= lo && k <= hi) ? 1 : 0);
    }
    return 0;
}
"""


@pytest.fixture(scope="module")
def harness3(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("needs nvcc")
    d = tmp_path_factory.mktemp("bits3")
    (d / "h.cu").write_text(HARNESS3)
    subprocess.run([nvcc, "-std=c++17", "-O2", "-Xcompiler", "-ffp-contract=off", "-I",
                    str(ROOT / "isce3_gb300" / "csrc"), str(d / "h.cu"), "-o", str(d / "h")],
                   check=True, capture_output=True)

    def run(rows):
        hx = lambda v: f"{int(np.float64(v).view(np.uint64)):x}"
        inp = "\n".join(f"{m} {n} {hx(a)} {hx(b)} {hx(c)} {hx(e)} {hx(x)}" for m, n, a, b, c, e, x in rows) + "\n"
        out = subprocess.run([str(d / "h")], input=inp, capture_output=True, text=True, check=True).stdout
        return [int(v) for v in out.split()]
    return run


def _near(v, k):
    """v and the k doubles on each side of it"""
    out = [v]
    lo = hi = np.float64(v)
    for _ in range(k):
        lo, hi = np.nextafter(lo, -np.inf), np.nextafter(hi, np.inf)
        out += [lo, hi]
    return out


def test_lut_contains_key_intervals(harness3):
    """LUT2d::contains as order-key intervals (lut_axis_keys) decides as the
    reference's (x - xStart) / dx in [0, width - 1] (core/LUT2d.h:84-95)
    does, at and beside the table's edges, for both spacing signs and
    degenerate spacings."""
    rng = np.random.default_rng(21)
    rows, want = [], []
    cases = [(848750.0, 1732.0564516128507, 32), (99.86842105263158, 0.35617572156196786, 32), (0.1, 0.3, 7),
             (5.0, -0.7, 9), (-3.0, 1e-3, 1), (1e6, 3.3, 2)]
    cases += [(float(rng.uniform(-1e6, 1e6)), float(rng.choice([-1, 1]) * 10 ** rng.uniform(-4, 4)),
               int(rng.integers(1, 200))) for _ in range(20)]
    for x0, dx, n in cases:
        x0, dx = np.float64(x0), np.float64(dx)
        end = x0 + (n - 1) * dx
        for x in _near(x0, 3) + _near(end, 3) + list(rng.uniform(min(x0, end) - 5 * abs(dx), max(x0, end) + 5 * abs(dx), 20)):
            x = np.float64(x)
            i = (x - x0) / dx
            rows.append((1, n, x0, dx, 0.0, 0.0, x))
            want.append(int(i >= 0.0 and i <= n - 1.0))
    for x0, dx, n, xs in [(1.0, 0.0, 5, [1.0, 2.0, 0.5]), (1.0, np.inf, 3, [-1e300, 0.0, 5.0]),
                          (np.inf, 1.0, 3, [1.0, 1e308]), (1.0, np.nan, 3, [1.0])]:
        for x in xs:
            with np.errstate(all="ignore"):
                i = (np.float64(x) - x0) / dx
            rows.append((1, n, x0, dx, 0.0, 0.0, x))
            want.append(int(i >= 0.0 and i <= n - 1.0))
    assert harness3(rows) == want


def test_chip_doppler_key_intervals(harness3):
    """The chip's contains(t0 + azc / prf, ...) as a key interval of azc
    (geocodeSlc.cpp:462-467) decides as the composed FP64 expression does."""
    rng = np.random.default_rng(22)
    rows, want = [], []
    for _ in range(30):
        t0, prf = np.float64(rng.uniform(0, 1e4)), np.float64(rng.uniform(100, 3000))
        n = int(rng.integers(2, 64))
        dy = np.float64(rng.choice([-1, 1]) * rng.uniform(0.01, 2.0))
        y0 = np.float64(t0 + rng.uniform(-5, 5))
        # azc near the table's two edges
        for edge in (y0, y0 + (n - 1) * dy):
            a0 = (edge - t0) * prf
            for azc in _near(a0, 4) + list(rng.uniform(a0 - 3, a0 + 3, 10)):
                azc = np.float64(azc)
                j = ((t0 + azc / prf) - y0) / dy
                rows.append((2, n, t0, prf, y0, dy, azc))
                want.append(int(j >= 0.0 and j <= n - 1.0))
    assert harness3(rows) == want
