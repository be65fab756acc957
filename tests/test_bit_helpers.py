"""The integer forms the kernels use in place of FP64 conversions
(isce3_gb300/csrc/gslc_math.cuh: split_bits, fixed64_to_float), compiled for
the host from the same header and checked against the FP64 operations they
replace: trunc(x), x - trunc(x) (exact) and its rounding to float."""
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
