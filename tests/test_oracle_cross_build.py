"""How far two correct builds of one geocoder disagree (CPU).

The reference builds with CMake's C++17 (-std=c++17 -O2, no contraction
flag: .cmake/ConfigISCE.cmake:49-51).  GCC contracts a * b + c into a fused
multiply-add by default for C++ even in ISO mode, and every aarch64 core has
FMA, so the reference's aarch64 build fuses where its x86-64 build (no -mfma)
cannot.  The oracle is built both ways (oracle/Makefile targets all and fma)
and run on the two stored scenes of tests/xbuild_scenes.py; the checker
(oracle/compare.py) classifies the differences the same way it classifies
the GPU's.  The GPU parity tests bound the GPU's split and flip fraction by
this measured disagreement.

The oracle proper must also reproduce the fixture the x86-64 build wrote
(tests/golden/make_xbuild_golden.py): bit for bit on x86-64; elsewhere the
host's libm may round a transcendental differently, and the pixels that
moves are counted with the same classification.
"""
import platform

import numpy as np
import pytest

import xbuild_scenes as xs
from oracle.compare import assert_parity


@pytest.fixture(scope="module")
def golden():
    return dict(np.load(xs.GOLDEN))


def _gold(golden, name):
    return {k: golden[f"{name}/out_{k}"] for k in ("geo", "mask", "az", "rg")}


@pytest.mark.parametrize("name", xs.NAMES)
def test_oracle_reproduces_x86_fixture(oracle_mod, golden, name):
    sc = xs.unpack(golden, name)
    out = xs.run_oracle(oracle_mod, sc, "")
    gold = _gold(golden, name)
    r = xs.report(out, gold)
    print(name, platform.machine(), r)
    if platform.machine() == "x86_64":
        for k in gold:
            np.testing.assert_array_equal(out[k].view(np.uint8), gold[k].view(np.uint8), err_msg=k)
    else:
        assert_parity(r, max_flip_fraction=1e-3)


@pytest.mark.parametrize("name", xs.NAMES)
def test_contracting_build_disagreement(oracle_mod, golden, name):
    """The fused build splits or flips a measurable fraction of pixels; masks,
    validity and every other pixel agree within the parity tolerance."""
    sc = xs.unpack(golden, name)
    plain = xs.run_oracle(oracle_mod, sc, "")
    fused = xs.run_oracle(oracle_mod, sc, "fma")
    r = xs.report(fused, plain)
    print(name, platform.machine(), r)
    assert_parity(r, max_flip_fraction=0.1)
    assert r["flip_fraction"] > 1e-4
