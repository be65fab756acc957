"""Writes tests/golden/oracle_xbuild.npz: the cross-build study's two scenes
(inputs, see tests/xbuild_scenes.py) and the outputs of the oracle built
for x86-64 with -ffp-contract=off.

Run from the repository root on an x86-64 host:
    python tests/golden/make_xbuild_golden.py
"""
import platform
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

import xbuild_scenes as xs  # noqa: E402
from oracle import oracle  # noqa: E402


def main():
    if platform.machine() != "x86_64":
        raise SystemExit("the fixture records the x86-64 build; run this on an x86-64 host")
    scenes = xs.build_scenes()
    out = xs.pack(scenes)
    for name in xs.NAMES:
        sc = xs.unpack(out, name)
        o = xs.run_oracle(oracle, sc, "")
        for k, v in o.items():
            out[f"{name}/out_{k}"] = v
        print(name, "valid px", int(np.isfinite(o["az"]).sum()), "of", o["az"].size)
    np.savez_compressed(xs.GOLDEN, **out)
    print("wrote", xs.GOLDEN, xs.GOLDEN.stat().st_size, "bytes")


if __name__ == "__main__":
    main()
