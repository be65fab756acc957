"""Regenerate the golden fixtures in this folder.

interpolator_data.npz
    The reference's interpolator known-answer data
    (tests/data/interpolator/data.txt of isce3, read as text): 200 points of
    z = sin(x^2 + y^2) with columns x, y, bilinear, bicubic, biquintic-ish, truth.
    The reference test (tests/cxx/isce3/core/interpolator/interpolator.cpp)
    checks bilinear to 1e-8, biquintic MSE < 0.058 and sinc MSE < 3e-4.
oracle_c1_small.npz
    Oracle output for a reduced version of the 1024 x 1024 scene (seed 7,
    256 x 256 SLC onto 128 x 128 EPSG:4326): a regression pin for the oracle.

Run from the repository root with the reference checkout available:
    python tests/golden/make_golden.py /path/to/isce3
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))


def interpolator_data(ref_root: Path):
    rows = [list(map(float, line.split())) for line in (ref_root / "tests/data/interpolator/data.txt").read_text().splitlines()
            if line.strip()]
    np.savez_compressed(HERE / "interpolator_data.npz", data=np.array(rows, dtype=np.float64))


def oracle_small():
    from isce3_gb300 import synth
    from oracle import oracle
    sc = synth.scene_c1(seed=7, length=256, width=256, geo=128, dem_px=128)
    g = sc.geogrid
    geo = np.zeros((g.length, g.width), np.complex64)
    mask = np.zeros((g.length, g.width), np.uint8)
    oracle.geocode_slc(geo, sc.slc, sc.dem, sc.radar_grid, g, sc.orbit, sc.native_doppler, sc.image_grid_doppler,
                       sc.ellipsoid, sc.threshold, sc.maxiter, mask_block=mask)
    np.savez_compressed(HERE / "oracle_c1_small.npz", geo=geo, mask=mask)


if __name__ == "__main__":
    ref = Path(sys.argv[1]) if len(sys.argv) > 1 else None
    if ref is not None:
        interpolator_data(ref)
    oracle_small()
