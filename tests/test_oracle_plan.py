"""CPU checks of the oracle's block-planning restatement.

- get_radar_bbox (geometry/boundingbox.cpp:434-641) against the properties
  of the reference's own test (tests/python/extensions/pybind/geometry/bbox.py:
  first < last, indices inside the radar grid), restated on synthetic
  geometry since its envisat.h5 / srtm_cropped.tif fixtures are absent;
- the same box composed from eight oracle geo2rdr solves (floor/ceil, the
  grid-size starting values, the clamped margin);
- the failure statuses (no convergence, no overlap) and argument errors;
- DEM statistics (DEMInterpolator.cpp:515-560) against NumPy.
"""
import math

import numpy as np
import pytest

import plan_cases


def _corners_box(oracle_mod, sc, g, hmin, hmax, margin):
    rg = sc.radar_grid
    first_az, last_az = rg.length - 1, 0
    first_rg, last_rg = rg.width - 1, 0
    for line in (0, 1):
        y = g.start_y + g.spacing_y * line * g.length
        for pixel in (0, 1):
            x = g.start_x + g.spacing_x * pixel * g.width
            lon, lat = oracle_mod.proj_inverse(g.epsg, x, y)[:2]
            for h in (hmin, hmax):
                t, r, ok = oracle_mod.geo2rdr([lon, lat, float(np.float32(h))], sc.ellipsoid, sc.orbit, sc.image_grid_doppler,
                                              rg.wavelength, rg.lookside, rg.sensing_mid)
                assert ok
                az = (t - rg.sensing_start) * rg.prf
                rr = (r - rg.starting_range) / rg.range_pixel_spacing
                first_az, last_az = min(first_az, math.floor(az)), max(last_az, math.ceil(az))
                first_rg, last_rg = min(first_rg, math.floor(rr)), max(last_rg, math.ceil(rr))
    return (max(first_az - margin, 0), min(last_az + margin, rg.length - 1),
            max(first_rg - margin, 0), min(last_rg + margin, rg.width - 1))


def test_bbox_reference_properties(oracle_mod):
    sc = plan_cases.lonlat_scene()
    rg = sc.radar_grid
    fa, la, fr, lr, st, _ = oracle_mod.radar_bbox(sc.geogrid, rg, sc.orbit, 0.0, 1500.0)
    assert st == 0
    assert fa < la and fr < lr
    for v, n in ((fa, rg.length), (la, rg.length), (fr, rg.width), (lr, rg.width)):
        assert 0 <= v < n


@pytest.mark.parametrize("margin", [0, 7, 50])
def test_bbox_equals_corner_solves(oracle_mod, margin):
    sc = plan_cases.lonlat_scene()
    g = sc.geogrid
    sub = plan_cases.shifted(g, 0.0, 0.0)
    sub.width, sub.length = g.width // 3, g.length // 3
    sub.start_x += g.spacing_x * g.width / 3
    sub.start_y += g.spacing_y * g.length / 3
    got = oracle_mod.radar_bbox(sub, sc.radar_grid, sc.orbit, 100.0, 1400.0, margin=margin)
    assert got[4] == 0
    assert got[:4] == _corners_box(oracle_mod, sc, sub, 100.0, 1400.0, margin)


def test_bbox_failure_statuses(oracle_mod):
    sc = plan_cases.lonlat_scene()
    g = sc.geogrid
    far = oracle_mod.radar_bbox(plan_cases.shifted(g, 0.0, 12.0), sc.radar_grid, sc.orbit, 0.0, 1500.0)
    assert far[4] == 1 and far[5] == 0xF          # beyond the orbit span: geo2rdr fails at all corners
    wrong = oracle_mod.radar_bbox(plan_cases.mirrored_lonlat(sc), sc.radar_grid, sc.orbit, 0.0, 1500.0)
    assert wrong[4] == 1 and wrong[5] == 0xF      # wrong look side
    east = oracle_mod.radar_bbox(plan_cases.shifted(g, 3.0 * g.spacing_x * g.width, 0.0), sc.radar_grid,
                                 sc.orbit, 0.0, 1500.0)
    assert east[4] == 2 and east[5] & (4 | 8)     # entirely outside the grid in range
    with pytest.raises(ValueError):
        oracle_mod.radar_bbox(g, sc.radar_grid, sc.orbit, 10.0, 0.0)
    with pytest.raises(ValueError):
        oracle_mod.radar_bbox(g, sc.radar_grid, sc.orbit, 0.0, 10.0, margin=-1)


def test_bbox_utm_blocks(oracle_mod):
    sc = plan_cases.utm_scene()
    res = [oracle_mod.radar_bbox(b, sc.radar_grid, sc.orbit, 0.0, 3000.0) for b in plan_cases.utm_blocks(sc)]
    st = [r[4] for r in res]
    assert st[0] == 0 and st[1] == 1
    assert st.count(0) > 2 and st.count(2) > 0


def test_dem_stats_against_numpy(oracle_mod):
    rng = np.random.default_rng(3)
    z = rng.uniform(-20.0, 3000.0, (300, 257)).astype(np.float32)
    z[rng.integers(0, 300, 500), rng.integers(0, 257, 500)] = np.nan
    mn, mx, mean, n = oracle_mod.dem_stats(z)
    assert mn == np.nanmin(z) and mx == np.nanmax(z)
    assert n == int(np.isfinite(z).sum())
    assert abs(mean - np.nanmean(z.astype(np.float64))) < 1e-9
    mn, mx, mean, n = oracle_mod.dem_stats(np.full((4, 4), np.nan, np.float32))
    assert n == 0 and np.isnan(mean) and mn == np.finfo(np.float32).max and mx == -np.finfo(np.float32).max
