"""Radar-grid metadata cubes on the GPU against the oracle's restatement of
makeRadarGridCubes (geometry/metadataCubes.cpp:276-489), which chains each
height layer's geo2rdr solves point to point as the reference does.

Validity (NaN) masks must be identical in every cube.  Azimuth time within
2e-8 s, twice the geo2rdr threshold: where neighbouring points share an
azimuth time the reference's warm-started solve can stop at its start, so
its own times depend on the visiting order by up to the threshold.  Slant
range within 1e-6 m (|dR/dt| is at most a few m/s at these Doppler
centroids), float32 angles and unit vectors within 2 float ulps of the
value, ground-track velocity within 1e-9 relative."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import cube_cases  # noqa: E402
import plan_cases  # noqa: E402
from isce3_gb300 import _lib as L  # noqa: E402
from isce3_gb300 import geometry  # noqa: E402
from isce3_gb300.core import LUT2d  # noqa: E402
from oracle.oracle import CUBE_NAMES  # noqa: E402

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)


def _gpu(sc, cube, heights, native, grid, names=None, **kw):
    shape = (len(heights), cube.length, cube.width)
    arrs = {n: np.full(shape, 7.0, dt) for n, dt in CUBE_NAMES if names is None or n in names}
    geometry.make_radar_grid_cubes(sc.radar_grid, cube, heights, sc.orbit, native, grid,
                                   **{f"{n}_raster": a for n, a in arrs.items()}, **kw)
    return arrs


def _compare(got, ref):
    for n, r in ref.items():
        g = got[n]
        assert np.array_equal(np.isfinite(g), np.isfinite(r)), n
        v = np.isfinite(r)
        if not v.any():
            continue
        d = np.abs(g[v].astype(np.float64) - r[v].astype(np.float64))
        if n == "azimuth_time":
            assert d.max() <= 2e-8, (n, d.max())
        elif n == "slant_range":
            assert d.max() <= 1e-6, (n, d.max())
        elif n == "ground_track_velocity":
            assert (d / np.abs(r[v])).max() <= 1e-9, n
        else:
            ulp = np.spacing(np.abs(r[v]).astype(np.float32)).astype(np.float64)
            assert np.all(d <= 2 * ulp + 1e-12), (n, (d / ulp).max())


def test_cubes_utm_native_doppler(oracle_mod):
    """UTM cube over and beyond the radar grid: the native-Doppler LUT's
    bounds make the vector cubes fail at its edges, where the reference's
    point-to-point chain decides convergence."""
    sc = plan_cases.utm_scene()
    cube = cube_cases.utm_cube(sc)
    h = cube_cases.HEIGHTS
    got = _gpu(sc, cube, h, sc.native_doppler, sc.image_grid_doppler)
    passes = L.lib().gslc_last_cube_passes(L.context(0))
    ref = oracle_mod.radar_grid_cubes(sc.radar_grid, cube, h, sc.orbit, sc.native_doppler, sc.image_grid_doppler)
    _compare(got, ref)
    v = np.isfinite(ref["incidence_angle"])
    assert 0.02 < v.mean() < 0.98                 # both outcomes occur
    assert 2 <= passes <= 16


def test_cubes_grid_doppler_equals_native(oracle_mod):
    """The image-grid Doppler set to the native one (non-zero Doppler in
    both solves, bounds checked)."""
    sc = plan_cases.utm_scene()
    cube = cube_cases.utm_cube(sc, spacing=300.0, n=48)
    h = cube_cases.HEIGHTS[::3]
    got = _gpu(sc, cube, h, sc.native_doppler, sc.native_doppler, delta_range=1e-8)
    ref = oracle_mod.radar_grid_cubes(sc.radar_grid, cube, h, sc.orbit, sc.native_doppler, sc.native_doppler,
                                      delta_range=1e-8)
    _compare(got, ref)


def test_cubes_lonlat_zero_doppler_subset(oracle_mod):
    """EPSG:4326 cube, zero Doppler, only some outputs (the others are skipped,
    as a null raster is in the reference)."""
    sc = plan_cases.lonlat_scene()
    cube = cube_cases.lonlat_cube(sc)
    h = [0.0, 750.0, 1500.0]
    names = ["slant_range", "azimuth_time", "elevation_angle"]
    got = _gpu(sc, cube, h, LUT2d(), LUT2d(), names=names)
    ref = oracle_mod.radar_grid_cubes(sc.radar_grid, cube, h, sc.orbit, LUT2d(), LUT2d(), outputs=names)
    _compare(got, ref)
    assert np.isfinite(ref["slant_range"]).all()


def test_cubes_few_iterations_chain_resets(oracle_mod):
    """numiter 6: many solves stop unconverged, so the chain resets to
    sensingMid and later points start from there, as in the reference."""
    sc = plan_cases.utm_scene()
    cube = cube_cases.utm_cube(sc, n=60)
    h = cube_cases.HEIGHTS[::2]
    got = _gpu(sc, cube, h, sc.native_doppler, sc.image_grid_doppler, numiter_geo2rdr=6)
    ref = oracle_mod.radar_grid_cubes(sc.radar_grid, cube, h, sc.orbit, sc.native_doppler, sc.image_grid_doppler,
                                      maxiter=6)
    _compare(got, ref)
    ok = np.isfinite(ref["azimuth_time"])
    assert 0.0 < ok.mean() < 1.0


def test_cubes_device_tensors_and_errors():
    sc = plan_cases.lonlat_scene()
    cube = cube_cases.lonlat_cube(sc, n=16)
    sr = torch.empty((2, 16, 16), dtype=torch.float64, device="cuda")
    geometry.make_radar_grid_cubes(sc.radar_grid, cube, [0.0, 10.0], sc.orbit, LUT2d(), LUT2d(), sr)
    assert torch.isfinite(sr).all()
    with pytest.raises(ValueError):
        geometry.make_radar_grid_cubes(sc.radar_grid, cube, [0.0], sc.orbit, LUT2d(), LUT2d(), sr)
    with pytest.raises(ValueError):
        geometry.make_radar_grid_cubes(sc.radar_grid, cube, [0.0, 10.0], sc.orbit, LUT2d(), LUT2d(),
                                       np.zeros((2, 16, 16), np.float32))
