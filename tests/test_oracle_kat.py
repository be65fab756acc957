"""Synthetic restatement of the reference's geocodeSlc known-answer test.

tests/cxx/isce3/geocode/geocodeSlc.cpp:231-405 and
tests/python/packages/isce3/geocode/geocode_slc.py:669-745 geocode SLCs whose
samples are exp(i*lon) / exp(i*lat) of each radar pixel's ground point and
require the output phase to equal the geogrid coordinate within 1e-6 rad; the
flattened output must equal the unflattened one times exp(i*flatten_phase);
shifted radar grids with cancelling correction LUTs must change nothing.
Their envisat fixture is absent, so the geometry here is synthetic (a forward
model independent of the geocoder: analytic orbit + rdr2geo).
"""
import numpy as np
import pytest

from isce3_gb300 import synth
from isce3_gb300.core import DataInterpMethod, LUT2d


@pytest.fixture(scope="module")
def scene():
    return synth.scene_c1(slc=False)


def _truth(g, axis):
    if axis == "x":
        return np.radians(g.start_x + g.spacing_x * (np.arange(g.width) + 0.5))[None, :] * np.ones((g.length, 1))
    return np.radians(g.start_y + g.spacing_y * (np.arange(g.length) + 0.5))[:, None] * np.ones((1, g.width))


@pytest.mark.parametrize("axis,height", [("x", 0.0), ("y", 0.0), ("x", 500.0)])
def test_lonlat_phase_kat(oracle_mod, scene, axis, height):
    g = scene.geogrid
    slc = synth.kat_slc(scene, axis, height)
    dem = synth.constant_dem_like(scene.dem, height)
    geo = np.zeros((g.length, g.width), np.complex64)
    oracle_mod.geocode_slc(geo, slc, dem, scene.radar_grid, g, scene.orbit, LUT2d(), LUT2d(), scene.ellipsoid,
                           1e-9, 25, flatten=False)
    v = np.isfinite(geo)
    assert v.sum() > 0.4 * v.size
    err = np.angle(geo[v] * np.exp(-1j * _truth(g, axis)[v]))
    assert np.abs(err).max() < 1e-6


def test_flatten_consistency(oracle_mod, scene):
    g = scene.geogrid
    slc = synth.kat_slc(scene, "x", 0.0)
    dem = synth.constant_dem_like(scene.dem, 0.0)
    flat = np.zeros((g.length, g.width), np.complex64)
    unflat = np.zeros_like(flat)
    fphase = np.full((g.length, g.width), np.nan)
    args = (dem, scene.radar_grid, g, scene.orbit, LUT2d(), LUT2d(), scene.ellipsoid, 1e-9, 25)
    oracle_mod.geocode_slc(flat, slc, *args, flatten=True, flatten_phase_block=fphase)
    oracle_mod.geocode_slc(unflat, slc, *args, flatten=False)
    v = np.isfinite(unflat)
    np.testing.assert_array_equal(v, np.isfinite(flat))
    d = np.angle(flat[v] * np.conj(unflat[v] * np.exp(1j * fphase[v])))
    assert np.abs(d).max() < 1e-6


@pytest.mark.parametrize("mode", ["rg", "az"])
def test_correction_cancels_shift(oracle_mod, scene, mode):
    """Shift the radar grid start by 10 pixels and add a correction LUT of the
    same amount (geocode_slc.py test cases 'rg', 'az')."""
    g = scene.geogrid
    slc = synth.kat_slc(scene, "x", 0.0)
    dem = synth.constant_dem_like(scene.dem, 0.0)
    rg = scene.radar_grid.copy()
    ones = np.ones(rg.shape)
    corr_rg, corr_az = LUT2d(), LUT2d()
    if mode == "rg":
        rg.starting_range += 10 * rg.range_pixel_spacing
    else:
        rg.sensing_start += 10 / rg.prf
    s_vec = np.linspace(rg.starting_range, rg.end_range, rg.width)
    t_vec = np.linspace(rg.sensing_start, rg.sensing_stop, rg.length)
    if mode == "rg":
        corr_rg = LUT2d(s_vec, t_vec, 10 * rg.range_pixel_spacing * ones, DataInterpMethod.NEAREST)
    else:
        corr_az = LUT2d(s_vec, t_vec, 10 / rg.prf * ones, DataInterpMethod.NEAREST)
    geo = np.zeros((g.length, g.width), np.complex64)
    oracle_mod.geocode_slc(geo, slc, dem, rg, g, scene.orbit, LUT2d(), LUT2d(), scene.ellipsoid, 1e-9, 25,
                           flatten=False, az_time_correction=corr_az, srange_correction=corr_rg)
    v = np.isfinite(geo)
    assert v.sum() > 0.3 * v.size
    err = np.angle(geo[v] * np.exp(-1j * _truth(g, "x")[v]))
    assert np.abs(err).max() < 1e-6


def test_newton_iteration_counts(oracle_mod, scene):
    """The oracle's per-pixel geo2rdr iteration count: set for every pixel
    it solved, within the iteration limit, and unchanged by the data."""
    g = scene.geogrid
    slc = synth.kat_slc(scene, "x", 0.0)
    geo = np.zeros((g.length, g.width), np.complex64)
    az = np.zeros((g.length, g.width))
    it = np.zeros((g.length, g.width), np.uint8)
    oracle_mod.geocode_slc(geo, slc, scene.dem, scene.radar_grid, g, scene.orbit, LUT2d(), LUT2d(),
                           scene.ellipsoid, 1e-8, 25, az_index_block=az, niter_block=it)
    solved = np.isfinite(az)
    assert solved.sum() > 0.4 * solved.size
    assert (it[solved] >= 1).all() and (it <= 25).all()
    # linear convergence from mid-swath: a few iterations at least
    assert 2 <= it[solved].mean() <= 25
