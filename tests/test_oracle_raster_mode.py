"""The oracle's raster mode of geocodeSlc (geocode/geocodeSlc.cpp:605-828).

The raster mode reads, per block of geogrid lines, only the radar bounding
box of the block's valid pixels widened by 5 samples (clamped to the radar
grid, :740-750), and loads a DEM window per block (:653-656).  The GPU reads
the whole radar raster instead, on the argument that the interpolator's chip
tests then reject exactly the same pixels.  With one block (the same DEM
window as array mode) the oracle's raster mode must therefore equal its
array mode over the whole raster bit for bit; with several blocks only the
DEM windows differ.  Blocks without valid pixels are filled with the invalid
value, and the phase rasters with its real part (:752-770).  CPU only.
"""
import numpy as np
import pytest

from isce3_gb300 import synth
from isce3_gb300.core import Poly2d
from isce3_gb300.io import Raster


def _raster_run(oracle_mod, sc, lines_per_block, bands, **kw):
    g = sc.geogrid
    out = Raster.empty(g.width, g.length, bands=len(bands))
    cph = Raster.empty(g.width, g.length, datatype=7)
    fph = Raster.empty(g.width, g.length, datatype=7)
    az, rg = np.zeros((g.length, g.width)), np.zeros((g.length, g.width))
    inp = Raster(np.stack(bands) if len(bands) > 1 else bands[0])
    oracle_mod.geocode_slc_raster(out, inp, sc.dem, sc.radar_grid, g, sc.orbit, sc.native_doppler,
                                  sc.image_grid_doppler, sc.ellipsoid, sc.threshold, sc.maxiter, lines_per_block,
                                  carrier_phase_raster=cph, flatten_phase_raster=fph, az_index_block=az,
                                  rg_index_block=rg, **kw)
    return out, cph, fph, az, rg, inp


def test_single_block_equals_array_mode(oracle_mod):
    sc = synth.scene_c2(length=1024, width=768, geo=320, spacing=12.0, dem_arcsec=3.0)
    kw = dict(azimuth_carrier=sc.az_carrier, range_carrier=Poly2d([[0.2, 1e-3]], x_mean=sc.radar_grid.mid_range))
    b2 = (sc.slc * np.complex64(0.25 + 0.5j)).astype(np.complex64)
    out, cph, fph, az, rg, inp = _raster_run(oracle_mod, sc, sc.geogrid.length, [sc.slc, b2], **kw)
    assert np.array_equal(inp.band(0), sc.slc)                  # the input raster is read only
    g = sc.geogrid
    shape = (g.length, g.width)
    geo = [np.zeros(shape, np.complex64) for _ in range(2)]
    carrier, flat = np.full(shape, -7.0), np.full(shape, -7.0)
    az_a, rg_a = np.zeros(shape), np.zeros(shape)
    oracle_mod.geocode_slc(geo, [sc.slc.copy(), b2.copy()], sc.dem, sc.radar_grid, g, sc.orbit, sc.native_doppler,
                           sc.image_grid_doppler, sc.ellipsoid, sc.threshold, sc.maxiter,
                           az_carrier=kw["azimuth_carrier"], rg_carrier=kw["range_carrier"],
                           carrier_phase_block=carrier, flatten_phase_block=flat, az_index_block=az_a,
                           rg_index_block=rg_a)
    for b in range(2):
        np.testing.assert_array_equal(out.band(b).view(np.uint64), geo[b].view(np.uint64))
    np.testing.assert_array_equal(az, az_a)
    np.testing.assert_array_equal(rg, rg_a)
    w = carrier != -7.0
    assert w.sum() > 50000
    np.testing.assert_array_equal(cph.data[w], carrier[w])
    np.testing.assert_array_equal(fph.data[w], flat[w])
    assert np.all(np.isnan(cph.data[~w])) and np.all(np.isnan(fph.data[~w]))


def test_blocks_and_empty_blocks(oracle_mod):
    """A geogrid reaching beyond the swath: blocks with no valid pixel are
    all invalid (and NaN phase), the others agree with the one-block run
    except where a block's own DEM window moves a height by a rounding."""
    sc = synth.scene_c1(seed=2, length=768, width=768, geo=192, dem_px=128)
    g = sc.geogrid
    g.start_y += 0.4 * g.length * abs(g.spacing_y)       # the top rows fall north of the swath
    full = _raster_run(oracle_mod, sc, g.length, [sc.slc], invalid_value=complex(-2.0, 3.0))
    blk = _raster_run(oracle_mod, sc, 40, [sc.slc], invalid_value=complex(-2.0, 3.0))
    v_full, v_blk = np.isfinite(full[3]), np.isfinite(blk[3])
    np.testing.assert_array_equal(v_full, v_blk)
    rows_valid = v_blk.any(axis=1)
    assert not rows_valid[:40].any() and rows_valid.any()      # the first block is empty
    out = blk[0].band(0)
    np.testing.assert_array_equal(out[~v_blk], np.complex64(complex(-2.0, 3.0)))
    assert np.all(blk[1].data[~v_blk] == -2.0)
    same = v_blk & (np.abs(full[3] - blk[3]) == 0) & (np.abs(full[4] - blk[4]) == 0)
    assert same.sum() > 0.99 * v_blk.sum()
    np.testing.assert_array_equal(full[0].band(0)[same], out[same])
