"""Raster mode of geocode_slc on the GPU (gslc_geocode_slc_raster) against
the oracle's restatement of geocodeSlc's raster loop
(geocode/geocodeSlc.cpp:605-828): blocks of geogrid lines with their own DEM
windows, multi-band rasters, carriers and phase rasters, a ragged last block
and blocks without valid pixels.  Same parity contract as the array mode:
validity exact, values within 1e-5 relative (+1e-6 rms), phase within
1e-4 rad, splits and sinc-table flips bounded."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from isce3_gb300 import synth  # noqa: E402
from isce3_gb300.core import LUT2d, Poly2d  # noqa: E402
from isce3_gb300.geocode import geocode_slc_raster  # noqa: E402
from isce3_gb300.io import Raster  # noqa: E402

from oracle.compare import assert_parity, compare  # noqa: E402

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)


def _both(oracle_mod, sc, bands, lines_per_block, **kw):
    g = sc.geogrid
    res = {}
    for side in ("gpu", "ora"):
        out = Raster.empty(g.width, g.length, bands=len(bands))
        cph = Raster.empty(g.width, g.length, datatype=7)
        fph = Raster.empty(g.width, g.length, datatype=7)
        az, rg = np.zeros((g.length, g.width)), np.zeros((g.length, g.width))
        inp = Raster(np.stack(bands) if len(bands) > 1 else bands[0].copy())
        fn = geocode_slc_raster if side == "gpu" else oracle_mod.geocode_slc_raster
        fn(out, inp, sc.dem, sc.radar_grid, g, sc.orbit, sc.native_doppler, sc.image_grid_doppler, sc.ellipsoid,
           sc.threshold, sc.maxiter, lines_per_block, carrier_phase_raster=cph, flatten_phase_raster=fph,
           az_index_block=az, rg_index_block=rg, **kw)
        res[side] = dict(out=out, cph=cph.data, fph=fph.data, az=az, rg=rg, inp=inp)
    return res["gpu"], res["ora"]


def _check(gpu, ora, nb):
    reps = []
    for b in range(nb):
        r = compare(gpu["out"].band(b), ora["out"].band(b), gpu["az"], ora["az"], gpu["rg"], ora["rg"])
        print(r)
        assert_parity(r, max_flip_fraction=1e-3)
        reps.append(r)
    with np.errstate(invalid="ignore"):
        split = (np.abs(gpu["az"] - ora["az"]) > 1e-6) | (np.abs(gpu["rg"] - ora["rg"]) > 1e-6)
    for k in ("cph", "fph"):
        ng, no = np.isnan(gpu[k]), np.isnan(ora[k])
        np.testing.assert_array_equal(ng, no)
        w = ~ng & ~split
        assert np.abs(gpu[k][w] - ora[k][w]).max() <= 1e-6, k
    return reps


@pytest.mark.parametrize("lines_per_block", [1000, 100, 37])
def test_utm_raster_mode_two_bands(oracle_mod, lines_per_block):
    sc = synth.scene_c2(length=2048, width=1024, geo=400, spacing=12.0)
    b2 = (sc.slc * np.complex64(0.5 - 0.25j)).astype(np.complex64)
    gpu, ora = _both(oracle_mod, sc, [sc.slc, b2], lines_per_block, azimuth_carrier=sc.az_carrier,
                     range_carrier=Poly2d([[0.1, 2e-3]], x_mean=sc.radar_grid.mid_range))
    reps = _check(gpu, ora, 2)
    assert reps[0]["n_valid"] > 100000
    np.testing.assert_array_equal(gpu["inp"].band(0), sc.slc)     # input raster untouched


def test_lonlat_raster_mode_empty_blocks_lut_carriers(oracle_mod):
    """EPSG:4326 grid reaching north of the swath (its first blocks have no
    valid pixel), data-bearing LUT2d carriers, a custom invalid value."""
    sc = synth.scene_c1(seed=4, length=768, width=768, geo=224, dem_px=128)
    g = sc.geogrid
    g.start_y += 0.35 * g.length * abs(g.spacing_y)
    rg = sc.radar_grid
    rr = np.linspace(rg.starting_range - 20 * rg.range_pixel_spacing, rg.end_range + 20 * rg.range_pixel_spacing, 16)
    tt = np.linspace(rg.sensing_start - 20 / rg.prf, rg.sensing_stop + 20 / rg.prf, 12)
    T, R = np.meshgrid(tt - rg.sensing_mid, rr - rg.mid_range, indexing="ij")
    azc = LUT2d(rr, tt, 2 * np.pi * 150.0 * T + np.pi * 700.0 * T ** 2)
    rgc = LUT2d(rr, tt, 1e-3 * R)
    gpu, ora = _both(oracle_mod, sc, [sc.slc], 32, azimuth_carrier=azc, range_carrier=rgc,
                     invalid_value=complex(-2.0, 3.0))
    _check(gpu, ora, 1)
    v = np.isfinite(gpu["az"])
    assert not v[:32].any() and v.sum() > 10000
    np.testing.assert_array_equal(gpu["out"].band(0)[:32], np.complex64(complex(-2.0, 3.0)))
    assert np.all(gpu["cph"][:32] == -2.0)
