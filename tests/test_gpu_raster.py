"""isce3_gb300.cuda.geocode.Geocode on the GPU against the oracle's restatement
of the reference CUDA raster geocoder (Geocode.cu), on the reference test's
cases (tests/python/extensions/pybind/cuda/geocode/geocode.py:233-450) and on
rough-DEM scenes with Doppler, corrections, subswaths and blocking."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from isce3_gb300 import synth  # noqa: E402
from isce3_gb300.container import RadarGeometry  # noqa: E402
from isce3_gb300.core import DataInterpMethod, LUT2d  # noqa: E402
from isce3_gb300.cuda.geocode import Geocode  # noqa: E402
from isce3_gb300.io import gdal  # noqa: E402
from isce3_gb300.product import SubSwaths  # noqa: E402
from oracle.compare import assert_parity, compare  # noqa: E402

import test_oracle_raster as kat  # noqa: E402

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)


def _gpu(geometry, geogrid, dem, inputs, lines_per_block, invalid, precision="fp64", device_io=True, **kw):
    g = geogrid
    outs = [torch.empty((g.length, g.width), dtype=torch.complex64, device="cuda") if device_io
            else np.zeros((g.length, g.width), np.complex64) for _ in inputs]
    ins = [torch.from_numpy(x).cuda() if device_io else x for x in inputs]
    az = torch.empty((g.length, g.width), dtype=torch.float64, device="cuda")
    rg = torch.empty_like(az)
    geo = Geocode(g, geometry, lines_per_block=lines_per_block)
    geo.geocode_rasters(outs, ins, [DataInterpMethod.SINC] * len(ins), [gdal.GDT_CFloat32] * len(ins),
                        [invalid] * len(ins), dem, geo2rdr_precision=precision, az_index_block=az,
                        rg_index_block=rg, **kw)
    outs = [o.cpu().numpy() if isinstance(o, torch.Tensor) else o for o in outs]
    return outs, az.cpu().numpy(), rg.cpu().numpy()


def _oracle(oracle_mod, geometry, geogrid, dem, inputs, lines_per_block, invalid, **kw):
    g = geogrid
    outs = [np.zeros((g.length, g.width), np.complex64) for _ in inputs]
    az, rg = np.zeros((g.length, g.width)), np.zeros((g.length, g.width))
    oracle_mod.geocode_rasters(outs, inputs, geometry, g, dem, lines_per_block, invalid_values=[invalid] * len(inputs),
                               az_index_block=az, rg_index_block=rg, **kw)
    return outs, az, rg


def _same(gpu, ora):
    (og, ag, rg_), (oo, ao, ro) = gpu, ora
    for a, b in zip(og, oo):
        r = compare(a, b, ag, ao, rg_, ro)
        assert_parity(r)
    return r


@pytest.fixture(scope="module")
def scene():
    return kat.build_scene()


@pytest.mark.parametrize("axis,mode", [("x", ""), ("x", "rg_az"), ("x", "blocked"), ("x", "subswath"),
                                       ("y", "az"), ("y", "subswath")])
def test_raster_kat_gpu(oracle_mod, scene, axis, mode):
    c = kat._case(scene, axis, mode)
    kw = dict(native_doppler=LUT2d(), az_time_correction=c.az_time_correction,
              srange_correction=c.srange_correction, subswaths=c.subswaths)
    gpu = _gpu(c.geometry, scene.geogrid, scene.flat_dem, [scene.kat[axis]], c.lines_per_block, np.nan, **kw)
    ora = _oracle(oracle_mod, c.geometry, scene.geogrid, scene.flat_dem, [scene.kat[axis]], c.lines_per_block,
                  np.nan, **kw)
    _same(gpu, ora)
    phase = np.ma.masked_invalid(np.angle(gpu[0][0]))
    assert np.abs(phase - scene.truth[axis]).max() < 1.0e-6
    if mode == "subswath":
        kept = phase.compressed()
        assert kept.size > 0 and np.all((kept >= c.lo) & (kept <= c.hi))


def _doppler_lut(grid, hz=40.0):
    rr = np.linspace(grid.starting_range - 50 * grid.range_pixel_spacing, grid.end_range, 16)
    tt = np.linspace(grid.sensing_start, grid.sensing_stop, 16)
    u = (rr - rr.mean()) / (rr.max() - rr.mean())
    return LUT2d(rr, tt, np.tile(hz * u, (16, 1)))


@pytest.mark.parametrize("precision", ["fp64", "ff"])
def test_raster_rough_dem_lonlat(oracle_mod, precision):
    """fBm DEM through the CUDA interpolator's spline, two rasters per call,
    blocks of 100 lines, a native-Doppler LUT that does not cover the near
    range (masked there), host I/O."""
    sc = synth.scene_c1(seed=11)
    rng = np.random.default_rng(12)
    second = synth.complex_gaussian(sc.slc.shape, rng)
    geom = RadarGeometry(sc.radar_grid, sc.orbit, LUT2d())
    nat = _doppler_lut(sc.radar_grid)
    nat_cut = LUT2d(np.linspace(sc.radar_grid.starting_range + 100 * 6.25, sc.radar_grid.end_range, 8),
                    np.linspace(sc.radar_grid.sensing_start, sc.radar_grid.sensing_stop, 8), np.zeros((8, 8)))
    for native in (nat, nat_cut):
        kw = dict(native_doppler=native)
        gpu = _gpu(geom, sc.geogrid, sc.dem, [sc.slc, second], 100, 0.0, precision, device_io=False, **kw)
        ora = _oracle(oracle_mod, geom, sc.geogrid, sc.dem, [sc.slc, second], 100, 0.0, **kw)
        r = _same(gpu, ora)
        assert r["n_valid"] > 0.3 * sc.geogrid.length * sc.geogrid.width
    # the cut LUT masks pixels the full one keeps
    assert np.isnan(gpu[1]).sum() > np.isnan(_gpu(geom, sc.geogrid, sc.dem, [sc.slc], 100, 0.0,
                                                   native_doppler=nat)[1]).sum()


def test_raster_utm_doppler_geometry(oracle_mod):
    """UTM geogrid, image-grid Doppler in the RadarGeometry (geo2rdr with the
    reference's delta_range = 10 m derivative step), corrections and
    subswaths, blocks of 64 lines."""
    sc = synth.scene_c2(seed=13, length=2048, width=1536, geo=384, spacing=30.0)
    g = sc.radar_grid
    geom = RadarGeometry(g, sc.orbit, _doppler_lut(g, 25.0))
    r = np.linspace(g.starting_range, g.end_range, 12)
    t = np.linspace(g.sensing_start, g.sensing_stop, 12)
    srange_corr = LUT2d(r, t, np.full((12, 12), 0.7))
    az_corr = LUT2d(r, t, np.full((12, 12), 2e-4))
    ss = SubSwaths(g.length, g.width, 1)
    sw = np.stack([np.full(g.length, 40, np.int32), np.full(g.length, g.width - 90, np.int32)], axis=1)
    ss.set_valid_samples_array(1, sw)
    kw = dict(native_doppler=sc.native_doppler, az_time_correction=az_corr, srange_correction=srange_corr,
              subswaths=ss)
    gpu = _gpu(geom, sc.geogrid, sc.dem, [sc.slc], 64, np.nan, **kw)
    ora = _oracle(oracle_mod, geom, sc.geogrid, sc.dem, [sc.slc], 64, np.nan, **kw)
    rep = _same(gpu, ora)
    assert rep["n_valid"] > 1000
    # the subswath excludes the first 40 and last 90 samples of every line
    rgc = gpu[2][np.isfinite(gpu[2])]
    assert rgc.min() >= 40 and rgc.max() < g.width - 90
