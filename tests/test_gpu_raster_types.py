"""The CUDA raster geocoder for every data type and interpolation method it
accepts (cxx/isce3/cuda/geocode/Geocode.cu:203-287, 722-775 with the device
interpolators of cxx/isce3/cuda/core/), on the GPU against the oracle's
restatement of those interpolators at the same radar coordinates.  The
coordinates themselves are checked against the fused SINC complex64 call,
which the other raster tests check against the oracle's geocoder.  Values
must be equal bit for bit (NaN where either is NaN)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from isce3_gb300 import synth  # noqa: E402
from isce3_gb300.container import RadarGeometry  # noqa: E402
from isce3_gb300.core import DataInterpMethod, LUT2d  # noqa: E402
from isce3_gb300.cuda.geocode import Geocode  # noqa: E402
from isce3_gb300.io import gdal  # noqa: E402

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

M = DataInterpMethod
FLOAT_TYPES = [(gdal.GDT_Float32, np.float32), (gdal.GDT_CFloat32, np.complex64), (gdal.GDT_Float64, np.float64),
               (gdal.GDT_CFloat64, np.complex128)]
UINT_TYPES = [(gdal.GDT_Byte, np.uint8), (gdal.GDT_UInt16, np.uint16), (gdal.GDT_UInt32, np.uint32)]


@pytest.fixture(scope="module")
def scene():
    sc = synth.scene_c1(seed=31, length=600, width=500, geo=160, dem_px=128, slc=True)
    sc.geometry = RadarGeometry(sc.radar_grid, sc.orbit, LUT2d())
    return sc


def _raster(sc, np_type, seed):
    rng = np.random.default_rng(seed)
    shape = sc.slc.shape
    if np.issubdtype(np_type, np.unsignedinteger):
        return rng.integers(0, np.iinfo(np_type).max, shape, dtype=np_type)
    if np.issubdtype(np_type, np.complexfloating):
        return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np_type)
    return rng.standard_normal(shape).astype(np_type)


def _geocode(sc, rasters, types, methods, invalids, precision="fp64"):
    g = sc.geogrid
    outs = [np.zeros((g.length, g.width), r.dtype) for r in rasters]
    az, rg = np.zeros((g.length, g.width)), np.zeros((g.length, g.width))
    Geocode(g, sc.geometry, lines_per_block=64).geocode_rasters(
        outs, rasters, methods, types, invalids, sc.dem, az_index_block=az, rg_index_block=rg,
        geo2rdr_precision=precision)
    return outs, az, rg


def _bits_equal(a, b):
    if np.issubdtype(a.dtype, np.complexfloating):
        a, b = a.view(a.real.dtype), b.view(b.real.dtype)
    both_nan = np.isnan(a) & np.isnan(b) if np.issubdtype(a.dtype, np.floating) else np.zeros(a.shape, bool)
    return bool(np.all((a == b) | both_nan))


@pytest.mark.parametrize("gtype,np_type", FLOAT_TYPES)
@pytest.mark.parametrize("method", [M.SINC, M.BILINEAR, M.BICUBIC, M.NEAREST, M.BIQUINTIC])
def test_float_types_match_oracle(oracle_mod, scene, gtype, np_type, method):
    r = _raster(scene, np_type, 7)
    (out,), az, rg = _geocode(scene, [r], [gtype], [method], [np.nan])
    ref = oracle_mod.interpolate_raster(az, rg, r, int(method), np.nan)
    assert _bits_equal(out, ref)
    assert np.isfinite(out).mean() > 0.3


@pytest.mark.parametrize("gtype,np_type", UINT_TYPES)
def test_uint_types_nearest(oracle_mod, scene, gtype, np_type):
    r = _raster(scene, np_type, 8)
    (out,), az, rg = _geocode(scene, [r], [gtype], [M.NEAREST], [3.0])
    ref = oracle_mod.interpolate_raster(az, rg, r, int(M.NEAREST), 3.0)
    assert np.array_equal(out, ref)
    assert (out != 3).mean() > 0.3


def test_mixed_call_equals_single_calls(scene):
    """One call with the fused SINC complex64 raster and per-raster ones
    gives each raster the output of its own call, and the coordinate pass
    of a call without a fused raster equals the fused call's coordinates."""
    rs = [scene.slc, _raster(scene, np.float32, 1), _raster(scene, np.uint16, 2), _raster(scene, np.complex128, 3)]
    ts = [gdal.GDT_CFloat32, gdal.GDT_Float32, gdal.GDT_UInt16, gdal.GDT_CFloat64]
    ms = [M.SINC, M.BILINEAR, M.NEAREST, M.BIQUINTIC]
    inv = [np.nan, -1.0, 9.0, 0.0]
    mixed, az, rg = _geocode(scene, rs, ts, ms, inv)
    for k in range(len(rs)):
        (single,), az1, rg1 = _geocode(scene, [rs[k]], [ts[k]], [ms[k]], [inv[k]])
        assert _bits_equal(mixed[k], single)
        assert _bits_equal(az1, az) and _bits_equal(rg1, rg)


def test_float_float_coordinates(oracle_mod, scene):
    r = _raster(scene, np.float64, 9)
    (out,), az, rg = _geocode(scene, [r], [gdal.GDT_Float64], [M.BICUBIC], [np.nan], precision="ff")
    assert _bits_equal(out, oracle_mod.interpolate_raster(az, rg, r, int(M.BICUBIC), np.nan))
