"""Argument checks of isce3_gb300.cuda.geocode.Geocode, in the order and with
the errors of the reference (Geocode.cu:290-376, cuGeocode.cpp:20-90); they
run before any device work, so no GPU is needed."""
import numpy as np
import pytest

pytest.importorskip("torch")

from isce3_gb300 import synth  # noqa: E402
from isce3_gb300.container import RadarGeometry  # noqa: E402
from isce3_gb300.core import DataInterpMethod  # noqa: E402
from isce3_gb300.cuda.geocode import Geocode  # noqa: E402
from isce3_gb300.io import Raster, gdal  # noqa: E402


@pytest.fixture(scope="module")
def small():
    sc = synth.scene_c1(seed=1, slc=False, length=64, width=64, geo=16)
    return sc, Geocode(sc.geogrid, RadarGeometry(sc.radar_grid, sc.orbit), 8)


def test_blocks_and_constructor(small):
    sc, geo = small
    assert geo.n_blocks == 2
    with pytest.raises(ValueError):
        Geocode(sc.geogrid, RadarGeometry(sc.radar_grid, sc.orbit), 0)
    with pytest.raises(TypeError):
        Geocode(sc.geogrid, sc.radar_grid)


def test_consistency_errors(small):
    sc, geo = small
    inp = [np.zeros((64, 64), np.complex64)]
    out = [np.zeros((16, 16), np.complex64)]
    S, C32 = DataInterpMethod.SINC, gdal.GDT_CFloat32
    with pytest.raises(ValueError, match="input and output rasters not equal"):
        geo.geocode_rasters(out, inp + inp, [S], [C32], [np.nan], sc.dem)
    with pytest.raises(ValueError, match="interp methods"):
        geo.geocode_rasters(out, inp, [S, S], [C32], [np.nan], sc.dem)
    with pytest.raises(ValueError, match="data types"):
        geo.geocode_rasters(out, inp, [S], [C32, C32], [np.nan], sc.dem)
    with pytest.raises(ValueError, match="invalid values"):
        geo.geocode_rasters(out, inp, [S], [C32], [], sc.dem)
    with pytest.raises(ValueError, match="not same datatype"):
        geo.geocode_rasters(out, [np.zeros((64, 64), np.float32)], [S], [C32], [np.nan], sc.dem)
    with pytest.raises(ValueError, match="expected datatype"):
        geo.geocode_rasters(out, inp, [S], [gdal.GDT_Float32], [np.nan], sc.dem)
    with pytest.raises(ValueError, match="nearest"):
        geo.geocode_rasters([np.zeros((16, 16), np.uint8)], [np.zeros((64, 64), np.uint8)], [S],
                            [gdal.GDT_Byte], [0.0], sc.dem)
    with pytest.raises(ValueError, match="NaN"):
        geo.geocode_rasters([np.zeros((16, 16), np.uint8)], [np.zeros((64, 64), np.uint8)],
                            [DataInterpMethod.NEAREST], [gdal.GDT_Byte], [np.nan], sc.dem)
    with pytest.raises(ValueError, match="exceeds"):
        geo.geocode_rasters(out, inp, [S], [C32], [1e39], sc.dem)


def test_unsupported_cases(small):
    sc, geo = small
    inp = [Raster(np.zeros((64, 64), np.complex64))]
    out = [Raster.empty(16, 16, gdal.GDT_CFloat32)]
    assert inp[0].datatype() == gdal.GDT_CFloat32
    # data types outside the CUDA geocoder's switch (Geocode.cu:722-775)
    with pytest.raises(NotImplementedError):
        geo.geocode_rasters([np.zeros((16, 16), np.int16)], [np.zeros((64, 64), np.int16)],
                            [DataInterpMethod.NEAREST], [gdal.GDT_Int16], [0.0], sc.dem)
    with pytest.raises(NotImplementedError):
        geo.geocode_rasters(out, inp, [DataInterpMethod.SINC], [gdal.GDT_CFloat32], [np.nan], sc.dem,
                            dem_interp_method=DataInterpMethod.BILINEAR)
    with pytest.raises(ValueError, match="geogrid"):
        geo.geocode_rasters([np.zeros((15, 16), np.complex64)], [np.zeros((64, 64), np.complex64)],
                            [DataInterpMethod.SINC], [gdal.GDT_CFloat32], [np.nan], sc.dem)
