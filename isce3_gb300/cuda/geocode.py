"""``isce3.cuda.geocode.Geocode``: block geocoding of radar rasters onto a geogrid.

The reference class (cxx/isce3/cuda/geocode/Geocode.h:70-128, Geocode.cu,
bound in python/extensions/pybind_isce3/cuda/geocode/cuGeocode.cpp:17-90)
splits the geogrid into blocks of ``lines_per_block`` lines; per block it
loads the DEM window, maps every geogrid pixel to radar coordinates with
geo2rdr (masking pixels whose corrections or native Doppler do not contain
them, that fall outside the radar grid or outside the subswaths), reads the
radar block around them and interpolates each raster.

Here SINC rasters of GDT_CFloat32 (the SLC case) run in one fused GB300
kernel per block, all such rasters of the call at once; the per-pixel rules
are the reference's, and the radar bounding box it reads is not needed
because the rasters are resident.  Every other data type the reference
accepts (Float32, Float64, CFloat64, Byte, UInt16, UInt32) and method (SINC,
BILINEAR, BICUBIC, NEAREST, BIQUINTIC; integer types nearest only) takes the
reference's own two steps: the same kernel writes the radar coordinates of
each geogrid pixel, then one interpolation kernel per raster samples it
(gslc_interpolate_raster).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from .. import _lib as L
from .. import _marshal as M
from ..container import RadarGeometry
from ..core import DataInterpMethod, Ellipsoid, LUT2d
from ..geocode import _Staged
from ..io import Raster, gdal, gdal_type_of
from ..product import GeoGridParameters, SubSwaths

_INT_TYPES = (gdal.GDT_Byte, gdal.GDT_UInt16, gdal.GDT_UInt32)
_TYPE_MAX = {gdal.GDT_Byte: 255, gdal.GDT_UInt16: 65535, gdal.GDT_UInt32: 4294967295}
_FLT_MAX = float(np.finfo(np.float32).max)
# the data types the reference's CUDA geocoder accepts (Geocode.cu:722-775)
_TORCH_TYPES = {gdal.GDT_Float32: torch.float32, gdal.GDT_CFloat32: torch.complex64, gdal.GDT_Float64: torch.float64,
                gdal.GDT_CFloat64: torch.complex128, gdal.GDT_Byte: torch.uint8, gdal.GDT_UInt16: torch.uint16,
                gdal.GDT_UInt32: torch.uint32}


def _samples(r):
    """The sample array of a raster argument (Raster, ndarray or tensor)."""
    return r.data if isinstance(r, Raster) else r


def _dtype_of(r) -> int:
    return r.datatype() if isinstance(r, Raster) else gdal_type_of(r)


class Geocode:
    """Geocode rasters that share a radar geometry onto one geogrid."""

    def __init__(self, geogrid_params: GeoGridParameters, radar_geometry: RadarGeometry,
                 lines_per_block: int = 1000):
        if not isinstance(radar_geometry, RadarGeometry):
            raise TypeError("radar_geometry must be an isce3_gb300.container.RadarGeometry")
        lines_per_block = int(lines_per_block)
        if lines_per_block < 1:
            raise ValueError("lines_per_block must be positive")
        self.geogrid = geogrid_params
        self.radar_geometry = radar_geometry
        self.lines_per_block = lines_per_block
        # Geocode.cu:343: number of blocks
        self.n_blocks = (geogrid_params.length + lines_per_block - 1) // lines_per_block
        self.ellipsoid = Ellipsoid()       # makeProjection(epsg)->ellipsoid(): WGS84 for 4326 and UTM

    @staticmethod
    def _check_consistency(output_rasters, input_rasters, data_interp_methods, raster_datatypes, invalid_values):
        """Geocode.cu:304-376 (ensureRasterConsistency), with its messages."""
        n = len(output_rasters)
        if n != len(input_rasters):
            raise ValueError("number of input and output rasters not equal")
        if n != len(data_interp_methods):
            raise ValueError("number of interp methods and output rasters not equal")
        if n != len(raster_datatypes):
            raise ValueError("number of interpolation methods and data types not equal")
        if n != len(invalid_values):
            raise ValueError("number of interpolation methods and invalid values not equal")
        for out, inp, method, dtype, inv in zip(output_rasters, input_rasters, data_interp_methods,
                                                raster_datatypes, invalid_values):
            in_dtype, out_dtype = _dtype_of(inp), _dtype_of(out)
            if in_dtype != out_dtype:
                raise ValueError("input and output rasters not same datatype")
            if in_dtype != int(dtype):
                raise ValueError("input and output rasters datatype does not match expected datatype")
            # Geocode.cu:290-302 (rasterDtypeInterpCheck)
            if int(dtype) in _INT_TYPES and DataInterpMethod(method) != DataInterpMethod.NEAREST:
                raise ValueError("int type of raster can only use nearest neighbor interp")
            # Geocode.cu:304-340 (invalidValueCheck)
            inv = float(inv)
            if np.isnan(inv) and int(dtype) in _INT_TYPES:
                raise ValueError("int-type datatype can not have NaN invalid value")
            if int(dtype) in _TYPE_MAX and inv > _TYPE_MAX[int(dtype)]:
                raise ValueError("unsigned datatype invalid value exceeds type max")
            if int(dtype) in (gdal.GDT_Float32, gdal.GDT_CFloat32) and abs(inv) > _FLT_MAX:
                raise ValueError("float32-type datatype invalid value exceeds type max")

    def geocode_rasters(self, output_rasters, input_rasters, data_interp_methods, raster_datatypes,
                        invalid_values, dem_raster, native_doppler: LUT2d | None = None,
                        az_time_correction: LUT2d | None = None, srange_correction: LUT2d | None = None,
                        subswaths: SubSwaths | None = None,
                        dem_interp_method: DataInterpMethod = DataInterpMethod.BIQUINTIC,
                        threshold: float = 1e-8, maxiter: int = 50, delta_range: float = 10.0, *,
                        geo2rdr_precision: str = "fp64", az_index_block=None, rg_index_block=None,
                        dem_margin: int = 50, device=None, stream: torch.cuda.Stream | None = None) -> None:
        """Geocode ``input_rasters`` into ``output_rasters`` (written in place).

        Arguments and defaults are those of the reference binding
        (cuGeocode.cpp:39-90).  Rasters are ``isce3_gb300.io.Raster`` objects,
        NumPy arrays or CUDA tensors: inputs of the radar grid's shape,
        outputs of the geogrid's.  Invalid output pixels hold
        complex(invalid, invalid) for complex types.  Extra keyword-only arguments:
        ``geo2rdr_precision`` ("fp64" or "ff"), ``az_index_block`` /
        ``rg_index_block`` (f64 radar coordinates of each geo pixel, NaN where
        masked), ``dem_margin``, ``device`` and ``stream``.
        """
        self._check_consistency(output_rasters, input_rasters, data_interp_methods, raster_datatypes,
                                invalid_values)
        for dtype in raster_datatypes:
            if int(dtype) not in _TORCH_TYPES:
                raise NotImplementedError(f"GDAL data type {int(dtype)} is not geocoded by the CUDA geocoder")
        if DataInterpMethod(dem_interp_method) != DataInterpMethod.BIQUINTIC:
            raise NotImplementedError("only the biquintic DEM interpolator is provided")
        if geo2rdr_precision not in ("fp64", "ff", "float-float"):
            raise ValueError("geo2rdr_precision must be 'fp64' or 'ff'")
        n = len(output_rasters)
        if n == 0:
            return
        rgrid = self.radar_geometry.radar_grid
        g = self.geogrid
        for inp, out in zip(input_rasters, output_rasters):
            if tuple(_samples(inp).shape) != (rgrid.length, rgrid.width):
                raise ValueError("input raster shape does not match the radar grid")
            if tuple(_samples(out).shape) != (g.length, g.width):
                raise ValueError("output raster shape does not match the geogrid")
        native_doppler = native_doppler if native_doppler is not None else LUT2d()
        az_time_correction = az_time_correction if az_time_correction is not None else LUT2d()
        srange_correction = srange_correction if srange_correction is not None else LUT2d()

        dev = M.device_of(device)
        fused = [i for i in range(n) if int(raster_datatypes[i]) == gdal.GDT_CFloat32
                 and DataInterpMethod(data_interp_methods[i]) == DataInterpMethod.SINC]
        others = [i for i in range(n) if i not in fused]
        with torch.cuda.device(dev):
            s = stream or torch.cuda.current_stream(dev)
            with torch.cuda.stream(s):
                ins = [_Staged(_samples(r), dev, True, _TORCH_TYPES[int(t)])
                       for r, t in zip(input_rasters, raster_datatypes)]
                outs = [_Staged(_samples(r), dev, False, _TORCH_TYPES[int(t)])
                        for r, t in zip(output_rasters, raster_datatypes)]
                extra = []
                for arr, what in ((az_index_block, "az_index_block"), (rg_index_block, "rg_index_block")):
                    if arr is None:
                        extra.append(None)
                        continue
                    if tuple(arr.shape) != (g.length, g.width):
                        raise ValueError(f"{what} shape does not match the geogrid")
                    extra.append(_Staged(arr, dev, False, torch.float64))
                # the radar coordinates the per-raster interpolation reads
                coords = [e.dev if e is not None else None for e in extra]
                if others:
                    coords = [c if c is not None else torch.empty((g.length, g.width), dtype=torch.float64,
                                                                  device=dev) for c in coords]
                a = L.RasterGeocodeArgs()
                a.radar_grid = M.radar_grid_desc(rgrid)
                a.geo_grid = M.geo_grid_desc(g)
                a.orbit = M.orbit_desc(self.radar_geometry.orbit)
                a.doppler = M.lut_desc(self.radar_geometry.doppler, dev)
                a.native_doppler = M.lut_desc(native_doppler, dev)
                a.az_time_correction = M.lut_desc(az_time_correction, dev)
                a.srange_correction = M.lut_desc(srange_correction, dev)
                a.dem, dem_keep = M.dem_raster_desc_blocks(dem_raster, g, self.lines_per_block, dem_margin, dev)
                ss = None
                if subswaths is not None:
                    ss = M.subswaths_desc(subswaths, dev)
                    a.subswaths = C.pointer(ss)
                a.ellipsoid_a, a.ellipsoid_e2 = self.ellipsoid.a, self.ellipsoid.e2
                a.threshold, a.delta_range = float(threshold), float(delta_range)
                a.maxiter, a.lines_per_block = int(maxiter), self.lines_per_block
                a.n_rasters = len(fused)
                a.geo2rdr_precision = 0 if geo2rdr_precision == "fp64" else 1
                in_ptrs = (C.c_void_p * max(len(fused), 1))(*[ins[i].ptr() for i in fused])
                out_ptrs = (C.c_void_p * max(len(fused), 1))(*[outs[i].ptr() for i in fused])
                invs = (C.c_double * max(len(fused), 1))(*[float(invalid_values[i]) for i in fused])
                a.input_rasters = C.cast(in_ptrs, C.POINTER(C.c_void_p))
                a.output_rasters = C.cast(out_ptrs, C.POINTER(C.c_void_p))
                a.invalid_values = C.cast(invs, C.POINTER(C.c_double))
                a.az_index = coords[0].data_ptr() if coords[0] is not None else None
                a.rg_index = coords[1].data_ptr() if coords[1] is not None else None
                a.dem_margin = int(dem_margin)
                ctx = L.context(dev.index)
                lib = L.lib()
                if fused or others or coords[0] is not None or coords[1] is not None:
                    st = lib.gslc_geocode_rasters(ctx, C.byref(a), C.c_void_p(s.cuda_stream))
                    L.check(st, ctx, "geocode_rasters")
                for i in others:
                    st = lib.gslc_interpolate_raster(
                        ctx, C.c_void_p(coords[0].data_ptr()), C.c_void_p(coords[1].data_ptr()), g.length * g.width,
                        C.c_void_p(ins[i].ptr()), rgrid.length, rgrid.width, C.c_void_p(outs[i].ptr()),
                        int(raster_datatypes[i]), int(DataInterpMethod(data_interp_methods[i])),
                        float(invalid_values[i]), C.c_void_p(s.cuda_stream))
                    L.check(st, ctx, "geocode_rasters")
                for o in outs + [e for e in extra if e is not None]:
                    o.copy_back()
                del dem_keep, ss, ins
