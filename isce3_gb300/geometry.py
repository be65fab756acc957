"""Block-planning geometry: radar bounding boxes of geogrids and DEM statistics.

Mirrors the parts of ``isce3.geometry`` that the GSLC workflow's block loop
uses (python/packages/isce3/core/rdr_geo_block_generator.py:7-117):

- ``RadarGridBoundingBox`` (python/extensions/pybind_isce3/geometry/boundingbox.cpp:22-39),
- ``Geo2RdrParams`` (python/extensions/pybind_isce3/geometry/geo2rdr.cpp:26-37),
- ``get_radar_bbox`` with its two overloads, min/max heights or a DEM
  (boundingbox.cpp:82-160 over cxx/isce3/geometry/boundingbox.cpp:413-641),
- ``DEMInterpolator`` construction from a raster and
  ``compute_min_max_mean_height`` (cxx/isce3/geometry/DEMInterpolator.cpp:515-560).

The work runs on the GPU through libgslc.so: ``get_radar_bboxes`` plans any
number of geogrid blocks in one kernel launch (eight geo2rdr sequences per
block, one thread each); ``get_radar_bbox`` is its one-block case.  Failures
raise ``RuntimeError`` with the reference's messages, which is what
``block_generator`` catches to skip a block.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib as L
from . import _marshal as M
from .core import LUT2d, Orbit
from .product import GeoGridParameters, RadarGridParameters

GLOBAL_MIN_HEIGHT = -500.0   # cxx/isce3/core/Constants.h:53
GLOBAL_MAX_HEIGHT = 9000.0   # cxx/isce3/core/Constants.h:56


@dataclass
class Geo2RdrParams:
    """geometry/detail/Geo2Rdr.h:13-22: threshold (s), maxiter, delta_range (m)."""
    threshold: float = 1e-8
    maxiter: int = 50
    delta_range: float = 10.0


@dataclass
class RadarGridBoundingBox:
    """Indices of a radar-grid bounding box (inclusive last line/sample)."""
    first_azimuth_line: int
    last_azimuth_line: int
    first_range_sample: int
    last_range_sample: int


class DEMInterpolator:
    """The DEM heights a planner needs: a constant reference height, or a
    raster whose statistics come from the GPU.

    ``DEMInterpolator(height)`` and ``DEMInterpolator(raster)`` follow the
    pybind constructors (python/extensions/pybind_isce3/geometry/DEMInterpolator.cpp:24-44;
    the raster form loads the whole raster like ``loadDEM(raster)``).
    """

    def __init__(self, height_or_raster=0.0, method=None, epsg: int = 4326):
        self.raster = None
        self.ref_height = 0.0
        if isinstance(height_or_raster, (int, float)):
            self.ref_height = float(height_or_raster)
            self.epsg_code = int(epsg)
        else:
            self.raster = height_or_raster
            self.epsg_code = int(height_or_raster.get_epsg())
        self._stats = None

    @property
    def have_raster(self) -> bool:
        return self.raster is not None

    def compute_min_max_mean_height(self, device=None):
        """(min, max, mean) of the DEM (DEMInterpolator.cpp:515-560): the
        reference height without a raster; NaN samples skipped; the reference
        height becomes the mean, as there."""
        if not self.have_raster:
            return (np.float32(self.ref_height),) * 3
        if self._stats is None:
            self._stats = dem_stats(self.raster, device)
            self.ref_height = float(self._stats[2])
        return self._stats

    @property
    def min_height(self) -> float:
        return float(self.compute_min_max_mean_height()[0])

    @property
    def max_height(self) -> float:
        return float(self.compute_min_max_mean_height()[1])

    @property
    def mean_height(self) -> float:
        return float(self.compute_min_max_mean_height()[2])


def dem_stats(raster, device=None):
    """Min, max (float32) and mean (float64) of a DEM raster's non-NaN samples
    on the GPU, folded in a fixed order."""
    dev = M.device_of(device)
    res = getattr(raster, "resident", None)
    if res is not None and res.device == dev:
        t = res
    else:
        t = torch.from_numpy(np.ascontiguousarray(raster.data, dtype=np.float32)).to(dev)
    if t.dtype != torch.float32 or t.dim() != 2 or t.stride(1) != 1:
        raise ValueError("DEM raster must be a 2-D float32 array with unit column stride")
    lib = L.lib()
    ctx = L.context(dev.index)
    mn, mx, mean, nv = C.c_float(), C.c_float(), C.c_double(), C.c_int64()
    s = torch.cuda.current_stream(dev)
    L.check(lib.gslc_dem_stats(ctx, C.c_void_p(t.data_ptr()), t.shape[0], t.shape[1], t.stride(0), C.byref(mn),
                               C.byref(mx), C.byref(mean), C.byref(nv), C.c_void_p(s.cuda_stream)), ctx,
            "dem_stats")
    return np.float32(mn.value), np.float32(mx.value), float(mean.value)


def _bbox_error(status: int, detail: int) -> str:
    if status == 1:
        # corner bit 2 * line + pixel; line 0 is the geogrid's first row
        # (north when spacing_y < 0), named as boundingbox.cpp:599-603 does
        names = ""
        for k in range(4):
            if detail >> k & 1:
                line, pixel = k >> 1, k & 1
                names += "(" + ("north" if line == 1 else "south") + ("east" if pixel == 1 else "west") + ") "
        return "ERROR: geo2rdr computations did not converge for at corner(s) " + names
    if status == 2:
        msg = "ERROR: The computed radar bounding box does not overlap with the input radar grid."
        if detail & 1:
            msg += " Azimuth first and last <= 0."
        if detail & 2:
            msg += " Azimuth first and last >= max azimuth."
        if detail & 4:
            msg += " Range first and last <= 0."
        if detail & 8:
            msg += " Range first and last >= max range."
        return msg
    return "Inverse projection transformation failed"


def get_radar_bboxes(geo_grids, radar_grid: RadarGridParameters, orbit: Orbit, min_height: float = GLOBAL_MIN_HEIGHT,
                     max_height: float = GLOBAL_MAX_HEIGHT, doppler: LUT2d | None = None, margin: int = 50,
                     geo2rdr_params: Geo2RdrParams | None = None, geogrid_expansion_threshold: int = 100,
                     device=None):
    """Bounding boxes of many geogrids (one EPSG) in one GPU launch.

    Returns a list with a ``RadarGridBoundingBox`` for each geogrid, or the
    ``RuntimeError`` the reference would raise for it.  Argument errors
    raise ``ValueError`` (the reference's InvalidArgument / OutOfRange).
    """
    geo_grids = list(geo_grids)
    if not geo_grids:
        return []
    epsg = geo_grids[0].epsg
    if any(g.epsg != epsg for g in geo_grids):
        raise ValueError("all geogrids of one planning call share an EPSG code")
    dev = M.device_of(device)
    doppler = doppler if doppler is not None else LUT2d()
    p = geo2rdr_params or Geo2RdrParams()
    blocks = (L.GeoBlock * len(geo_grids))()
    for b, g in zip(blocks, geo_grids):
        b.start_x, b.start_y, b.spacing_x, b.spacing_y = g.start_x, g.start_y, g.spacing_x, g.spacing_y
        b.width, b.length = g.width, g.length
    a = L.BBoxArgs()
    a.radar_grid = M.radar_grid_desc(radar_grid)
    a.orbit = M.orbit_desc(orbit)
    a.doppler = M.lut_desc(doppler, dev)
    a.epsg = epsg
    a.n_blocks = len(geo_grids)
    a.blocks = C.cast(blocks, C.c_void_p)
    a.min_height, a.max_height = float(np.float32(min_height)), float(np.float32(max_height))
    a.margin = int(margin)
    a.geogrid_expansion_threshold = int(geogrid_expansion_threshold)
    a.threshold, a.maxiter, a.delta_range = float(p.threshold), int(p.maxiter), float(p.delta_range)
    out = (L.RadarBBox * len(geo_grids))()
    lib = L.lib()
    ctx = L.context(dev.index)
    s = torch.cuda.current_stream(dev)
    L.check(lib.gslc_radar_bbox_blocks(ctx, C.byref(a), C.cast(out, C.c_void_p), C.c_void_p(s.cuda_stream)), ctx,
            "get_radar_bbox")
    res = []
    for o in out:
        if o.status == 0:
            res.append(RadarGridBoundingBox(o.first_azimuth_line, o.last_azimuth_line, o.first_range_sample,
                                            o.last_range_sample))
        else:
            res.append(RuntimeError(_bbox_error(o.status, o.detail)))
    return res


def get_radar_bbox(geo_grid: GeoGridParameters, radar_grid: RadarGridParameters, orbit: Orbit, *args, **kwargs):
    """``isce3.geometry.get_radar_bbox`` (both overloads).

    ``get_radar_bbox(geo_grid, radar_grid, orbit, min_height=-500,
    max_height=9000, doppler=LUT2d(), margin=50, geo2rdr_params=Geo2RdrParams(),
    geogrid_expansion_threshold=100)`` or, with a ``DEMInterpolator`` in
    fourth place or as ``dem=``, ``get_radar_bbox(geo_grid, radar_grid, orbit,
    dem, doppler=LUT2d(), margin=5, ...)`` whose heights are the DEM's
    min and max (boundingbox.cpp:413-432).
    """
    dem = kwargs.pop("dem", None)
    if dem is None and args and isinstance(args[0], DEMInterpolator):
        dem, args = args[0], args[1:]
    device = kwargs.pop("device", None)
    if dem is not None:
        names = ["doppler", "margin", "geo2rdr_params", "geogrid_expansion_threshold"]
        kw = dict(zip(names, args))
        kw.update(kwargs)
        kw.setdefault("margin", 5)
        mn, mx, _ = dem.compute_min_max_mean_height(device)
        r = get_radar_bboxes([geo_grid], radar_grid, orbit, float(mn), float(mx), device=device, **kw)[0]
    else:
        names = ["min_height", "max_height", "doppler", "margin", "geo2rdr_params", "geogrid_expansion_threshold"]
        kw = dict(zip(names, args))
        kw.update(kwargs)
        r = get_radar_bboxes([geo_grid], radar_grid, orbit, device=device, **kw)[0]
    if isinstance(r, Exception):
        raise r
    return r


_CUBE_OUTPUTS = [("slant_range_raster", "slant_range", np.float64),
                 ("azimuth_time_raster", "azimuth_time", np.float64),
                 ("incidence_angle_raster", "incidence_angle", np.float32),
                 ("los_unit_vector_x_raster", "los_unit_vector_x", np.float32),
                 ("los_unit_vector_y_raster", "los_unit_vector_y", np.float32),
                 ("along_track_unit_vector_x_raster", "along_track_unit_vector_x", np.float32),
                 ("along_track_unit_vector_y_raster", "along_track_unit_vector_y", np.float32),
                 ("elevation_angle_raster", "elevation_angle", np.float32),
                 ("ground_track_velocity_raster", "ground_track_velocity", np.float64)]
_TORCH = {np.float64: torch.float64, np.float32: torch.float32}


def make_radar_grid_cubes(radar_grid: RadarGridParameters, geogrid: GeoGridParameters, heights, orbit: Orbit,
                          native_doppler: LUT2d, grid_doppler: LUT2d, slant_range_raster=None,
                          azimuth_time_raster=None, incidence_angle_raster=None, los_unit_vector_x_raster=None,
                          los_unit_vector_y_raster=None, along_track_unit_vector_x_raster=None,
                          along_track_unit_vector_y_raster=None, elevation_angle_raster=None,
                          ground_track_velocity_raster=None, threshold_geo2rdr: float = 1e-8,
                          numiter_geo2rdr: int = 50, delta_range: float = 10.0,
                          flag_set_output_rasters_geolocation: bool = False, *, device=None,
                          lo_unit_vector_x_raster=None) -> None:
    """``isce3.geometry.make_radar_grid_cubes`` on the GPU, one launch.

    Argument order and defaults follow the pybind binding
    (python/extensions/pybind_isce3/geometry/metadataCubes.cpp:16-35, whose
    keyword for the LOS x cube is ``lo_unit_vector_x_raster``; both names are
    accepted).  Each output is an array of shape (len(heights), length,
    width) — NumPy (host) or a CUDA torch tensor — of float64 (slant range,
    azimuth time, ground-track velocity) or float32 (the angles and unit
    vectors), or None to skip it.  Band k of the reference's rasters is
    plane k here.  Points where geo2rdr does not converge are NaN.
    ``flag_set_output_rasters_geolocation`` only tags GDAL rasters in the
    reference and has nothing to tag here.
    """
    if lo_unit_vector_x_raster is not None:
        if los_unit_vector_x_raster is not None:
            raise ValueError("give one of lo_unit_vector_x_raster and los_unit_vector_x_raster")
        los_unit_vector_x_raster = lo_unit_vector_x_raster
    given = dict(slant_range_raster=slant_range_raster, azimuth_time_raster=azimuth_time_raster,
                 incidence_angle_raster=incidence_angle_raster, los_unit_vector_x_raster=los_unit_vector_x_raster,
                 los_unit_vector_y_raster=los_unit_vector_y_raster,
                 along_track_unit_vector_x_raster=along_track_unit_vector_x_raster,
                 along_track_unit_vector_y_raster=along_track_unit_vector_y_raster,
                 elevation_angle_raster=elevation_angle_raster,
                 ground_track_velocity_raster=ground_track_velocity_raster)
    h = np.ascontiguousarray(np.asarray(heights, dtype=np.float64).ravel())
    shape = (h.size, geogrid.length, geogrid.width)
    dev = M.device_of(device)
    a = L.CubeArgs()
    a.radar_grid = M.radar_grid_desc(radar_grid)
    a.geo_grid = M.geo_grid_desc(geogrid)
    a.heights = h.ctypes.data
    a.n_heights = h.size
    a.maxiter = int(numiter_geo2rdr)
    a.orbit = M.orbit_desc(orbit)
    a.native_doppler = M.lut_desc(native_doppler if native_doppler is not None else LUT2d(), dev)
    a.grid_doppler = M.lut_desc(grid_doppler if grid_doppler is not None else LUT2d(), dev)
    a.threshold, a.delta_range = float(threshold_geo2rdr), float(delta_range)
    copies = []
    keep = [h]
    for name, field, dt in _CUBE_OUTPUTS:
        arr = given[name]
        if arr is None:
            continue
        if tuple(arr.shape) != shape:
            raise ValueError(f"{name}: shape {tuple(arr.shape)} != (heights, length, width) {shape}")
        if isinstance(arr, torch.Tensor) and arr.device.type == "cuda":
            if arr.dtype != _TORCH[dt] or not arr.is_contiguous():
                raise ValueError(f"{name}: must be a C-contiguous {np.dtype(dt).name} tensor")
            t = arr
        else:
            if np.asarray(arr).dtype != dt:
                raise ValueError(f"{name}: dtype must be {np.dtype(dt).name}")
            t = torch.empty(shape, dtype=_TORCH[dt], device=dev)
            copies.append((arr, t))
        keep.append(t)
        setattr(a, field, t.data_ptr())
    lib = L.lib()
    ctx = L.context(dev.index)
    s = torch.cuda.current_stream(dev)
    L.check(lib.gslc_make_radar_grid_cubes(ctx, C.byref(a), C.c_void_p(s.cuda_stream)), ctx,
            "make_radar_grid_cubes")
    for host, t in copies:
        if isinstance(host, torch.Tensor):
            host.copy_(t)
        else:
            host[...] = t.cpu().numpy()
