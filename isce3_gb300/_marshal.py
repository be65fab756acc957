"""Conversion of the host object model into the C-ABI descriptors of gslc.h.

Device copies of small metadata (LUT2d samples, subswath intervals, DEM
windows) are cached on the objects, so repeated calls and the resident serving
path upload them once.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib as L
from .core import LUT2d, Poly2d, Orbit, OrbitInterpMethod
from .product import GeoGridParameters, RadarGridParameters, SubSwaths


def device_of(device) -> torch.device:
    if device is None:
        device = torch.cuda.current_device() if torch.cuda.is_available() else 0
    if isinstance(device, int):
        return torch.device("cuda", device)
    return torch.device(device)


def _cached_device(obj, key, make):
    cache = obj.__dict__.setdefault("_gslc_dev", {})
    if key not in cache:
        cache[key] = make()
    return cache[key]


def lut_desc(lut: LUT2d, dev: torch.device) -> L.Lut2d:
    d = L.Lut2d()
    d.have_data = int(lut.have_data)
    d.bounds_error = int(lut.bounds_error)
    d.method = int(lut.interp_method)
    d.ref_value = float(lut.ref_value)
    if lut.have_data:
        d.nx, d.ny = lut.width, lut.length
        d.x0, d.y0, d.dx, d.dy = lut.x_start, lut.y_start, lut.x_spacing, lut.y_spacing
        t = _cached_device(lut, (str(dev), "data"),
                           lambda: torch.from_numpy(np.ascontiguousarray(lut.data, dtype=np.float64)).to(dev))
        d.data = t.data_ptr()
    else:
        d.nx = d.ny = 0
        d.dx = d.dy = 1.0
    return d


class AzRgHolder:
    """Keeps host coefficient buffers alive while a descriptor is in use."""

    def __init__(self):
        self.keep = []


def azrg_desc(f, dev: torch.device, holder: AzRgHolder) -> L.AzRgFunc:
    d = L.AzRgFunc()
    if isinstance(f, Poly2d):
        d.kind = 1
        d.poly.x_order, d.poly.y_order = f.x_order, f.y_order
        d.poly.x_mean, d.poly.y_mean = f.x_mean, f.y_mean
        d.poly.x_norm, d.poly.y_norm = f.x_std, f.y_std
        c = np.ascontiguousarray(f.coeffs, dtype=np.float64).ravel()
        if c.size == 0:
            c = np.zeros(1)
        holder.keep.append(c)
        d.poly.coeffs = c.ctypes.data_as(C.POINTER(C.c_double))
    elif isinstance(f, LUT2d):
        d.kind = 0
        d.lut = lut_desc(f, dev)
    else:
        raise TypeError(f"carrier must be LUT2d or Poly2d, got {type(f).__name__}")
    return d


def radar_grid_desc(g: RadarGridParameters) -> L.RadarGrid:
    d = L.RadarGrid()
    d.sensing_start, d.wavelength, d.prf = g.sensing_start, g.wavelength, g.prf
    d.starting_range, d.range_pixel_spacing = g.starting_range, g.range_pixel_spacing
    d.look_side = int(g.lookside)
    d.length, d.width = g.length, g.width
    return d


def geo_grid_desc(g: GeoGridParameters) -> L.GeoGrid:
    d = L.GeoGrid()
    d.start_x, d.start_y, d.spacing_x, d.spacing_y = g.start_x, g.start_y, g.spacing_x, g.spacing_y
    d.width, d.length, d.epsg = g.width, g.length, g.epsg
    return d


def orbit_desc(o: Orbit) -> L.OrbitDesc:
    d = L.OrbitDesc()
    d.t0, d.spacing, d.n = o.t0, o.spacing, o.size
    d.method = 0 if o.interp_method == OrbitInterpMethod.HERMITE else 1
    d.pos = o.position.ctypes.data_as(C.POINTER(C.c_double))
    d.vel = o.velocity.ctypes.data_as(C.POINTER(C.c_double))
    return d


def dem_raster_desc(raster, geogrid: GeoGridParameters, margin: int, dev: torch.device):
    """Descriptor with only the DEM window of ``geogrid`` resident on ``dev``
    (or the whole raster, when ``raster.to_device`` made it resident)."""
    if raster.data.ndim != 2:
        raise ValueError("a DEM raster has one band")
    res = getattr(raster, "resident", None)
    if res is not None and res.device == dev:
        return dem_raster_desc_resident(res, raster.get_geotransform(), raster.get_epsg()), res
    d = L.DemRaster()
    d.width, d.length = raster.width, raster.length
    gt = raster.get_geotransform()
    for i in range(6):
        d.gt[i] = gt[i]
    d.epsg = raster.get_epsg()
    w = L.DemWindow()
    g = geo_grid_desc(geogrid)
    st = L.lib().gslc_compute_dem_window(C.byref(d), C.byref(g), int(margin), C.byref(w))
    if st == L.GSLC_EPROJ:
        raise ValueError("projection transformation between geogrid and DEM failed")
    if st == L.GSLC_EUNSUPPORTED:
        raise NotImplementedError("DEM and geogrid EPSG must be 4326 or UTM, without rotation")
    if st != L.GSLC_OK:
        raise ValueError(f"invalid DEM raster (status {st})")
    if not w.have_raster:
        d.data = None
        return d, None
    if w.wraps:
        raise NotImplementedError("DEM window crossing the DEM file discontinuity")
    key = (str(dev), "win", w.x_off, w.y_off, w.width, w.length)

    def make():
        sub = np.ascontiguousarray(raster.data[w.y_off:w.y_off + w.length, w.x_off:w.x_off + w.width],
                                   dtype=np.float32)
        return torch.from_numpy(sub).to(dev)

    t = _cached_device(raster, key, make)
    d.data = t.data_ptr()
    d.data_x_off, d.data_y_off = w.x_off, w.y_off
    d.data_width, d.data_length, d.data_stride = w.width, w.length, w.width
    return d, t


def dem_raster_desc_deferred(raster, geogrid: GeoGridParameters, margin: int, dev: torch.device):
    """As dem_raster_desc, but a window that is not on the device yet is only
    allocated there: the geocode call uploads it (gslc_geocode_slc_host_io).
    Returns (descriptor, device tensor, host address of the window's first
    sample or None, host row stride in samples, commit) where commit() keeps
    the device window cached on the raster once the call has filled it."""
    res = getattr(raster, "resident", None)
    if (res is not None and res.device == dev) or raster.data.dtype != np.float32 or \
            not raster.data.flags.c_contiguous:
        d, t = dem_raster_desc(raster, geogrid, margin, dev)
        return d, t, None, 0, lambda: None
    if raster.data.ndim != 2:
        raise ValueError("a DEM raster has one band")
    d = L.DemRaster()
    d.width, d.length = raster.width, raster.length
    gt = raster.get_geotransform()
    for i in range(6):
        d.gt[i] = gt[i]
    d.epsg = raster.get_epsg()
    w = L.DemWindow()
    g = geo_grid_desc(geogrid)
    st = L.lib().gslc_compute_dem_window(C.byref(d), C.byref(g), int(margin), C.byref(w))
    if st == L.GSLC_EPROJ:
        raise ValueError("projection transformation between geogrid and DEM failed")
    if st == L.GSLC_EUNSUPPORTED:
        raise NotImplementedError("DEM and geogrid EPSG must be 4326 or UTM, without rotation")
    if st != L.GSLC_OK:
        raise ValueError(f"invalid DEM raster (status {st})")
    if not w.have_raster:
        d.data = None
        return d, None, None, 0, lambda: None
    if w.wraps:
        raise NotImplementedError("DEM window crossing the DEM file discontinuity")
    key = (str(dev), "win", w.x_off, w.y_off, w.width, w.length)
    cache = raster.__dict__.setdefault("_gslc_dev", {})
    host = None
    if key in cache:
        t = cache[key]

        def commit():
            return None
    else:
        t = torch.empty((w.length, w.width), dtype=torch.float32, device=dev)
        host = raster.data.ctypes.data + (w.y_off * raster.width + w.x_off) * 4

        def commit():
            cache[key] = t
    d.data = t.data_ptr()
    d.data_x_off, d.data_y_off = w.x_off, w.y_off
    d.data_width, d.data_length, d.data_stride = w.width, w.length, w.width
    return d, t, host, raster.width, commit


def dem_raster_desc_blocks(raster, geogrid: GeoGridParameters, lines_per_block: int, margin: int,
                           dev: torch.device, whole_window: bool = False):
    """Descriptor whose device samples cover the DEM window of every block of
    ``lines_per_block`` geogrid lines (each block loads its own window, as
    cuda/geocode/Geocode.cu:402-407 and geocode/geocodeSlc.cpp:653-656 do):
    the union of those windows (and, with ``whole_window``, of the whole
    geogrid's window) is uploaded once, or the resident raster is used."""
    if raster.data.ndim != 2:
        raise ValueError("a DEM raster has one band")
    res = getattr(raster, "resident", None)
    if res is not None and res.device == dev:
        return dem_raster_desc_resident(res, raster.get_geotransform(), raster.get_epsg()), res
    d = L.DemRaster()
    d.width, d.length = raster.width, raster.length
    gt = raster.get_geotransform()
    for i in range(6):
        d.gt[i] = gt[i]
    d.epsg = raster.get_epsg()
    g = geo_grid_desc(geogrid)
    lib = L.lib()
    x0 = y0 = None
    x1 = y1 = None
    blocks = [(ls, min(lines_per_block, geogrid.length - ls)) for ls in range(0, geogrid.length, lines_per_block)]
    if whole_window:
        blocks.append((0, geogrid.length))
    for line_start, n in blocks:
        w = L.DemWindow()
        st = lib.gslc_compute_dem_window_block(C.byref(d), C.byref(g), int(line_start), int(n), int(geogrid.width),
                                               int(margin), C.byref(w))
        if st == L.GSLC_EPROJ:
            raise ValueError("projection transformation between geogrid and DEM failed")
        if st == L.GSLC_EUNSUPPORTED:
            raise NotImplementedError("DEM and geogrid EPSG must be 4326 or UTM, without rotation")
        if st != L.GSLC_OK:
            raise ValueError(f"invalid DEM raster (status {st})")
        if w.wraps:
            raise NotImplementedError("DEM window crossing the DEM file discontinuity")
        if not w.have_raster:
            continue
        x0 = w.x_off if x0 is None else min(x0, w.x_off)
        y0 = w.y_off if y0 is None else min(y0, w.y_off)
        x1 = w.x_off + w.width if x1 is None else max(x1, w.x_off + w.width)
        y1 = w.y_off + w.length if y1 is None else max(y1, w.y_off + w.length)
    if x0 is None:
        d.data = None
        return d, None
    key = (str(dev), "win", x0, y0, x1 - x0, y1 - y0)

    def make():
        sub = np.ascontiguousarray(raster.data[y0:y1, x0:x1], dtype=np.float32)
        return torch.from_numpy(sub).to(dev)

    t = _cached_device(raster, key, make)
    d.data = t.data_ptr()
    d.data_x_off, d.data_y_off = x0, y0
    d.data_width, d.data_length, d.data_stride = x1 - x0, y1 - y0, x1 - x0
    return d, t


def dem_raster_desc_resident(raster_tensor: torch.Tensor, geotransform, epsg: int) -> L.DemRaster:
    """Descriptor of a whole DEM raster already resident on the device."""
    d = L.DemRaster()
    d.length, d.width = raster_tensor.shape
    for i in range(6):
        d.gt[i] = float(geotransform[i])
    d.epsg = int(epsg)
    d.data = raster_tensor.data_ptr()
    d.data_x_off = d.data_y_off = 0
    d.data_width, d.data_length, d.data_stride = d.width, d.length, d.width
    return d


def subswaths_desc(s: SubSwaths, dev: torch.device):
    d = L.SubSwathsDesc()
    d.n = s.num_sub_swaths
    d.length, d.width = s.length, s.width
    t = _cached_device(s, (str(dev), id(s._arrays), tuple(a.ctypes.data for a in s._arrays)),
                       lambda: torch.from_numpy(s.packed()).to(dev))
    d.valid = t.data_ptr()
    return d
