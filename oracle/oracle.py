"""ctypes front end of the CPU oracle (oracle/gslc_oracle.cpp).

TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg use it as the checker.  The product (isce3_gb300) never
imports it.  It takes the same host objects as isce3_gb300.geocode.geocode_slc
(read by attribute) and runs the C++ restatement of the reference.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libgslc_oracle.so"
# Build variants: "" is the oracle proper (-ffp-contract=off, the reference's
# x86-64 arithmetic on any host); "fma" is the same source with
# floating-point contraction on (oracle/Makefile, target fma), used only to
# measure how far two correct builds of one code disagree.
_VARIANTS = {"": ("all", LIB), "fma": ("fma", HERE / "_build" / "libgslc_oracle_fma.so")}


def build(force: bool = False, variant: str = "") -> Path:
    target, lib_path = _VARIANTS[variant]
    src = [HERE / "gslc_oracle.cpp", HERE / "gslc_oracle.h"]
    if force or not lib_path.exists() or lib_path.stat().st_mtime < max(p.stat().st_mtime for p in src):
        cmd = ["make", "-C", str(HERE)] + (["-B"] if force else []) + [target]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return lib_path


class Lut(C.Structure):
    _fields_ = [("have_data", C.c_int32), ("bounds_error", C.c_int32), ("method", C.c_int32),
                ("nx", C.c_int32), ("ny", C.c_int32), ("x0", C.c_double), ("y0", C.c_double),
                ("dx", C.c_double), ("dy", C.c_double), ("ref_value", C.c_double), ("data", C.c_void_p)]


class Poly(C.Structure):
    _fields_ = [("x_order", C.c_int32), ("y_order", C.c_int32), ("x_mean", C.c_double), ("y_mean", C.c_double),
                ("x_norm", C.c_double), ("y_norm", C.c_double), ("coeffs", C.c_void_p)]


class AzRg(C.Structure):
    _fields_ = [("kind", C.c_int32), ("lut", Lut), ("poly", Poly)]


class RadarGrid(C.Structure):
    _fields_ = [("sensing_start", C.c_double), ("wavelength", C.c_double), ("prf", C.c_double),
                ("starting_range", C.c_double), ("range_pixel_spacing", C.c_double), ("look_side", C.c_int32),
                ("length", C.c_int64), ("width", C.c_int64)]


class GeoGrid(C.Structure):
    _fields_ = [("start_x", C.c_double), ("start_y", C.c_double), ("spacing_x", C.c_double),
                ("spacing_y", C.c_double), ("width", C.c_int32), ("length", C.c_int32), ("epsg", C.c_int32)]


class OrbitS(C.Structure):
    _fields_ = [("t0", C.c_double), ("spacing", C.c_double), ("n", C.c_int32), ("method", C.c_int32),
                ("pos", C.c_void_p), ("vel", C.c_void_p)]


class DemRaster(C.Structure):
    _fields_ = [("data", C.c_void_p), ("width", C.c_int64), ("length", C.c_int64), ("gt", C.c_double * 6),
                ("epsg", C.c_int32)]


class SubSw(C.Structure):
    _fields_ = [("n", C.c_int32), ("length", C.c_int64), ("width", C.c_int64), ("valid", C.c_void_p)]


class Args(C.Structure):
    _fields_ = [("radar_grid", RadarGrid), ("sliced_radar_grid", RadarGrid), ("geo_grid", GeoGrid),
                ("orbit", OrbitS), ("native_doppler", Lut), ("image_grid_doppler", Lut),
                ("az_time_correction", Lut), ("srange_correction", Lut), ("az_carrier", AzRg),
                ("rg_carrier", AzRg), ("ell_a", C.c_double), ("ell_e2", C.c_double),
                ("threshold_geo2rdr", C.c_double), ("numiter_geo2rdr", C.c_int32),
                ("first_azimuth_line", C.c_int64), ("first_range_sample", C.c_int64),
                ("flatten", C.c_int32), ("reramp", C.c_int32), ("flatten_with_corrected_srange", C.c_int32),
                ("invalid_re", C.c_float), ("invalid_im", C.c_float), ("n_blocks", C.c_int32),
                ("rdr_length", C.c_int64), ("rdr_width", C.c_int64), ("rdr_blocks", C.POINTER(C.c_void_p)),
                ("geo_blocks", C.POINTER(C.c_void_p)), ("mask", C.c_void_p), ("carrier_phase", C.c_void_p),
                ("flatten_phase", C.c_void_p), ("dem", DemRaster), ("subswaths", C.POINTER(SubSw)),
                ("out_az_index", C.c_void_p), ("out_rg_index", C.c_void_p),
                ("out_uncorrected_srange", C.c_void_p), ("dem_margin", C.c_int32), ("nthreads", C.c_int32),
                ("phase_seconds", C.c_double * 4), ("out_niter", C.c_void_p)]


class RasterArgs(C.Structure):
    _fields_ = [("radar_grid", RadarGrid), ("geo_grid", GeoGrid), ("orbit", OrbitS), ("doppler", Lut),
                ("native_doppler", Lut), ("az_time_correction", Lut), ("srange_correction", Lut),
                ("ell_a", C.c_double), ("ell_e2", C.c_double), ("threshold", C.c_double),
                ("delta_range", C.c_double), ("maxiter", C.c_int32), ("lines_per_block", C.c_int32),
                ("n_rasters", C.c_int32), ("dem_margin", C.c_int32), ("input_rasters", C.POINTER(C.c_void_p)),
                ("output_rasters", C.POINTER(C.c_void_p)), ("invalid_values", C.POINTER(C.c_double)),
                ("dem", DemRaster), ("subswaths", C.POINTER(SubSw)), ("out_az_index", C.c_void_p),
                ("out_rg_index", C.c_void_p), ("nthreads", C.c_int32)]


_libs: dict = {}


def lib(variant: str = "") -> C.CDLL:
    _lib = _libs.get(variant)
    if _lib is None:
        _lib = C.CDLL(str(build(variant=variant)))
        _libs[variant] = _lib
        _lib.orc_geocode_slc.restype = C.c_int
        _lib.orc_geocode_slc.argtypes = [C.POINTER(Args)]
        _lib.orc_geocode_slc_raster.restype = C.c_int
        _lib.orc_geocode_slc_raster.argtypes = [C.POINTER(Args), C.c_int32]
        _lib.orc_geocode_rasters.restype = C.c_int
        _lib.orc_geocode_rasters.argtypes = [C.POINTER(RasterArgs)]
        _lib.orc_last_error.restype = C.c_char_p
        _lib.orc_orbit_interpolate.argtypes = [C.POINTER(OrbitS), C.c_double, C.c_void_p, C.c_void_p]
        _lib.orc_interp2d_double.restype = C.c_double
        _lib.orc_interp2d_double.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_double]
        _lib.orc_spline2d_float.restype = C.c_float
        _lib.orc_spline2d_float.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_double]
        _lib.orc_sinc2d_cfloat.restype = None
        _lib.orc_sinc2d_cfloat.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_double, C.c_void_p]
        _lib.orc_lut2d_eval.restype = C.c_double
        _lib.orc_lut2d_eval.argtypes = [C.POINTER(Lut), C.c_double, C.c_double]
        _lib.orc_lut2d_contains.argtypes = [C.POINTER(Lut), C.c_double, C.c_double]
        _lib.orc_poly2d_eval.restype = C.c_double
        _lib.orc_poly2d_eval.argtypes = [C.POINTER(Poly), C.c_double, C.c_double]
        _lib.orc_proj_forward.argtypes = [C.c_int, C.c_void_p, C.c_void_p]
        _lib.orc_proj_inverse.argtypes = [C.c_int, C.c_void_p, C.c_void_p]
        _lib.orc_lonlat_to_xyz.argtypes = [C.c_double, C.c_double, C.c_void_p, C.c_void_p]
        _lib.orc_geo2rdr.argtypes = [C.c_void_p, C.c_double, C.c_double, C.POINTER(OrbitS), C.POINTER(Lut),
                                     C.c_void_p, C.c_void_p, C.c_double, C.c_int, C.c_double, C.c_int, C.c_double]
        _lib.orc_sinc_table.argtypes = [C.c_void_p]
        _lib.orc_dem_subset.argtypes = [C.POINTER(DemRaster), C.POINTER(GeoGrid), C.c_int] + [C.c_void_p] * 6
        _lib.orc_radar_bbox.argtypes = [C.POINTER(GeoGrid), C.POINTER(RadarGrid), C.POINTER(OrbitS), C.POINTER(Lut),
                                        C.c_float, C.c_float, C.c_int, C.c_double, C.c_int, C.c_double, C.c_int,
                                        C.c_void_p]
        _lib.orc_radar_grid_cubes.argtypes = [C.POINTER(RadarGrid), C.POINTER(GeoGrid), C.c_void_p, C.c_int,
                                              C.POINTER(OrbitS), C.POINTER(Lut), C.POINTER(Lut), C.c_double, C.c_int,
                                              C.c_double] + [C.c_void_p] * 9 + [C.c_int]
        _lib.orc_interpolate_raster.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_int64,
                                                C.c_void_p, C.c_int, C.c_int, C.c_double]
        _lib.orc_dem_stats.argtypes = [C.c_void_p, C.c_int64, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_void_p]
    return _lib


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


class _Keep(list):
    def arr(self, a, dtype):
        a = np.ascontiguousarray(a, dtype=dtype)
        self.append(a)
        return a


def lut_struct(lut, keep: _Keep) -> Lut:
    s = Lut()
    s.have_data = int(lut.have_data)
    s.bounds_error = int(lut.bounds_error)
    s.method = int(lut.interp_method)
    s.ref_value = float(lut.ref_value)
    if lut.have_data:
        d = keep.arr(lut.data, np.float64)
        s.nx, s.ny = d.shape[1], d.shape[0]
        s.x0, s.y0, s.dx, s.dy = lut.x_start, lut.y_start, lut.x_spacing, lut.y_spacing
        s.data = _ptr(d)
    return s


def poly_struct(p, keep: _Keep) -> Poly:
    s = Poly()
    s.x_order, s.y_order = p.x_order, p.y_order
    s.x_mean, s.y_mean, s.x_norm, s.y_norm = p.x_mean, p.y_mean, p.x_std, p.y_std
    c = keep.arr(p.coeffs if p.coeffs.size else np.zeros(1), np.float64)
    s.coeffs = _ptr(c)
    return s


def azrg_struct(f, keep: _Keep) -> AzRg:
    s = AzRg()
    if hasattr(f, "x_order"):
        s.kind = 1
        s.poly = poly_struct(f, keep)
    else:
        s.kind = 0
        s.lut = lut_struct(f, keep)
    return s


def radar_struct(g) -> RadarGrid:
    s = RadarGrid()
    s.sensing_start, s.wavelength, s.prf = g.sensing_start, g.wavelength, g.prf
    s.starting_range, s.range_pixel_spacing = g.starting_range, g.range_pixel_spacing
    s.look_side, s.length, s.width = int(g.lookside), g.length, g.width
    return s


def geo_struct(g) -> GeoGrid:
    s = GeoGrid()
    s.start_x, s.start_y, s.spacing_x, s.spacing_y = g.start_x, g.start_y, g.spacing_x, g.spacing_y
    s.width, s.length, s.epsg = g.width, g.length, g.epsg
    return s


def orbit_struct(o, keep: _Keep) -> OrbitS:
    s = OrbitS()
    s.t0, s.spacing, s.n = o.t0, o.spacing, o.size
    s.method = int(o.interp_method)
    s.pos = _ptr(keep.arr(o.position, np.float64))
    s.vel = _ptr(keep.arr(o.velocity, np.float64))
    return s


def dem_struct(r, keep: _Keep) -> DemRaster:
    s = DemRaster()
    d = keep.arr(r.data, np.float32)
    s.data = _ptr(d)
    s.length, s.width = d.shape
    for i, v in enumerate(r.get_geotransform()):
        s.gt[i] = v
    s.epsg = r.get_epsg()
    return s


def geocode_slc(geo_data_blocks, rdr_data_blocks, dem_raster, radargrid, geogrid, orbit, native_doppler,
                image_grid_doppler, ellipsoid, threshold_geo2rdr, num_iter_geo2rdr, mask_block=None,
                sliced_radargrid=None, subswaths=None, first_azimuth_line=0, first_range_sample=0, flatten=True,
                reramp=True, az_carrier=None, rg_carrier=None, az_time_correction=None, srange_correction=None,
                flatten_with_corrected_srange=False, invalid_value=np.nan + np.nan * 1j,
                carrier_phase_block=None, flatten_phase_block=None, *, az_index_block=None, rg_index_block=None,
                uncorrected_srange_block=None, dem_margin=50, nthreads=0, inplace_deramp=False, niter_block=None,
                build_variant=""):
    """Run the oracle with geocode_slc's arguments; outputs are written in place.

    Radar blocks are deramped on copies unless ``inplace_deramp``.  Returns
    the per-phase wall times (index pass, deramp, interpolate, reramp) in s.
    ``build_variant`` selects the oracle build ("" or "fma").
    """
    from isce3_gb300.core import LUT2d
    az_carrier = az_carrier if az_carrier is not None else LUT2d()
    rg_carrier = rg_carrier if rg_carrier is not None else LUT2d()
    az_time_correction = az_time_correction if az_time_correction is not None else LUT2d()
    srange_correction = srange_correction if srange_correction is not None else LUT2d()
    if not isinstance(geo_data_blocks, list):
        geo_data_blocks, rdr_data_blocks = [geo_data_blocks], [rdr_data_blocks]
    keep = _Keep()
    rdr = [r if inplace_deramp else np.array(r, dtype=np.complex64, copy=True) for r in rdr_data_blocks]
    keep.extend(rdr)
    a = Args()
    a.radar_grid = radar_struct(radargrid)
    a.sliced_radar_grid = radar_struct(sliced_radargrid or radargrid)
    a.geo_grid = geo_struct(geogrid)
    a.orbit = orbit_struct(orbit, keep)
    a.native_doppler = lut_struct(native_doppler, keep)
    a.image_grid_doppler = lut_struct(image_grid_doppler, keep)
    a.az_time_correction = lut_struct(az_time_correction, keep)
    a.srange_correction = lut_struct(srange_correction, keep)
    a.az_carrier = azrg_struct(az_carrier, keep)
    a.rg_carrier = azrg_struct(rg_carrier, keep)
    a.ell_a, a.ell_e2 = ellipsoid.a, ellipsoid.e2
    a.threshold_geo2rdr, a.numiter_geo2rdr = threshold_geo2rdr, num_iter_geo2rdr
    a.first_azimuth_line, a.first_range_sample = first_azimuth_line, first_range_sample
    a.flatten, a.reramp = int(flatten), int(reramp)
    a.flatten_with_corrected_srange = int(flatten_with_corrected_srange)
    inv = complex(invalid_value)
    a.invalid_re, a.invalid_im = np.float32(inv.real), np.float32(inv.imag)
    a.n_blocks = len(rdr)
    a.rdr_length, a.rdr_width = rdr[0].shape
    rp = (C.c_void_p * len(rdr))(*[_ptr(r) for r in rdr])
    gp = (C.c_void_p * len(geo_data_blocks))(*[_ptr(g) for g in geo_data_blocks])
    a.rdr_blocks = C.cast(rp, C.POINTER(C.c_void_p))
    a.geo_blocks = C.cast(gp, C.POINTER(C.c_void_p))

    def opt(x):
        return _ptr(x) if x is not None and x.size else None
    a.mask = opt(mask_block)
    a.carrier_phase = opt(carrier_phase_block)
    a.flatten_phase = opt(flatten_phase_block)
    a.out_az_index = opt(az_index_block)
    a.out_rg_index = opt(rg_index_block)
    a.out_uncorrected_srange = opt(uncorrected_srange_block)
    a.out_niter = opt(niter_block)
    a.dem = dem_struct(dem_raster, keep)
    a.dem_margin = dem_margin
    a.nthreads = nthreads
    if subswaths is not None:
        ss = SubSw()
        ss.n, ss.length, ss.width = subswaths.num_sub_swaths, subswaths.length, subswaths.width
        packed = keep.arr(subswaths.packed(), np.int32)
        ss.valid = _ptr(packed)
        keep.append(ss)
        a.subswaths = C.pointer(ss)
    L = lib(build_variant)
    st = L.orc_geocode_slc(C.byref(a))
    if st != 0:
        raise ValueError(L.orc_last_error().decode())
    return list(a.phase_seconds)


def geocode_slc_raster(output_raster, input_raster, dem_raster, radargrid, geogrid, orbit, native_doppler,
                       image_grid_doppler, ellipsoid, threshold_geo2rdr=1.0e-9, numiter_geo2rdr=25,
                       lines_per_block=1000, flatten=True, reramp=True, azimuth_carrier=None, range_carrier=None,
                       az_time_correction=None, srange_correction=None, flatten_with_corrected_srange=False,
                       invalid_value=np.nan + np.nan * 1j, carrier_phase_raster=None, flatten_phase_raster=None, *,
                       az_index_block=None, rg_index_block=None, dem_margin=50, nthreads=0):
    """The raster mode of geocodeSlc (geocode/geocodeSlc.cpp:605-828) on the
    CPU, with the pybind overload's arguments: every band of
    ``input_raster`` (read only) into ``output_raster``, written in place."""
    from isce3_gb300.core import LUT2d, Poly2d
    azimuth_carrier = azimuth_carrier if azimuth_carrier is not None else Poly2d()
    range_carrier = range_carrier if range_carrier is not None else Poly2d()
    az_time_correction = az_time_correction if az_time_correction is not None else LUT2d()
    srange_correction = srange_correction if srange_correction is not None else LUT2d()
    keep = _Keep()
    n = input_raster.num_bands()
    rdr = [np.ascontiguousarray(input_raster.band(i), dtype=np.complex64) for i in range(n)]
    geo = [output_raster.band(i) for i in range(n)]
    for g in geo:
        assert g.flags.c_contiguous and g.dtype == np.complex64
    keep.extend(rdr)
    a = Args()
    a.radar_grid = radar_struct(radargrid)
    a.sliced_radar_grid = radar_struct(radargrid)
    a.geo_grid = geo_struct(geogrid)
    a.orbit = orbit_struct(orbit, keep)
    a.native_doppler = lut_struct(native_doppler, keep)
    a.image_grid_doppler = lut_struct(image_grid_doppler, keep)
    a.az_time_correction = lut_struct(az_time_correction, keep)
    a.srange_correction = lut_struct(srange_correction, keep)
    a.az_carrier = azrg_struct(azimuth_carrier, keep)
    a.rg_carrier = azrg_struct(range_carrier, keep)
    a.ell_a, a.ell_e2 = ellipsoid.a, ellipsoid.e2
    a.threshold_geo2rdr, a.numiter_geo2rdr = threshold_geo2rdr, numiter_geo2rdr
    a.flatten, a.reramp = int(flatten), int(reramp)
    a.flatten_with_corrected_srange = int(flatten_with_corrected_srange)
    inv = complex(invalid_value)
    a.invalid_re, a.invalid_im = np.float32(inv.real), np.float32(inv.imag)
    a.n_blocks = n
    a.rdr_length, a.rdr_width = rdr[0].shape
    rp = (C.c_void_p * n)(*[_ptr(r) for r in rdr])
    gp = (C.c_void_p * n)(*[_ptr(g) for g in geo])
    a.rdr_blocks = C.cast(rp, C.POINTER(C.c_void_p))
    a.geo_blocks = C.cast(gp, C.POINTER(C.c_void_p))

    def opt(x):
        return _ptr(x) if x is not None and x.size else None
    a.carrier_phase = opt(carrier_phase_raster.data if carrier_phase_raster is not None else None)
    a.flatten_phase = opt(flatten_phase_raster.data if flatten_phase_raster is not None else None)
    a.out_az_index = opt(az_index_block)
    a.out_rg_index = opt(rg_index_block)
    a.dem = dem_struct(dem_raster, keep)
    a.dem_margin = dem_margin
    a.nthreads = nthreads
    L = lib()
    st = L.orc_geocode_slc_raster(C.byref(a), int(lines_per_block))
    if st != 0:
        raise ValueError(L.orc_last_error().decode())


def geocode_rasters(output_rasters, input_rasters, radar_geometry, geogrid, dem_raster, lines_per_block=1000,
                    invalid_values=None, native_doppler=None, az_time_correction=None, srange_correction=None,
                    subswaths=None, threshold=1e-8, maxiter=50, delta_range=10.0, *, ellipsoid=None,
                    az_index_block=None, rg_index_block=None, dem_margin=50, nthreads=0):
    """The reference CUDA raster geocoder (Geocode::geocodeRasters, SINC on
    complex64) restated on the CPU; outputs are written in place."""
    from isce3_gb300.core import Ellipsoid, LUT2d
    ellipsoid = ellipsoid or Ellipsoid()
    keep = _Keep()
    n = len(input_rasters)
    ins = [np.ascontiguousarray(r, dtype=np.complex64) for r in input_rasters]
    keep.extend(ins)
    for o in output_rasters:
        if o.dtype != np.complex64 or not o.flags.c_contiguous:
            raise ValueError("outputs must be C-contiguous complex64 arrays")
    a = RasterArgs()
    a.radar_grid = radar_struct(radar_geometry.radar_grid)
    a.geo_grid = geo_struct(geogrid)
    a.orbit = orbit_struct(radar_geometry.orbit, keep)
    a.doppler = lut_struct(radar_geometry.doppler, keep)
    a.native_doppler = lut_struct(native_doppler or LUT2d(), keep)
    a.az_time_correction = lut_struct(az_time_correction or LUT2d(), keep)
    a.srange_correction = lut_struct(srange_correction or LUT2d(), keep)
    a.ell_a, a.ell_e2 = ellipsoid.a, ellipsoid.e2
    a.threshold, a.delta_range = threshold, delta_range
    a.maxiter, a.lines_per_block = maxiter, lines_per_block
    a.n_rasters, a.dem_margin = n, dem_margin
    ip = (C.c_void_p * n)(*[_ptr(r) for r in ins])
    op = (C.c_void_p * n)(*[_ptr(r) for r in output_rasters])
    iv = (C.c_double * n)(*([np.nan] * n if invalid_values is None else [float(v) for v in invalid_values]))
    keep.extend([ip, op, iv])
    a.input_rasters = C.cast(ip, C.POINTER(C.c_void_p))
    a.output_rasters = C.cast(op, C.POINTER(C.c_void_p))
    a.invalid_values = C.cast(iv, C.POINTER(C.c_double))
    a.dem = dem_struct(dem_raster, keep)
    a.out_az_index = _ptr(az_index_block) if az_index_block is not None else None
    a.out_rg_index = _ptr(rg_index_block) if rg_index_block is not None else None
    a.nthreads = nthreads
    if subswaths is not None:
        ss = SubSw()
        ss.n, ss.length, ss.width = subswaths.num_sub_swaths, subswaths.length, subswaths.width
        packed = keep.arr(subswaths.packed(), np.int32)
        ss.valid = _ptr(packed)
        keep.append(ss)
        a.subswaths = C.pointer(ss)
    st = lib().orc_geocode_rasters(C.byref(a))
    if st != 0:
        raise ValueError(lib().orc_last_error().decode())


def orbit_interpolate(orbit, t):
    keep = _Keep()
    o = orbit_struct(orbit, keep)
    pos, vel = np.zeros(3), np.zeros(3)
    st = lib().orc_orbit_interpolate(C.byref(o), float(t), _ptr(pos), _ptr(vel))
    return pos, vel, st


def interp2d(method: int, z: np.ndarray, x: float, y: float) -> float:
    z = np.ascontiguousarray(z, dtype=np.float64)
    return lib().orc_interp2d_double(method, _ptr(z), z.shape[0], z.shape[1], x, y)


def spline2d_float(z: np.ndarray, x: float, y: float) -> np.float32:
    z = np.ascontiguousarray(z, dtype=np.float32)
    return np.float32(lib().orc_spline2d_float(_ptr(z), z.shape[0], z.shape[1], x, y))


def sinc2d_cfloat(z: np.ndarray, x: float, y: float) -> np.complex64:
    """The SLC interpolator (Sinc2d on complex64) at (x, y) of the table z."""
    z = np.ascontiguousarray(z, dtype=np.complex64)
    out = np.zeros(2, np.float32)
    lib().orc_sinc2d_cfloat(_ptr(z), z.shape[0], z.shape[1], x, y, _ptr(out))
    return np.complex64(out[0] + 1j * out[1])


def lut_eval(lut, y, x) -> float:
    keep = _Keep()
    s = lut_struct(lut, keep)
    return lib().orc_lut2d_eval(C.byref(s), y, x)


def poly_eval(p, y, x) -> float:
    keep = _Keep()
    s = poly_struct(p, keep)
    return lib().orc_poly2d_eval(C.byref(s), y, x)


def proj_inverse(epsg, x, y):
    inp, out = np.array([x, y, 0.0]), np.zeros(3)
    st = lib().orc_proj_inverse(epsg, _ptr(inp), _ptr(out))
    return out[0], out[1], st


def proj_forward(epsg, lon, lat):
    inp, out = np.array([lon, lat, 0.0]), np.zeros(3)
    st = lib().orc_proj_forward(epsg, _ptr(inp), _ptr(out))
    return out[0], out[1], st


def geo2rdr(llh, ellipsoid, orbit, doppler, wavelength, side, t0, threshold=1e-8, maxiter=50, delta_range=10.0):
    keep = _Keep()
    o = orbit_struct(orbit, keep)
    d = lut_struct(doppler, keep)
    llh = np.asarray(llh, dtype=np.float64)
    t, r = np.array([t0], dtype=np.float64), np.zeros(1)
    ok = lib().orc_geo2rdr(_ptr(llh), ellipsoid.a, ellipsoid.e2, C.byref(o), C.byref(d), _ptr(t), _ptr(r),
                           wavelength, int(side), threshold, maxiter, delta_range)
    return t[0], r[0], ok


def radar_bbox(geo_grid, radar_grid, orbit, min_height=-500.0, max_height=9000.0, doppler=None, margin=50,
               threshold=1e-8, maxiter=50, delta_range=10.0, geogrid_expansion_threshold=100):
    """geometry/boundingbox.cpp:434-641 on the CPU: (first_az, last_az,
    first_rg, last_rg, status, detail) as gslc_radar_bbox reports them."""
    keep = _Keep()
    g = geo_struct(geo_grid)
    rg = radar_struct(radar_grid)
    o = orbit_struct(orbit, keep)
    if doppler is None:
        d = Lut()
        d.have_data, d.bounds_error, d.method, d.dx, d.dy = 0, 1, 1, 1.0, 1.0
    else:
        d = lut_struct(doppler, keep)
    out = np.zeros(6, dtype=np.int32)
    st = lib().orc_radar_bbox(C.byref(g), C.byref(rg), C.byref(o), C.byref(d), float(min_height), float(max_height),
                              int(margin), threshold, int(maxiter), delta_range, int(geogrid_expansion_threshold),
                              _ptr(out))
    if st:
        raise ValueError(lib().orc_last_error().decode())
    return tuple(int(v) for v in out)


CUBE_NAMES = [("slant_range", np.float64), ("azimuth_time", np.float64), ("incidence_angle", np.float32),
              ("los_unit_vector_x", np.float32), ("los_unit_vector_y", np.float32),
              ("along_track_unit_vector_x", np.float32), ("along_track_unit_vector_y", np.float32),
              ("elevation_angle", np.float32), ("ground_track_velocity", np.float64)]


def radar_grid_cubes(radar_grid, geogrid, heights, orbit, native_doppler, grid_doppler, threshold=1e-8,
                     maxiter=50, delta_range=10.0, outputs=None, nthreads=0):
    """geometry/metadataCubes.cpp:276-489 on the CPU; returns {name: array of
    (heights, length, width)} for the names in ``outputs`` (default: all)."""
    keep = _Keep()
    rg, g = radar_struct(radar_grid), geo_struct(geogrid)
    o = orbit_struct(orbit, keep)
    nd, gd = lut_struct(native_doppler, keep), lut_struct(grid_doppler, keep)
    h = np.ascontiguousarray(np.asarray(heights, dtype=np.float64).ravel())
    shape = (h.size, geogrid.length, geogrid.width)
    want = [n for n, _ in CUBE_NAMES] if outputs is None else list(outputs)
    arrs = {n: np.empty(shape, dt) for n, dt in CUBE_NAMES if n in want}
    ptrs = [(_ptr(arrs[n]) if n in arrs else None) for n, _ in CUBE_NAMES]
    st = lib().orc_radar_grid_cubes(C.byref(rg), C.byref(g), _ptr(h), h.size, C.byref(o), C.byref(nd), C.byref(gd),
                                    threshold, int(maxiter), delta_range, *ptrs, int(nthreads))
    if st:
        raise RuntimeError(lib().orc_last_error().decode())
    return arrs


_GDT = {np.dtype(np.uint8): 1, np.dtype(np.uint16): 2, np.dtype(np.uint32): 4, np.dtype(np.float32): 6,
        np.dtype(np.float64): 7, np.dtype(np.complex64): 10, np.dtype(np.complex128): 11}


def interpolate_raster(az: np.ndarray, rg: np.ndarray, raster: np.ndarray, method: int, invalid: float) -> np.ndarray:
    """cuda/geocode/Geocode.cu:203-287 on the CPU: ``raster`` sampled at the
    radar coordinates (az, rg) of each output pixel (NaN: masked)."""
    az = np.ascontiguousarray(az, dtype=np.float64)
    rg = np.ascontiguousarray(rg, dtype=np.float64)
    raster = np.ascontiguousarray(raster)
    out = np.empty(az.shape, raster.dtype)
    st = lib().orc_interpolate_raster(_ptr(az), _ptr(rg), az.size, _ptr(raster), raster.shape[0], raster.shape[1],
                                      _ptr(out), _GDT[raster.dtype], int(method), float(invalid))
    if st:
        raise ValueError(lib().orc_last_error().decode())
    return out


def dem_stats(z: np.ndarray):
    """DEMInterpolator::computeMinMaxMeanHeight (DEMInterpolator.cpp:515-560)."""
    z = np.ascontiguousarray(z, dtype=np.float32)
    mn, mx = np.zeros(1, np.float32), np.zeros(1, np.float32)
    mean, n = np.zeros(1, np.float64), np.zeros(1, np.int64)
    lib().orc_dem_stats(_ptr(z), z.shape[0], z.shape[1], _ptr(mn), _ptr(mx), _ptr(mean), _ptr(n))
    return mn[0], mx[0], mean[0], int(n[0])


def sinc_table() -> np.ndarray:
    out = np.zeros((8192, 8), dtype=np.float32)
    lib().orc_sinc_table(_ptr(out))
    return out


def timed_geocode(*args, **kw):
    t0 = time.perf_counter()
    phases = geocode_slc(*args, **kw)
    return time.perf_counter() - t0, phases


def ncores() -> int:
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count() or 1
