"""Loader and ctypes mirror of the C ABI in include/gslc.h (libgslc.so).

The library is built in-tree by :func:`build` (nvcc, sm_103a only).  There is
no CPU fallback: :func:`lib` raises if the shared library is missing or a GPU
is not available, so a caller can never silently get another code path.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIBPATH = BUILD / "libgslc.so"
HEADER = ROOT / "include" / "gslc.h"
SOURCES = ["gslc_kernels.cu", "gslc_persistent.cu", "gslc_capi.cu", "gslc_plan.cu", "gslc_raster.cu"]

NVCC_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-std=c++17",
              "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", str(ROOT / "include")]

GSLC_OK, GSLC_EINVAL, GSLC_EUNSUPPORTED, GSLC_EPROJ = 0, 1, 2, 3
GSLC_ECUDA, GSLC_ETIMEOUT = -1, -2


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile libgslc.so for sm_103a (translation units in parallel)."""
    BUILD.mkdir(exist_ok=True)
    srcs = [CSRC / s for s in SOURCES if (CSRC / s).exists()]
    deps = srcs + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.cu")) + [HEADER]
    if not force and LIBPATH.exists():
        newest = max(p.stat().st_mtime for p in deps)
        if LIBPATH.stat().st_mtime >= newest:
            return LIBPATH
    nvcc = _nvcc()
    objs, procs = [], []
    for s in srcs:
        o = BUILD / (s.stem + ".o")
        objs.append(o)
        cmd = [nvcc, *NVCC_FLAGS, "-c", str(s), "-o", str(o)]
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{out}")
        if verbose and out:
            print(out)
    tmp = LIBPATH.with_suffix(".so.tmp")
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-shared", "-o", str(tmp), *map(str, objs)]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc link failed: {' '.join(cmd)}\n{r.stdout}")
    os.replace(tmp, LIBPATH)
    return LIBPATH


# ---------------------------------------------------------------- structs
class Lut2d(C.Structure):
    _fields_ = [("have_data", C.c_int32), ("bounds_error", C.c_int32), ("method", C.c_int32),
                ("nx", C.c_int32), ("ny", C.c_int32), ("_pad", C.c_int32),
                ("x0", C.c_double), ("y0", C.c_double), ("dx", C.c_double), ("dy", C.c_double),
                ("ref_value", C.c_double), ("data", C.c_void_p)]


class Poly2d(C.Structure):
    _fields_ = [("x_order", C.c_int32), ("y_order", C.c_int32), ("x_mean", C.c_double), ("y_mean", C.c_double),
                ("x_norm", C.c_double), ("y_norm", C.c_double), ("coeffs", C.POINTER(C.c_double))]


class AzRgFunc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("_pad", C.c_int32), ("lut", Lut2d), ("poly", Poly2d)]


class RadarGrid(C.Structure):
    _fields_ = [("sensing_start", C.c_double), ("wavelength", C.c_double), ("prf", C.c_double),
                ("starting_range", C.c_double), ("range_pixel_spacing", C.c_double),
                ("look_side", C.c_int32), ("_pad", C.c_int32), ("length", C.c_int64), ("width", C.c_int64)]


class GeoGrid(C.Structure):
    _fields_ = [("start_x", C.c_double), ("start_y", C.c_double), ("spacing_x", C.c_double),
                ("spacing_y", C.c_double), ("width", C.c_int32), ("length", C.c_int32), ("epsg", C.c_int32),
                ("_pad", C.c_int32)]


class OrbitDesc(C.Structure):
    _fields_ = [("t0", C.c_double), ("spacing", C.c_double), ("n", C.c_int32), ("method", C.c_int32),
                ("pos", C.POINTER(C.c_double)), ("vel", C.POINTER(C.c_double))]


class DemRaster(C.Structure):
    _fields_ = [("width", C.c_int64), ("length", C.c_int64), ("gt", C.c_double * 6), ("epsg", C.c_int32),
                ("_pad", C.c_int32), ("data", C.c_void_p), ("data_x_off", C.c_int64), ("data_y_off", C.c_int64),
                ("data_width", C.c_int64), ("data_length", C.c_int64), ("data_stride", C.c_int64)]


class DemWindow(C.Structure):
    _fields_ = [("have_raster", C.c_int32), ("wraps", C.c_int32), ("x_off", C.c_int64), ("y_off", C.c_int64),
                ("width", C.c_int64), ("length", C.c_int64), ("x_start", C.c_double), ("y_start", C.c_double),
                ("dx", C.c_double), ("dy", C.c_double)]


class SubSwathsDesc(C.Structure):
    _fields_ = [("n", C.c_int32), ("_pad", C.c_int32), ("length", C.c_int64), ("width", C.c_int64),
                ("valid", C.c_void_p)]


class GeocodeArgs(C.Structure):
    _fields_ = [("radar_grid", RadarGrid), ("sliced_radar_grid", RadarGrid), ("geo_grid", GeoGrid),
                ("orbit", OrbitDesc), ("native_doppler", Lut2d), ("image_grid_doppler", Lut2d),
                ("az_time_correction", Lut2d), ("srange_correction", Lut2d),
                ("az_carrier", AzRgFunc), ("rg_carrier", AzRgFunc),
                ("ellipsoid_a", C.c_double), ("ellipsoid_e2", C.c_double), ("threshold_geo2rdr", C.c_double),
                ("numiter_geo2rdr", C.c_int32), ("flatten", C.c_int32), ("reramp", C.c_int32),
                ("flatten_with_corrected_srange", C.c_int32),
                ("first_azimuth_line", C.c_int64), ("first_range_sample", C.c_int64),
                ("invalid_re", C.c_float), ("invalid_im", C.c_float), ("n_blocks", C.c_int32),
                ("inplace_deramp", C.c_int32), ("rdr_length", C.c_int64), ("rdr_width", C.c_int64),
                ("rdr_blocks", C.POINTER(C.c_void_p)), ("geo_blocks", C.POINTER(C.c_void_p)),
                ("mask", C.c_void_p), ("carrier_phase", C.c_void_p), ("flatten_phase", C.c_void_p),
                ("az_index", C.c_void_p), ("rg_index", C.c_void_p), ("dem", DemRaster),
                ("dem_margin", C.c_int32), ("geo2rdr_precision", C.c_int32),
                ("subswaths", C.POINTER(SubSwathsDesc)), ("rdr_deramped", C.c_int32), ("_pad2", C.c_int32),
                ("rdr_format", C.c_int32), ("geo_format", C.c_int32), ("mantissa_bits", C.c_int32),
                ("_pad3", C.c_int32)]


class RasterGeocodeArgs(C.Structure):
    _fields_ = [("radar_grid", RadarGrid), ("geo_grid", GeoGrid), ("orbit", OrbitDesc), ("doppler", Lut2d),
                ("native_doppler", Lut2d), ("az_time_correction", Lut2d), ("srange_correction", Lut2d),
                ("dem", DemRaster), ("subswaths", C.POINTER(SubSwathsDesc)),
                ("ellipsoid_a", C.c_double), ("ellipsoid_e2", C.c_double), ("threshold", C.c_double),
                ("delta_range", C.c_double), ("maxiter", C.c_int32), ("lines_per_block", C.c_int32),
                ("n_rasters", C.c_int32), ("geo2rdr_precision", C.c_int32),
                ("input_rasters", C.POINTER(C.c_void_p)), ("output_rasters", C.POINTER(C.c_void_p)),
                ("invalid_values", C.POINTER(C.c_double)), ("az_index", C.c_void_p), ("rg_index", C.c_void_p),
                ("dem_margin", C.c_int32), ("_pad", C.c_int32)]


class HostIo(C.Structure):
    _fields_ = [("rdr_blocks", C.POINTER(C.c_void_p)), ("dem", C.c_void_p), ("dem_stride", C.c_int64),
                ("geo_blocks", C.POINTER(C.c_void_p)), ("mask", C.c_void_p), ("bands", C.c_int32),
                ("margin", C.c_int32)]


class BatchTuning(C.Structure):
    _fields_ = [("tiles_per_pop", C.c_int32), ("blocks_per_sm", C.c_int32), ("use_graph", C.c_int32),
                ("rows_per_thread", C.c_int32), ("per_request", C.c_int32)]


class GeoBlock(C.Structure):
    _fields_ = [("start_x", C.c_double), ("start_y", C.c_double), ("spacing_x", C.c_double),
                ("spacing_y", C.c_double), ("width", C.c_int32), ("length", C.c_int32)]


class RadarBBox(C.Structure):
    _fields_ = [("first_azimuth_line", C.c_int32), ("last_azimuth_line", C.c_int32),
                ("first_range_sample", C.c_int32), ("last_range_sample", C.c_int32),
                ("status", C.c_int32), ("detail", C.c_int32)]


class BBoxArgs(C.Structure):
    _fields_ = [("radar_grid", RadarGrid), ("orbit", OrbitDesc), ("doppler", Lut2d), ("epsg", C.c_int32),
                ("n_blocks", C.c_int32), ("blocks", C.c_void_p), ("min_height", C.c_float),
                ("max_height", C.c_float), ("margin", C.c_int32), ("geogrid_expansion_threshold", C.c_int32),
                ("threshold", C.c_double), ("maxiter", C.c_int32), ("_pad", C.c_int32),
                ("delta_range", C.c_double)]


class CubeArgs(C.Structure):
    _fields_ = [("radar_grid", RadarGrid), ("geo_grid", GeoGrid), ("heights", C.c_void_p), ("n_heights", C.c_int32),
                ("maxiter", C.c_int32), ("orbit", OrbitDesc), ("native_doppler", Lut2d), ("grid_doppler", Lut2d),
                ("threshold", C.c_double), ("delta_range", C.c_double), ("slant_range", C.c_void_p),
                ("azimuth_time", C.c_void_p), ("incidence_angle", C.c_void_p), ("los_unit_vector_x", C.c_void_p),
                ("los_unit_vector_y", C.c_void_p), ("along_track_unit_vector_x", C.c_void_p),
                ("along_track_unit_vector_y", C.c_void_p), ("elevation_angle", C.c_void_p),
                ("ground_track_velocity", C.c_void_p)]


_EXPORTS = {
    "gslc_ctx_create": (C.c_int, [C.c_int, C.POINTER(C.c_void_p)]),
    "gslc_ctx_destroy": (C.c_int, [C.c_void_p]),
    "gslc_last_error": (C.c_char_p, [C.c_void_p]),
    "gslc_version": (C.c_char_p, []),
    "gslc_compute_dem_window": (C.c_int, [C.POINTER(DemRaster), C.POINTER(GeoGrid), C.c_int32,
                                          C.POINTER(DemWindow)]),
    "gslc_compute_dem_window_block": (C.c_int, [C.POINTER(DemRaster), C.POINTER(GeoGrid), C.c_int32, C.c_int32,
                                                C.c_int32, C.c_int32, C.POINTER(DemWindow)]),
    "gslc_geocode_slc": (C.c_int, [C.c_void_p, C.POINTER(GeocodeArgs), C.c_void_p]),
    "gslc_geocode_slc_to_host": (C.c_int, [C.c_void_p, C.POINTER(GeocodeArgs), C.POINTER(C.c_void_p),
                                           C.c_void_p, C.c_void_p]),
    "gslc_geocode_rasters": (C.c_int, [C.c_void_p, C.POINTER(RasterGeocodeArgs), C.c_void_p]),
    "gslc_last_launch_count": (C.c_int64, [C.c_void_p]),
    "gslc_orbit_interpolate": (C.c_int, [C.POINTER(OrbitDesc), C.c_double, C.POINTER(C.c_double),
                                         C.POINTER(C.c_double)]),
    "gslc_geo2rdr_zero_doppler": (C.c_int, [C.POINTER(OrbitDesc), C.c_void_p, C.c_double, C.c_int32, C.c_double,
                                            C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                            C.POINTER(C.c_int32)]),
    "gslc_complex64_to_complex32": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]),
    "gslc_complex32_to_complex64": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]),
    "gslc_truncate_mantissa": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_void_p]),
    "gslc_sinc_table": (C.c_int, [C.c_void_p]),
    "gslc_ctx_set_timing": (C.c_int, [C.c_void_p, C.c_int32]),
    "gslc_ctx_set_stage_wait": (C.c_int, [C.c_void_p, C.c_int64]),
    "gslc_geocode_slc_raster": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p]),
    "gslc_geocode_slc_host_io": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "gslc_last_io_reruns": (C.c_int, [C.c_void_p]),
    "gslc_last_kernel_ms": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "gslc_probe_fp64_gflops": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "gslc_geocode_slc_noalloc": (C.c_int, [C.POINTER(GeocodeArgs), C.c_void_p, C.c_char_p, C.c_size_t]),
    "gslc_batch_create": (C.c_int, [C.c_void_p, C.POINTER(GeocodeArgs), C.c_int32, C.c_int32,
                                    C.POINTER(BatchTuning), C.c_void_p, C.POINTER(C.c_void_p)]),
    "gslc_batch_create_signaled": (C.c_int, [C.c_void_p, C.POINTER(GeocodeArgs), C.c_int32, C.c_int32,
                                             C.POINTER(BatchTuning), C.c_void_p, C.c_void_p,
                                             C.POINTER(C.c_void_p)]),
    "gslc_host_flags_create": (C.c_int, [C.c_int32, C.POINTER(C.c_void_p)]),
    "gslc_host_flags_destroy": (C.c_int, [C.c_void_p]),
    "gslc_batch_launch": (C.c_int, [C.c_void_p, C.c_void_p]),
    "gslc_batch_status": (C.c_int, [C.c_void_p, C.c_void_p]),
    "gslc_batch_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                  C.POINTER(C.c_int64)]),
    "gslc_batch_destroy": (C.c_int, [C.c_void_p]),
    "gslc_radar_bbox_blocks": (C.c_int, [C.c_void_p, C.POINTER(BBoxArgs), C.c_void_p, C.c_void_p]),
    "gslc_make_radar_grid_cubes": (C.c_int, [C.c_void_p, C.POINTER(CubeArgs), C.c_void_p]),
    "gslc_last_cube_passes": (C.c_int, [C.c_void_p]),
    "gslc_interpolate_raster": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64,
                                          C.c_int64, C.c_void_p, C.c_int32, C.c_int32, C.c_double, C.c_void_p]),
    "gslc_dem_stats": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.POINTER(C.c_float),
                                 C.POINTER(C.c_float), C.POINTER(C.c_double), C.POINTER(C.c_int64), C.c_void_p]),
    "gslc_deramp_block": (C.c_int, [C.c_void_p, C.POINTER(RadarGrid), C.POINTER(AzRgFunc), C.POINTER(AzRgFunc),
                                    C.c_int64, C.c_int64, C.c_void_p, C.c_void_p, C.c_int64, C.c_int64,
                                    C.c_void_p]),
}

_lock = threading.Lock()
_lib = None


def declared_symbols() -> list[str]:
    """Function names declared in include/gslc.h."""
    import re
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:int|int64_t|const char\*)\s+(gslc_\w+)\s*\(", text, re.M)))


def load(path: Path | None = None) -> C.CDLL:
    """Load libgslc.so (building it if absent) and declare its signatures.

    Loading needs no GPU; calling the geocoder does.
    """
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = Path(path) if path else LIBPATH
        if not p.exists():
            build()
        lib = C.CDLL(str(p))
        for name, (res, args) in _EXPORTS.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
        return lib


def lib() -> C.CDLL:
    return load()


class GslcError(RuntimeError):
    """A CUDA error (GSLC_ECUDA) or a device-side wait that ran out
    (GSLC_ETIMEOUT); ``status`` holds the C-ABI code."""

    def __init__(self, msg: str, status: int = GSLC_ECUDA):
        super().__init__(msg)
        self.status = status


def check(status: int, ctx=None, what: str = "gslc") -> None:
    """Map a C-ABI status to the exception the reference raises."""
    if status == GSLC_OK:
        return
    msg = lib().gslc_last_error(ctx).decode() if ctx else ""
    msg = f"{what}: {msg}" if msg else f"{what}: status {status}"
    if status in (GSLC_EINVAL, GSLC_EPROJ):
        raise ValueError(msg)
    if status == GSLC_EUNSUPPORTED:
        raise NotImplementedError(msg)
    raise GslcError(msg, status)


_ctx_local = threading.local()


def set_stage_wait(clocks: int, device: int = 0) -> None:
    """SM clocks each thread waits for the orbit tables' copy into shared
    memory (gslc_ctx_set_stage_wait) on this thread's context of ``device``;
    0 restores the default (2^31)."""
    ctx = context(device)
    check(lib().gslc_ctx_set_stage_wait(ctx, int(clocks)), ctx, "gslc_ctx_set_stage_wait")


def context(device: int = 0) -> C.c_void_p:
    """One C context per (host thread, device), created on first use."""
    ctxs = getattr(_ctx_local, "ctxs", None)
    if ctxs is None:
        ctxs = _ctx_local.ctxs = {}
    if device not in ctxs:
        h = C.c_void_p()
        st = lib().gslc_ctx_create(device, C.byref(h))
        if st != GSLC_OK:
            raise GslcError(f"gslc_ctx_create(device={device}) failed with status {st}")
        ctxs[device] = h
    return ctxs[device]
