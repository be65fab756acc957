"""Drop-in for ``isce3.geocode.geocode_slc`` backed by the sm_103a kernel.

Argument names, defaults, the list/array validation and the error types follow
python/packages/isce3/geocode/geocode_slc.py:11-240 and the pybind binding
python/extensions/pybind_isce3/geocode/GeocodeSlc.cpp:218-334.  The C++ call
it replaces is isce3::geocode::geocodeSlc (array mode,
cxx/isce3/geocode/geocodeSlc.cpp:831-968); here it is gslc_geocode_slc in
libgslc.so.

Arrays may be NumPy (host; copied to the GPU and results copied back, like a
call on host memory) or CUDA ``torch.Tensor`` (device-resident; no copies).
One difference is deliberate: the reference deramps the caller's radar
arrays in place (geocodeSlc.cpp:952-953); this call leaves them unchanged
unless ``inplace_deramp=True`` is given for device tensors.
"""
from __future__ import annotations

import ctypes as C
import logging
from types import SimpleNamespace
from typing import Union

import numpy as np
import torch

from . import _lib as L
from . import _marshal as M
from .core import Ellipsoid, LUT2d, Orbit, Poly2d
from .product import GeoGridParameters, RadarGridParameters, SubSwaths

log = logging.getLogger("isce3_gb300.geocode.geocode_slc")

ArrayLike = Union[np.ndarray, torch.Tensor]

# complex32 as isce3.core.types.complex32 (python/packages/isce3/core/types.py:12):
# pairs of float16; torch.complex32 tensors are the device-side equivalent
COMPLEX32 = np.dtype([("r", np.float16), ("i", np.float16)])


def sample_format(x) -> int | None:
    """0 for complex64, 1 for complex32 (NumPy pairs of float16 or
    torch.complex32), None otherwise."""
    if isinstance(x, torch.Tensor):
        return {torch.complex64: 0, torch.complex32: 1}.get(x.dtype)
    if x.dtype == np.complex64:
        return 0
    if x.dtype == COMPLEX32:
        return 1
    return None


def _raw(x):
    """A NumPy complex32 array as its 32-bit words (torch has no structured
    dtypes); everything else unchanged."""
    if isinstance(x, np.ndarray) and x.dtype == COMPLEX32:
        return x.view(np.int32)
    return x


def _is_array(x) -> bool:
    return isinstance(x, (np.ndarray, torch.Tensor))


def _size(x) -> int:
    return x.numel() if isinstance(x, torch.Tensor) else x.size


def _io_value_check(io):
    """geocode_slc.py:11-58."""
    chk = SimpleNamespace(is_list=False, is_array=False, n_items=0, shapes_consistent=False,
                          dtypes_consistent=False, is_valid=False)
    if isinstance(io, list):
        chk.is_list = True
        if io:
            chk.n_items = len(io)
            if all(_is_array(x) for x in io):
                shapes = [tuple(x.shape) for x in io]
                chk.shapes_consistent = all(s == shapes[0] for s in shapes)
                dtypes = [x.dtype for x in io]
                chk.dtypes_consistent = all(d == dtypes[0] for d in dtypes)
                chk.is_valid = chk.shapes_consistent and chk.dtypes_consistent
    elif _is_array(io):
        chk.is_array = True
        chk.n_items = 1
        chk.shapes_consistent = chk.dtypes_consistent = chk.is_valid = True
    return chk


def _io_valid(geo, rdr):
    """geocode_slc.py:61-92: log then raise ValueError."""
    def contents(x):
        return str(x)[10:-1]

    def err(msg):
        log.error(msg)
        raise ValueError(msg)

    if not rdr.is_valid:
        err(f"radar input is invalid: {contents(rdr)}")
    if not geo.is_valid:
        err(f"geo input is invalid: {contents(geo)}")
    if (geo.is_array and rdr.is_list) or (geo.is_list and rdr.is_array):
        err("geo and radar inputs are not the same type")
    if geo.is_list and rdr.is_list and geo.n_items != rdr.n_items:
        err(f"length of geo input list ({geo.n_items}) and radar input list ({rdr.n_items}) do not match")


def _output_array_valid(output_array, geo_array, which):
    """geocode_slc.py:95-109."""
    if output_array is None:
        return
    size = output_array.numel() if isinstance(output_array, torch.Tensor) else output_array.size
    if size and tuple(output_array.shape) != tuple(geo_array.shape):
        msg = f"{which} output array shape does not match geocoded array shape"
        log.error(msg)
        raise ValueError(msg)


def _check_dtype(x, np_dtype, torch_dtype, what):
    if isinstance(x, torch.Tensor):
        if x.dtype != torch_dtype:
            raise TypeError(f"{what} must be {torch_dtype}, got {x.dtype}")
    elif x.dtype != np_dtype:
        raise TypeError(f"{what} must be {np.dtype(np_dtype).name}, got {x.dtype}")


class _Staged:
    """A caller array as a device tensor, with copy-back for host outputs.

    Host arrays may be NumPy arrays or CPU torch tensors; pinned CPU tensors
    copy by DMA without staging.
    """

    def __init__(self, arr, dev, upload: bool, torch_dtype):
        self.host = None
        if isinstance(arr, torch.Tensor) and arr.device.type == "cuda":
            if not arr.is_contiguous():
                raise ValueError("arrays must be C-contiguous")
            self.dev = arr
            return
        if isinstance(arr, torch.Tensor):
            if not arr.is_contiguous():
                raise ValueError("arrays must be C-contiguous")
            host = arr
        else:
            if not arr.flags.c_contiguous:
                raise ValueError("arrays must be C-contiguous")
            host = torch.from_numpy(arr)
        self.host = host
        if upload:
            self.dev = host.to(dev, non_blocking=host.is_pinned())
        else:
            self.dev = torch.empty(tuple(host.shape), dtype=host.dtype, device=dev)

    def ptr(self) -> int:
        return self.dev.data_ptr()

    def copy_back(self):
        if self.host is not None:
            self.host.copy_(self.dev)


def geocode_slc(geo_data_blocks, rdr_data_blocks, dem_raster, radargrid: RadarGridParameters,
                geogrid: GeoGridParameters, orbit: Orbit, native_doppler: LUT2d, image_grid_doppler: LUT2d,
                ellipsoid: Ellipsoid, threshold_geo2rdr: float, num_iter_geo2rdr: int,
                mask_block=None, sliced_radargrid=None, subswaths: SubSwaths | None = None,
                first_azimuth_line: int = 0, first_range_sample: int = 0, flatten: bool = True,
                reramp: bool = True, az_carrier=None, rg_carrier=None, az_time_correction=None,
                srange_correction=None, flatten_with_corrected_srange: bool = False,
                invalid_value=np.nan + np.nan * 1j,
                carrier_phase_block=None, flatten_phase_block=None, *,
                geo2rdr_precision: str = "fp64", inplace_deramp: bool = False,
                az_index_block=None, rg_index_block=None, dem_margin: int = 50, rdr_deramped: bool = False,
                output_nonzero_mantissa_bits: int | None = None,
                device=None, stream: torch.cuda.Stream | None = None) -> None:
    """Geocode radar SLC arrays sharing one radar grid onto one geogrid.

    Parameters and semantics are those of ``isce3.geocode.geocode_slc``
    (python/packages/isce3/geocode/geocode_slc.py:112-191).  Extra keyword-only
    arguments: ``geo2rdr_precision`` ("fp64" reference numerics, or "ff"
    float-float), ``inplace_deramp`` (mutate device radar tensors like the
    reference), ``az_index_block``/``rg_index_block`` (f64 outputs of the radar
    coordinates per geo pixel), ``dem_margin``, ``rdr_deramped`` (the radar
    blocks already carry the carrier deramp, as resident stores keep them),
    ``output_nonzero_mantissa_bits`` (complex64 outputs keep only this many
    mantissa bits, as isce3.core.types.truncate_mantissa after the call),
    ``device`` and ``stream``.

    Radar blocks may be complex32 (NumPy arrays of isce3's complex32 dtype, or
    torch.complex32 tensors): the kernel decodes them exactly as
    read_c4_dataset_as_c8 would.  Geo blocks of complex32 receive the
    float16 encoding of the result (isce3.core.types.to_complex32).
    """
    call = _normalize_call(geo_data_blocks, rdr_data_blocks, dem_raster, radargrid, geogrid, orbit, native_doppler,
                           image_grid_doppler, ellipsoid, threshold_geo2rdr, num_iter_geo2rdr, mask_block,
                           sliced_radargrid, subswaths, first_azimuth_line, first_range_sample, flatten, reramp,
                           az_carrier, rg_carrier, az_time_correction, srange_correction,
                           flatten_with_corrected_srange, invalid_value, carrier_phase_block, flatten_phase_block,
                           geo2rdr_precision, inplace_deramp, az_index_block, rg_index_block, dem_margin,
                           rdr_deramped, output_nonzero_mantissa_bits)
    dev = M.device_of(device)
    lib = L.lib()
    ctx = L.context(dev.index)
    with torch.cuda.device(dev):
        s = stream if stream is not None else torch.cuda.current_stream(dev)
        with torch.cuda.stream(s):
            _geocode_on_stream(lib, ctx, s, dev, *call)


def geocode_slc_raster(output_raster, input_raster, dem_raster, radargrid: RadarGridParameters,
                       geogrid: GeoGridParameters, orbit: Orbit, native_doppler: LUT2d, image_grid_doppler: LUT2d,
                       ellipsoid: Ellipsoid, threshold_geo2rdr: float = 1.0e-9, numiter_geo2rdr: int = 25,
                       lines_per_block: int = 1000, flatten: bool = True, reramp: bool = True,
                       azimuth_carrier=None, range_carrier=None, az_time_correction=None, srange_correction=None,
                       flatten_with_corrected_srange: bool = False, invalid_value=np.nan + np.nan * 1j,
                       carrier_phase_raster=None, flatten_phase_raster=None, *, geo2rdr_precision: str = "fp64",
                       az_index_block=None, rg_index_block=None, dem_margin: int = 50, device=None,
                       stream: torch.cuda.Stream | None = None) -> None:
    """Raster overload of geocode_slc: geocode every band of ``input_raster``
    (the SLC over the whole radar grid) into the same band of
    ``output_raster`` (the whole geogrid), block by block.

    Names and defaults are those of the pybind overload
    (python/extensions/pybind_isce3/geocode/GeocodeSlc.cpp:26-102) of
    isce3::geocode::geocodeSlc's raster mode (cxx/isce3/geocode/geocodeSlc.cpp:
    605-828): blocks of ``lines_per_block`` geogrid lines, each with the DEM
    window of that block alone; pixels without a result hold
    ``invalid_value``, and the optional float64 phase rasters its real part.
    Rasters are ``isce3_gb300.io.Raster`` objects (GDAL's file I/O has no
    place here); results are written into their samples.  The input raster is
    not modified.  Extra keyword-only arguments as in ``geocode_slc``.
    """
    from .io import Raster
    for r, what in ((output_raster, "output_raster"), (input_raster, "input_raster")):
        if not isinstance(r, Raster):
            raise TypeError(f"{what} must be an isce3_gb300.io.Raster")
    if output_raster.num_bands() != input_raster.num_bands():
        raise ValueError("input and output rasters have different numbers of bands")
    if (input_raster.length, input_raster.width) != (radargrid.length, radargrid.width):
        raise ValueError("input raster shape differs from the radar grid")
    if (output_raster.length, output_raster.width) != (geogrid.length, geogrid.width):
        raise ValueError("output raster shape differs from the geogrid")
    if int(lines_per_block) < 1:
        raise ValueError("lines_per_block must be positive")
    phases = []
    for ph, what in ((carrier_phase_raster, "carrier_phase_raster"), (flatten_phase_raster, "flatten_phase_raster")):
        if ph is None:
            phases.append(None)
            continue
        if not isinstance(ph, Raster) or ph.data.dtype != np.float64 or ph.num_bands() != 1:
            raise TypeError(f"{what} must be a single-band float64 isce3_gb300.io.Raster")
        if (ph.length, ph.width) != (geogrid.length, geogrid.width):
            raise ValueError(f"{what} shape differs from the geogrid")
        phases.append(ph.data)
    azimuth_carrier = Poly2d() if azimuth_carrier is None else azimuth_carrier
    range_carrier = Poly2d() if range_carrier is None else range_carrier
    n = input_raster.num_bands()
    rdr = [input_raster.band(i) for i in range(n)]
    geo = [output_raster.band(i) for i in range(n)]
    call = _normalize_call(geo, rdr, dem_raster, radargrid, geogrid, orbit, native_doppler, image_grid_doppler,
                           ellipsoid, threshold_geo2rdr, numiter_geo2rdr, None, None, None, 0, 0, flatten, reramp,
                           azimuth_carrier, range_carrier, az_time_correction, srange_correction,
                           flatten_with_corrected_srange, invalid_value, phases[0], phases[1], geo2rdr_precision,
                           False, az_index_block, rg_index_block, dem_margin)
    dev = M.device_of(device)
    lib = L.lib()
    ctx = L.context(dev.index)
    with torch.cuda.device(dev):
        s = stream if stream is not None else torch.cuda.current_stream(dev)
        with torch.cuda.stream(s):
            a, outs, keep = _build_args(dev, *call, dem_lines_per_block=int(lines_per_block))
            st = lib.gslc_geocode_slc_raster(ctx, C.byref(a), int(lines_per_block), C.c_void_p(s.cuda_stream))
            L.check(st, ctx, "geocode_slc")
            for o in outs:
                o.copy_back()
            del keep


def _normalize_call(geo_data_blocks, rdr_data_blocks, dem_raster, radargrid, geogrid, orbit, native_doppler,
                    image_grid_doppler, ellipsoid, threshold_geo2rdr, num_iter_geo2rdr, mask_block,
                    sliced_radargrid, subswaths, first_azimuth_line, first_range_sample, flatten, reramp,
                    az_carrier, rg_carrier, az_time_correction, srange_correction, flatten_with_corrected_srange,
                    invalid_value, carrier_phase_block, flatten_phase_block, geo2rdr_precision, inplace_deramp,
                    az_index_block, rg_index_block, dem_margin, rdr_deramped=False,
                    output_nonzero_mantissa_bits=None):
    """Defaults and validation of geocode_slc (geocode_slc.py:192-213); the
    arguments of _build_args in its order."""
    az_carrier = LUT2d() if az_carrier is None else az_carrier
    rg_carrier = LUT2d() if rg_carrier is None else rg_carrier
    az_time_correction = LUT2d() if az_time_correction is None else az_time_correction
    srange_correction = LUT2d() if srange_correction is None else srange_correction
    if carrier_phase_block is None:
        carrier_phase_block = np.array([], dtype=np.float64)
    if flatten_phase_block is None:
        flatten_phase_block = np.array([], dtype=np.float64)

    geo_chk = _io_value_check(geo_data_blocks)
    rdr_chk = _io_value_check(rdr_data_blocks)
    _io_valid(geo_chk, rdr_chk)
    if sliced_radargrid is None:
        sliced_radargrid = radargrid
    if geo_chk.is_array and rdr_chk.is_array:
        geo_data_blocks = [geo_data_blocks]
        rdr_data_blocks = [rdr_data_blocks]
    for arr, which in zip([carrier_phase_block, flatten_phase_block, mask_block],
                          ["carrier", "flattening", "mask"]):
        _output_array_valid(arr, geo_data_blocks[0], which)
    if type(az_carrier) is not type(rg_carrier):
        raise TypeError("az_carrier and rg_carrier must both be LUT2d or both be Poly2d")
    if not isinstance(az_carrier, (LUT2d, Poly2d)):
        raise TypeError("carriers must be LUT2d or Poly2d")
    for g in geo_data_blocks:
        if sample_format(g) is None:
            raise TypeError(f"geo_data_blocks must be complex64 or complex32, got {g.dtype}")
        if tuple(g.shape) != (geogrid.length, geogrid.width):
            raise ValueError("geo_data_blocks shape does not match the geogrid")
    for r in rdr_data_blocks:
        if sample_format(r) is None:
            raise TypeError(f"rdr_data_blocks must be complex64 or complex32, got {r.dtype}")
    rdr_format = sample_format(rdr_data_blocks[0])
    geo_format = sample_format(geo_data_blocks[0])
    if any(sample_format(r) != rdr_format for r in rdr_data_blocks) or \
            any(sample_format(g) != geo_format for g in geo_data_blocks):
        raise TypeError("all radar blocks, and all geo blocks, must share one sample type")
    mantissa_bits = 23
    if output_nonzero_mantissa_bits is not None:
        if geo_format != 0:
            raise ValueError("output_nonzero_mantissa_bits applies to complex64 geo blocks")
        mantissa_bits = int(output_nonzero_mantissa_bits)
        if not 0 < mantissa_bits <= 23:
            raise ValueError(f"Require 0 < significant_bits={mantissa_bits} <= 23")
        if mantissa_bits < 23:
            geo_format = 2
    if rdr_format == 1 and inplace_deramp:
        raise ValueError("inplace_deramp needs complex64 radar blocks")
    if mask_block is not None:
        _check_dtype(mask_block, np.uint8, torch.uint8, "mask_block")
    precision = {"fp64": 0, "ff": 1, "float-float": 1}.get(geo2rdr_precision)
    if precision is None:
        raise ValueError(f"unknown geo2rdr_precision {geo2rdr_precision!r}")

    return (rdr_data_blocks, geo_data_blocks, dem_raster, radargrid, sliced_radargrid, geogrid, orbit,
            native_doppler, image_grid_doppler, ellipsoid, threshold_geo2rdr, num_iter_geo2rdr, mask_block,
            subswaths, first_azimuth_line, first_range_sample, flatten, reramp, az_carrier, rg_carrier,
            az_time_correction, srange_correction, flatten_with_corrected_srange, invalid_value,
            carrier_phase_block, flatten_phase_block, precision, inplace_deramp, az_index_block,
            rg_index_block, dem_margin, rdr_deramped, rdr_format, geo_format, mantissa_bits)


_upload_streams: dict = {}


def _upload_stream(dev: torch.device) -> torch.cuda.Stream:
    """One side stream per device for radar-block uploads."""
    if dev not in _upload_streams:
        _upload_streams[dev] = torch.cuda.Stream(dev)
    return _upload_streams[dev]


def _build_args(dev, rdr_data_blocks, geo_data_blocks, dem_raster, radargrid, sliced_radargrid, geogrid, orbit,
                native_doppler, image_grid_doppler, ellipsoid, threshold_geo2rdr, num_iter_geo2rdr, mask_block,
                subswaths, first_azimuth_line, first_range_sample, flatten, reramp, az_carrier, rg_carrier,
                az_time_correction, srange_correction, flatten_with_corrected_srange, invalid_value,
                carrier_phase_block, flatten_phase_block, precision, inplace_deramp, az_index_block,
                rg_index_block, dem_margin, rdr_deramped=False, rdr_format=0, geo_format=0, mantissa_bits=23,
                *, dem_lines_per_block=0, host_io=None):
    """Stage arrays on ``dev`` and fill a gslc_geocode_args.  With
    ``dem_lines_per_block`` the device DEM samples cover the window of every
    block of that many geogrid lines (the raster mode).  With ``host_io`` (a
    dict) host radar blocks and a DEM window not yet on the device are only
    allocated there, and ``host_io`` receives what gslc_geocode_slc_host_io
    needs to upload them.

    Returns (args, outputs to copy back, objects to keep alive)."""
    # Radar blocks in pinned host memory upload on a side stream while the DEM
    # window and LUT samples (pageable host memory, synchronous copies) are
    # prepared on the call's stream, which then waits for the upload.
    # Pageable radar blocks upload after them, so that the small synchronous
    # copies do not queue behind the large one.
    s = torch.cuda.current_stream(dev)
    raws = [_raw(r) for r in rdr_data_blocks]
    side = None
    if host_io is not None:
        rdr = [_Staged(r, dev, False, torch.complex64) for r in raws]
    elif any(isinstance(r, torch.Tensor) and r.device.type == "cpu" and r.is_pinned() for r in raws):
        side = _upload_stream(dev)
        side.wait_stream(s)
        with torch.cuda.stream(side):
            rdr = [_Staged(r, dev, True, torch.complex64) for r in raws]
        for st in rdr:
            if st.host is not None:
                st.dev.record_stream(s)
    holder = M.AzRgHolder()
    a = L.GeocodeArgs()
    if dem_lines_per_block > 0:
        a.dem, dem_keep = M.dem_raster_desc_blocks(dem_raster, geogrid, dem_lines_per_block, dem_margin, dev,
                                                   whole_window=True)
    elif host_io is not None:
        a.dem, dem_keep, host_io["dem"], host_io["dem_stride"], host_io["dem_commit"] = \
            M.dem_raster_desc_deferred(dem_raster, geogrid, dem_margin, dev)
    else:
        a.dem, dem_keep = M.dem_raster_desc(dem_raster, geogrid, dem_margin, dev)
    a.native_doppler = M.lut_desc(native_doppler, dev)
    a.image_grid_doppler = M.lut_desc(image_grid_doppler, dev)
    a.az_time_correction = M.lut_desc(az_time_correction, dev)
    a.srange_correction = M.lut_desc(srange_correction, dev)
    a.az_carrier = M.azrg_desc(az_carrier, dev, holder)
    a.rg_carrier = M.azrg_desc(rg_carrier, dev, holder)
    if host_io is not None:
        pass
    elif side is None:
        rdr = [_Staged(r, dev, True, torch.complex64) for r in raws]
    else:
        s.wait_stream(side)
    if any(r.host is not None for r in rdr) and inplace_deramp:
        raise ValueError("inplace_deramp needs device-resident radar tensors")
    geo_t = torch.complex64 if geo_format != 1 else torch.int32
    geo = [_Staged(_raw(g), dev, False, geo_t) for g in geo_data_blocks]
    outs = list(geo)

    def opt_out(arr, np_dtype, t_dtype, what, upload):
        if arr is None or _size(arr) == 0:
            return None
        _check_dtype(arr, np_dtype, t_dtype, what)
        st = _Staged(arr, dev, upload, t_dtype)
        outs.append(st)
        return st

    # the mask and radar coordinates are written at every pixel; the phase
    # outputs only at valid ones, so those keep the caller's other values
    mask = opt_out(mask_block, np.uint8, torch.uint8, "mask_block", False)
    carrier = opt_out(carrier_phase_block, np.float64, torch.float64, "carrier_phase_block", True)
    flat = opt_out(flatten_phase_block, np.float64, torch.float64, "flatten_phase_block", True)
    azi = opt_out(az_index_block, np.float64, torch.float64, "az_index_block", False)
    rgi = opt_out(rg_index_block, np.float64, torch.float64, "rg_index_block", False)

    a.radar_grid = M.radar_grid_desc(radargrid)
    a.sliced_radar_grid = M.radar_grid_desc(sliced_radargrid)
    a.geo_grid = M.geo_grid_desc(geogrid)
    a.orbit = M.orbit_desc(orbit)
    a.ellipsoid_a, a.ellipsoid_e2 = ellipsoid.a, ellipsoid.e2
    a.threshold_geo2rdr = float(threshold_geo2rdr)
    a.numiter_geo2rdr = int(num_iter_geo2rdr)
    a.flatten, a.reramp = int(bool(flatten)), int(bool(reramp))
    a.flatten_with_corrected_srange = int(bool(flatten_with_corrected_srange))
    a.first_azimuth_line, a.first_range_sample = int(first_azimuth_line), int(first_range_sample)
    inv = complex(invalid_value)
    a.invalid_re, a.invalid_im = np.float32(inv.real), np.float32(inv.imag)
    a.n_blocks = len(rdr)
    a.inplace_deramp = int(bool(inplace_deramp))
    a.rdr_deramped = int(bool(rdr_deramped))
    a.rdr_length, a.rdr_width = rdr[0].dev.shape
    rdr_ptrs = (C.c_void_p * len(rdr))(*[r.ptr() for r in rdr])
    geo_ptrs = (C.c_void_p * len(geo))(*[g.ptr() for g in geo])
    a.rdr_blocks = C.cast(rdr_ptrs, C.POINTER(C.c_void_p))
    a.geo_blocks = C.cast(geo_ptrs, C.POINTER(C.c_void_p))
    a.mask = mask.ptr() if mask else None
    a.carrier_phase = carrier.ptr() if carrier else None
    a.flatten_phase = flat.ptr() if flat else None
    a.az_index = azi.ptr() if azi else None
    a.rg_index = rgi.ptr() if rgi else None
    a.dem_margin = int(dem_margin)
    a.geo2rdr_precision = precision
    a.rdr_format, a.geo_format, a.mantissa_bits = int(rdr_format), int(geo_format), int(mantissa_bits)
    ss = None
    if subswaths is not None:
        ss = M.subswaths_desc(subswaths, dev)
        a.subswaths = C.pointer(ss)
    keep = [holder, rdr, geo, rdr_ptrs, geo_ptrs, dem_keep, ss]
    return a, outs, keep


# geogrid row bands of the pipelined host-input call, and the radar lines and
# DEM rows planned around each band beyond its perimeter's footprint
HOST_IO_BANDS = 6
HOST_IO_MARGIN = 16


def _host_inputs(call) -> bool:
    """Radar blocks all in host memory, deramped on copies (not in place)."""
    rdr, inplace = call[0], call[27]
    return not inplace and all(not (isinstance(r, torch.Tensor) and r.device.type == "cuda") for r in rdr)


def _geocode_on_stream(lib, ctx, s, dev, *args):
    if _host_inputs(args):
        return _geocode_host_inputs(lib, ctx, s, dev, *args)
    a, outs, keep = _build_args(dev, *args)
    geo = keep[2]
    if all(g.host is not None for g in geo):
        # host geo blocks (and mask): the library copies them back band by
        # band while later bands compute
        mask = next((o for o in outs if a.mask and o.ptr() == a.mask and o.host is not None), None)
        host_ptrs = (C.c_void_p * len(geo))(*[g.host.data_ptr() for g in geo])
        st = lib.gslc_geocode_slc_to_host(ctx, C.byref(a), host_ptrs,
                                          C.c_void_p(mask.host.data_ptr() if mask else None),
                                          C.c_void_p(s.cuda_stream))
        L.check(st, ctx, "geocode_slc")
        done = set(map(id, geo)) | ({id(mask)} if mask else set())
        for o in outs:
            if id(o) not in done:
                o.copy_back()
    else:
        st = lib.gslc_geocode_slc(ctx, C.byref(a), C.c_void_p(s.cuda_stream))
        L.check(st, ctx, "geocode_slc")
        for o in outs:
            o.copy_back()
    del keep


def _geocode_host_inputs(lib, ctx, s, dev, *args):
    """Host radar blocks: gslc_geocode_slc_host_io uploads them (and a DEM
    window not yet on the device) band by band while earlier bands compute,
    and copies host geo blocks and mask back behind each band."""
    hio = {}
    a, outs, keep = _build_args(dev, *args, host_io=hio)
    rdr, geo = keep[1], keep[2]
    io = L.HostIo()
    rp = (C.c_void_p * len(rdr))(*[r.host.data_ptr() for r in rdr])
    io.rdr_blocks = C.cast(rp, C.POINTER(C.c_void_p))
    io.dem = hio.get("dem")
    io.dem_stride = int(hio.get("dem_stride") or 0)
    host_geo = all(g.host is not None for g in geo)
    mask = next((o for o in outs if a.mask and o.ptr() == a.mask and o.host is not None), None)
    gp = None
    if host_geo:
        gp = (C.c_void_p * len(geo))(*[g.host.data_ptr() for g in geo])
        io.geo_blocks = C.cast(gp, C.POINTER(C.c_void_p))
        io.mask = mask.host.data_ptr() if mask else None
    io.bands = HOST_IO_BANDS
    io.margin = HOST_IO_MARGIN
    st = lib.gslc_geocode_slc_host_io(ctx, C.byref(a), C.byref(io), C.c_void_p(s.cuda_stream))
    L.check(st, ctx, "geocode_slc")
    hio["dem_commit"]()
    done = (set(map(id, geo)) | ({id(mask)} if mask else set())) if host_geo else set()
    for o in outs:
        if id(o) not in done:
            o.copy_back()
    del keep, rp, gp
