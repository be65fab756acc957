"""Batched SLC geocoding: many requests in one persistent, graph-captured launch.

A request is the argument set of one ``geocode_slc`` call (a burst, or a tile
of a larger job) with device-resident arrays.  ``GeocodeBatch`` binds a list
of requests once — launch parameters, orbit polynomials, deramp scratch, the
tile prefix sums — and each ``launch()`` replays one CUDA graph: the carrier
deramp passes followed by a single persistent kernel whose blocks pop runs of
32x8-pixel tiles of any request from a device counter.  Requests of very
different sizes therefore share the GPU without per-request launches, tail
waves or host round trips, and each request's outputs equal its plain call.

The reference geocodes one block per call, driven from the host
(python/packages/nisar/workflows/gslc.py:173-214 over
python/packages/isce3/core/rdr_geo_block_generator.py:7-117); this form has
no counterpart there.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Any

import numpy as np
import torch

from . import _lib as L
from . import _marshal as M
from .geocode import _build_args, _normalize_call


@dataclass
class GeocodeRequest:
    """Arguments of one geocode_slc call (same names), arrays on the GPU."""
    geo_data_blocks: Any
    rdr_data_blocks: Any
    dem_raster: Any
    radargrid: Any
    geogrid: Any
    orbit: Any
    native_doppler: Any
    image_grid_doppler: Any
    ellipsoid: Any
    threshold_geo2rdr: float
    num_iter_geo2rdr: int
    kwargs: dict = field(default_factory=dict)

    def normalized(self, precision: str):
        kw = dict(mask_block=None, sliced_radargrid=None, subswaths=None, first_azimuth_line=0,
                  first_range_sample=0, flatten=True, reramp=True, az_carrier=None, rg_carrier=None,
                  az_time_correction=None, srange_correction=None, flatten_with_corrected_srange=False,
                  invalid_value=complex(float("nan"), float("nan")), carrier_phase_block=None,
                  flatten_phase_block=None, inplace_deramp=False, az_index_block=None, rg_index_block=None,
                  dem_margin=50, rdr_deramped=False, output_nonzero_mantissa_bits=None)
        unknown = set(self.kwargs) - set(kw)
        if unknown:
            raise TypeError(f"unknown geocode_slc arguments {sorted(unknown)}")
        kw.update(self.kwargs)
        return _normalize_call(self.geo_data_blocks, self.rdr_data_blocks, self.dem_raster, self.radargrid,
                               self.geogrid, self.orbit, self.native_doppler, self.image_grid_doppler,
                               self.ellipsoid, self.threshold_geo2rdr, self.num_iter_geo2rdr, kw["mask_block"],
                               kw["sliced_radargrid"], kw["subswaths"], kw["first_azimuth_line"],
                               kw["first_range_sample"], kw["flatten"], kw["reramp"], kw["az_carrier"],
                               kw["rg_carrier"], kw["az_time_correction"], kw["srange_correction"],
                               kw["flatten_with_corrected_srange"], kw["invalid_value"],
                               kw["carrier_phase_block"], kw["flatten_phase_block"], precision,
                               kw["inplace_deramp"], kw["az_index_block"], kw["rg_index_block"], kw["dem_margin"],
                               kw["rdr_deramped"], kw["output_nonzero_mantissa_bits"])


@dataclass
class BatchTuning:
    """Launch shape of the persistent kernel (see isce3_gb300.autotune)."""
    tiles_per_pop: int = 2
    blocks_per_sm: int = 0          # 0: occupancy maximum
    use_graph: bool = True
    rows_per_thread: int = 4        # geogrid lines per thread: tiles of 32 x 8*rows_per_thread pixels
    per_request: bool = False       # each request's own fused kernel on concurrent streams, no queue

    def to_c(self) -> L.BatchTuning:
        t = L.BatchTuning()
        t.tiles_per_pop, t.blocks_per_sm, t.use_graph = self.tiles_per_pop, self.blocks_per_sm, int(self.use_graph)
        t.rows_per_thread = self.rows_per_thread
        t.per_request = int(self.per_request)
        return t


class HostFlags:
    """Words of mapped host memory that a batch's kernel sets to 1 when the
    last tile of a request has been written (``GeocodeBatch(done_flags=...)``).

    ``array`` is a NumPy view over them; the host clears it before a launch
    and polls it while the batch runs."""

    def __init__(self, n: int):
        if n < 1:
            raise ValueError("HostFlags needs at least one word")
        self.lib = L.lib()
        p = C.c_void_p()
        if self.lib.gslc_host_flags_create(int(n), C.byref(p)) != L.GSLC_OK:
            raise RuntimeError("could not allocate mapped host memory for completion flags")
        self.ptr = p.value
        self.n = int(n)
        self.array = np.ctypeslib.as_array((C.c_uint32 * self.n).from_address(self.ptr))

    def clear(self) -> None:
        self.array[:] = 0

    def close(self) -> None:
        if getattr(self, "ptr", None):
            self.array = None
            self.lib.gslc_host_flags_destroy(C.c_void_p(self.ptr))
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GeocodeBatch:
    """A bound batch of geocode requests; ``launch()`` runs them all at once.

    With ``done_flags`` (a ``HostFlags`` of at least ``len(requests)`` words)
    word i turns 1 as soon as request i's outputs are written, while the rest
    of the batch still runs; ``wait()`` still reports the batch's errors."""

    def __init__(self, requests: list[GeocodeRequest], geo2rdr_precision: str = "fp64",
                 tuning: BatchTuning | None = None, device=None, stream: torch.cuda.Stream | None = None,
                 done_flags: HostFlags | None = None):
        self.dev = M.device_of(device)
        self.precision = geo2rdr_precision
        self.tuning = tuning or BatchTuning()
        self.lib = L.lib()
        self.ctx = L.context(self.dev.index)
        self._keep = []
        n = len(requests)
        arr = (L.GeocodeArgs * max(n, 1))()
        with torch.cuda.device(self.dev):
            for i, r in enumerate(requests):
                call = r.normalized(geo2rdr_precision)
                for blk in list(call[0]) + list(call[1]):
                    if not (isinstance(blk, torch.Tensor) and blk.is_cuda):
                        raise ValueError("batched requests need CUDA tensors for their data blocks")
                a, outs, keep = _build_args(self.dev, *call)
                if any(o.host is not None for o in outs):
                    raise ValueError("batched requests need CUDA tensors for their outputs")
                arr[i] = a
                self._keep.append(keep)
            # the batch's buffers are ordered on this stream (staging ran on the current one)
            self.stream = stream or torch.cuda.current_stream(self.dev)
            if self.stream != torch.cuda.current_stream(self.dev):
                self.stream.wait_stream(torch.cuda.current_stream(self.dev))
            h = C.c_void_p()
            tc = self.tuning.to_c()
            prec = 1 if geo2rdr_precision in ("ff", "float-float") else 0
            if done_flags is None:
                st = self.lib.gslc_batch_create(self.ctx, arr, n, prec, C.byref(tc),
                                                C.c_void_p(self.stream.cuda_stream), C.byref(h))
            else:
                if done_flags.n < n:
                    raise ValueError(f"done_flags holds {done_flags.n} words for {n} requests")
                st = self.lib.gslc_batch_create_signaled(self.ctx, arr, n, prec, C.byref(tc),
                                                         C.c_void_p(self.stream.cuda_stream),
                                                         C.c_void_p(done_flags.ptr), C.byref(h))
            L.check(st, self.ctx, "gslc_batch_create")
        self.handle = h
        self._args = arr

    def info(self) -> dict:
        nt, nl = C.c_int64(), C.c_int64()
        bl, tp = C.c_int32(), C.c_int32()
        self.lib.gslc_batch_info(self.handle, C.byref(nt), C.byref(bl), C.byref(tp), C.byref(nl))
        return {"tiles": nt.value, "blocks": bl.value, "tiles_per_pop": tp.value, "launches_per_run": nl.value}

    def launch(self, stream: torch.cuda.Stream | None = None) -> None:
        s = stream or self.stream
        L.check(self.lib.gslc_batch_launch(self.handle, C.c_void_p(s.cuda_stream)), self.ctx, "gslc_batch_launch")

    def wait(self, stream: torch.cuda.Stream | None = None) -> None:
        s = stream or self.stream
        L.check(self.lib.gslc_batch_status(self.handle, C.c_void_p(s.cuda_stream)), self.ctx, "gslc_batch")

    def run(self, stream=None) -> None:
        self.launch(stream)
        self.wait(stream)

    def close(self) -> None:
        if getattr(self, "handle", None):
            self.lib.gslc_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
