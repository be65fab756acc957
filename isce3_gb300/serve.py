"""Serving loop: continuous batching of geocode requests over resident data.

- ``ResidentStore`` keeps SLCs (deramped once, with their orbit, Doppler LUTs
  and carriers) and one shared DEM resident in HBM.
- ``AdmissionPolicy`` admits queued requests first-in first-out while their
  HBM footprint (outputs + batch metadata) fits what the budget leaves after
  the resident store and the requests in flight, and a batch slot is free; a
  request larger than the budget less the resident store is rejected.
- ``GeocodeServer.serve`` runs an arrival trace: each scheduling tick it
  moves arrived requests into the queue, marks finished requests, retires
  finished batches (CUDA event polling, no device synchronisation), and
  launches the newly admitted requests as ONE batch on a free stream.  By
  default a batch of two or more requests runs each request's own fused
  kernel on the batch's branch streams (``BatchTuning(per_request=True)``:
  on the 200-request trace at saturation 1899M px/s FP64 and 2216M
  float-float, against 1839M and 2080M for the persistent queue) and a
  single request runs on the persistent queue (p50 latency at 200 req/s
  2.09 ms against 2.32 ms for its own kernel); a ``tuning`` given to the
  server applies to every batch.  Requests that arrive while earlier batches run join the next
  batch as soon as a slot and memory free up, and batches on different
  streams overlap on the device (the next batch's blocks start on the SMs
  that the running batch's blocks leave at its tail).
- Per-request completion: a request's word in mapped host memory
  (``HostFlags``) is set as soon as its own kernel has written it (in the
  persistent queue: by the block that writes its last tile), not when its
  whole batch is.
- ``serve_plain`` runs the same trace one synchronous ``geocode_slc`` call
  per request, first-in first-out: the baseline.

Latency is completion minus arrival on the host clock; p50/p99 and px/s over
the trace are reported.  Results do not depend on co-scheduling: each
request's outputs equal its plain call (no cross-request state).
"""
from __future__ import annotations

import collections
import ctypes as C
import time
from dataclasses import dataclass, field
from typing import Any

import numpy as np
import torch

from . import _lib as L
from . import _marshal as M
from .batch import BatchTuning, GeocodeBatch, GeocodeRequest, HostFlags
from .core import LUT2d, Poly2d
from .geocode import geocode_slc

# bytes per output pixel held while a request is in flight: complex64 + mask
BYTES_PER_PX = 9
REQUEST_OVERHEAD = 64 * 1024          # launch parameters, orbit polynomials, tile table share


@dataclass
class ResidentSlc:
    slc: torch.Tensor                 # deramped once at load
    radar_grid: Any
    orbit: Any
    native_doppler: Any
    image_grid_doppler: Any
    az_carrier: Any
    rg_carrier: Any
    nbytes: int


class ResidentStore:
    """SLCs and a DEM kept in HBM for the lifetime of the server."""

    def __init__(self, dem, device=None):
        self.dev = M.device_of(device)
        self.dem = dem.to_device(self.dev)
        self.slcs: dict[Any, ResidentSlc] = {}
        self.nbytes = dem.data.nbytes

    def add(self, key, slc, radar_grid, orbit, native_doppler=None, image_grid_doppler=None, az_carrier=None,
            rg_carrier=None, copy: bool = True) -> ResidentSlc:
        """Make ``slc`` resident and deramp it once.  With ``copy=False`` a
        device tensor is taken over (deramped in place)."""
        native_doppler = native_doppler if native_doppler is not None else LUT2d()
        image_grid_doppler = image_grid_doppler if image_grid_doppler is not None else LUT2d()
        az_carrier = az_carrier if az_carrier is not None else Poly2d()
        rg_carrier = rg_carrier if rg_carrier is not None else Poly2d()
        t = slc if isinstance(slc, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(slc))
        t = t.to(self.dev, copy=copy).contiguous()
        # deramp once (geocodeSlc.cpp:240-274); requests then pass rdr_deramped
        holder = M.AzRgHolder()
        az_d, rg_d = M.azrg_desc(az_carrier, self.dev, holder), M.azrg_desc(rg_carrier, self.dev, holder)
        g = M.radar_grid_desc(radar_grid)
        ctx = L.context(self.dev.index)
        s = torch.cuda.current_stream(self.dev)
        st = L.lib().gslc_deramp_block(ctx, C.byref(g), C.byref(az_d), C.byref(rg_d), 0, 0, t.data_ptr(),
                                       t.data_ptr(), t.shape[0], t.shape[1], C.c_void_p(s.cuda_stream))
        L.check(st, ctx, "gslc_deramp_block")
        r = ResidentSlc(t, radar_grid, orbit, native_doppler, image_grid_doppler, az_carrier, rg_carrier,
                        t.numel() * 8)
        self.slcs[key] = r
        self.nbytes += r.nbytes
        return r

    def evict(self, key) -> None:
        r = self.slcs.pop(key)
        self.nbytes -= r.nbytes


@dataclass
class ServeRequest:
    """One geocode request against a resident SLC.  ``threshold_geo2rdr`` and
    ``num_iter_geo2rdr`` are the request's geo2rdr convergence arguments
    (geocode_slc's of the same names); ``kwargs`` adds other geocode_slc
    keyword arguments (outputs such as ``az_index_block`` included)."""
    slc_key: Any
    geogrid: Any
    arrival: float = 0.0              # seconds from the start of the trace
    kwargs: dict = field(default_factory=dict)
    threshold_geo2rdr: float = 1e-8
    num_iter_geo2rdr: int = 25
    # filled in by the server
    geo: torch.Tensor | None = None
    mask: torch.Tensor | None = None
    t_admit: float | None = None
    t_done: float | None = None
    error: str | None = None

    @property
    def npx(self) -> int:
        return self.geogrid.length * self.geogrid.width

    @property
    def footprint(self) -> int:
        return self.npx * BYTES_PER_PX + REQUEST_OVERHEAD

    @property
    def latency(self) -> float | None:
        return None if self.t_done is None else self.t_done - self.arrival


class AdmissionPolicy:
    """First-in first-out admission by HBM footprint and batch slots."""

    def __init__(self, budget_bytes: int, max_in_flight: int = 4, max_batch: int = 64):
        if budget_bytes <= 0 or max_in_flight < 1 or max_batch < 1:
            raise ValueError("invalid admission limits")
        self.budget = int(budget_bytes)
        self.max_in_flight = max_in_flight
        self.max_batch = max_batch

    def select(self, pending: collections.deque, used_bytes: int, in_flight: int, resident_bytes: int = 0):
        """Pop and return (admitted, rejected) requests from the head of
        ``pending``.  ``resident_bytes`` (the resident store) and
        ``used_bytes`` (requests in flight) are held against the budget."""
        admitted, rejected = [], []
        if in_flight >= self.max_in_flight:
            return admitted, rejected
        free = self.budget - resident_bytes - used_bytes
        while pending and len(admitted) < self.max_batch:
            r = pending[0]
            if r.footprint > self.budget - resident_bytes:
                pending.popleft()
                r.error = "request larger than the HBM budget left by the resident store"
                rejected.append(r)
                continue
            if r.footprint > free:
                break                     # keep order: wait for memory to free up
            pending.popleft()
            free -= r.footprint
            admitted.append(r)
        return admitted, rejected


class _InFlight:
    def __init__(self, batch, requests, event, slot, nbytes):
        self.batch, self.requests, self.event, self.slot, self.nbytes = batch, requests, event, slot, nbytes
        self.open = list(range(len(requests)))     # requests not yet seen complete


class _Slot:
    """A stream and, with per-request completion, its batch's flag words."""

    def __init__(self, dev, max_batch: int, signaled: bool):
        self.stream = torch.cuda.Stream(dev)
        self.flags = HostFlags(max_batch) if signaled else None


class GeocodeServer:
    """Continuous-batching geocode server over a ``ResidentStore``."""

    def __init__(self, store: ResidentStore, budget_bytes: int = 150 * 10 ** 9, max_in_flight: int = 3,
                 max_batch: int = 64, geo2rdr_precision: str = "fp64", tuning: BatchTuning | None = None,
                 per_request_completion: bool = True):
        self.store = store
        self.dev = store.dev
        self.policy = AdmissionPolicy(budget_bytes, max_in_flight, max_batch)
        self.precision = geo2rdr_precision
        self.tuning = tuning          # None: per-request kernels for 2+ requests, else the queue
        self.signaled = bool(per_request_completion)
        self.slots = [_Slot(self.dev, max_batch, self.signaled) for _ in range(max_in_flight)]
        self.free_slots = list(self.slots)
        self.pending: collections.deque = collections.deque()
        self.in_flight: list[_InFlight] = []
        self.used = 0
        self.batches = 0
        self.batch_sizes: list[int] = []
        self.max_concurrent = 0

    def _request(self, r: ServeRequest) -> GeocodeRequest:
        s = self.store.slcs[r.slc_key]
        g = r.geogrid
        r.geo = torch.empty((g.length, g.width), dtype=torch.complex64, device=self.dev)
        r.mask = torch.empty((g.length, g.width), dtype=torch.uint8, device=self.dev)
        kw = dict(mask_block=r.mask, az_carrier=s.az_carrier, rg_carrier=s.rg_carrier, rdr_deramped=True)
        kw.update(r.kwargs)
        return GeocodeRequest(r.geo, s.slc, self.store.dem, s.radar_grid, g, s.orbit, s.native_doppler,
                              s.image_grid_doppler, r.kwargs.get("ellipsoid") or _default_ellipsoid(),
                              r.threshold_geo2rdr, r.num_iter_geo2rdr,
                              {k: v for k, v in kw.items() if k != "ellipsoid"})

    def _retire(self, now_fn) -> int:
        done = 0
        still = []
        for f in self.in_flight:
            finished = f.event.query()
            if f.slot.flags is not None and f.open:
                flags = f.slot.flags.array
                t = None
                keep = []
                for i in f.open:
                    if flags[i]:
                        t = now_fn() if t is None else t
                        f.requests[i].t_done = t
                        done += 1
                    else:
                        keep.append(i)
                f.open = keep
            if finished:
                try:
                    f.batch.wait(f.slot.stream)
                except Exception as e:     # report per request, keep serving
                    for r in f.requests:
                        r.error = str(e)
                t = now_fn()
                for i in f.open:
                    f.requests[i].t_done = t
                done += len(f.open)
                f.open = []
                f.batch.close()
                self.used -= f.nbytes
                self.free_slots.append(f.slot)
            else:
                still.append(f)
        self.in_flight = still
        return done

    def _admit(self, now_fn, finished: list) -> int:
        if not self.free_slots or not self.pending:
            return 0
        admitted, rejected = self.policy.select(self.pending, self.used, len(self.in_flight), self.store.nbytes)
        for r in rejected:
            r.t_done = now_fn()
            finished.append(r)
        if not admitted:
            return 0
        slot = self.free_slots.pop(0)
        stream = slot.stream
        t = now_fn()
        with torch.cuda.stream(stream):
            reqs = []
            for r in admitted:
                r.t_admit = t
                reqs.append(self._request(r))
            if slot.flags is not None:
                slot.flags.clear()         # the slot's previous batch has retired
            tuning = self.tuning or BatchTuning(use_graph=False, per_request=len(reqs) > 1)
            batch = GeocodeBatch(reqs, self.precision, tuning, self.dev, stream, done_flags=slot.flags)
            batch.launch(stream)
            ev = torch.cuda.Event()
            ev.record(stream)
        nbytes = sum(r.footprint for r in admitted)
        self.used += nbytes
        self.in_flight.append(_InFlight(batch, admitted, ev, slot, nbytes))
        self.batches += 1
        self.batch_sizes.append(len(admitted))
        self.max_concurrent = max(self.max_concurrent, len(self.in_flight))
        finished.extend(admitted)
        return len(admitted)

    def serve(self, trace: list[ServeRequest], keep_outputs: bool = False) -> dict:
        """Run ``trace`` (requests with arrival times in seconds) to completion."""
        order = sorted(trace, key=lambda r: r.arrival)
        t0 = time.perf_counter()

        def now():
            return time.perf_counter() - t0

        nxt = 0
        finished: list[ServeRequest] = []
        while nxt < len(order) or self.pending or self.in_flight:
            t = now()
            while nxt < len(order) and order[nxt].arrival <= t:
                self.pending.append(order[nxt])
                nxt += 1
            self._retire(now)
            self._admit(now, finished)
            if not self.in_flight and not self.pending and nxt < len(order):
                time.sleep(max(0.0, order[nxt].arrival - now()))
            elif self.in_flight and (not self.free_slots or not self.pending):
                # yield, then poll again: a timed sleep of even 50 us wakes
                # 60-100 us later and delays every completion by that much
                time.sleep(0)
        if not keep_outputs:
            for r in order:
                r.geo = r.mask = None
        out = summarize(order, self.batches, self.batch_sizes)
        out["max_concurrent_batches"] = self.max_concurrent
        out["per_request_completion"] = self.signaled
        return out

    def close(self) -> None:
        for s in self.slots:
            if s.flags is not None:
                s.flags.close()


def _default_ellipsoid():
    from .core import Ellipsoid
    return Ellipsoid()


def summarize(requests: list[ServeRequest], batches: int = 0, batch_sizes=None) -> dict:
    ok = [r for r in requests if r.error is None and r.t_done is not None]
    lat = np.array([r.latency for r in ok]) * 1e3
    px = sum(r.npx for r in ok)
    span = (max(r.t_done for r in ok) - min(r.arrival for r in ok)) if ok else 0.0
    out = {"requests": len(requests), "completed": len(ok), "rejected": len(requests) - len(ok),
           "output_px": int(px), "makespan_s": span, "px_per_s": px / span if span > 0 else 0.0,
           "p50_ms": float(np.percentile(lat, 50)) if lat.size else None,
           "p99_ms": float(np.percentile(lat, 99)) if lat.size else None,
           "mean_ms": float(lat.mean()) if lat.size else None}
    if batches:
        out["batches"] = batches
        out["mean_batch_requests"] = float(np.mean(batch_sizes)) if batch_sizes else 0.0
    return out


def serve_plain(store: ResidentStore, trace: list[ServeRequest], geo2rdr_precision: str = "fp64",
                keep_outputs: bool = False) -> dict:
    """Baseline: one synchronous geocode_slc per request, first-in first-out."""
    order = sorted(trace, key=lambda r: r.arrival)
    t0 = time.perf_counter()
    for r in order:
        wait = r.arrival - (time.perf_counter() - t0)
        if wait > 0:
            time.sleep(wait)
        s = store.slcs[r.slc_key]
        g = r.geogrid
        r.geo = torch.empty((g.length, g.width), dtype=torch.complex64, device=store.dev)
        r.mask = torch.empty((g.length, g.width), dtype=torch.uint8, device=store.dev)
        r.t_admit = time.perf_counter() - t0
        kw = dict(mask_block=r.mask, az_carrier=s.az_carrier, rg_carrier=s.rg_carrier, rdr_deramped=True)
        kw.update({k: v for k, v in r.kwargs.items() if k != "ellipsoid"})
        geocode_slc(r.geo, s.slc, store.dem, s.radar_grid, g, s.orbit, s.native_doppler, s.image_grid_doppler,
                    r.kwargs.get("ellipsoid") or _default_ellipsoid(), r.threshold_geo2rdr, r.num_iter_geo2rdr,
                    geo2rdr_precision=geo2rdr_precision, **kw)
        r.t_done = time.perf_counter() - t0
        if not keep_outputs:
            r.geo = r.mask = None
    return summarize(order)
