#!/usr/bin/env python
"""Throughput of the GB300 SLC geocoder on the frame-scale workload.

Workload ("frame", the single-GPU configuration the metric is quoted on): a
16384 x 8192 complex64 SLC (circular complex Gaussian, seeded) geocoded onto
an 8000 x 8000 UTM (EPSG:32611) 10 m geogrid over a 1 arc-second EPSG:4326
fBm DEM (0-3000 m), with a 32 x 32 native-Doppler LUT2d (quadratic in range,
+-50 Hz) and a linear azimuth carrier.  One step = one plain geocode_slc call
over the whole frame (64M output pixels).

Printed JSON (one line):
- value: output px/s with inputs resident in HBM (CUDA events, K steps);
- e2e: the same through the drop-in call with pinned host buffers, H2D of the
  SLC and DEM window and D2H of the geocoded frame and mask inside the timing;
- roofline: the fused geocode kernel's algorithmic bytes per launch over its
  CUDA-event duration, against the measured HBM copy bandwidth; plus the FP64
  pipe it is actually bound by;
- cpu_baseline: the CPU oracle (a restatement of the reference's OpenMP
  geocodeSlc) on a bounded sample of geogrid rows, all host cores;
- parity_sample: the GPU frame against the oracle on that sample.
``--impl reference`` times the oracle alone (the reference's CPU algorithm) on
the same workload, metric and units.
"""
from __future__ import annotations

import argparse
import gc
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "geocoded px/s (batched/served vs plain, 1 GB300, ≤1e-4 rad); p50/p99 latency"
UNIT = "px/s"


def parse_args():
    p = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["gslc", "reference"], default="gslc")
    p.add_argument("--workload", choices=["frame", "medium", "small"], default="frame")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-batched", action="store_true", help="skip the burst (batched vs plain) measurement")
    p.add_argument("--no-served", action="store_true", help="skip the serving-loop measurement")
    p.add_argument("--no-geometry", action="store_true", help="skip the block-planner and metadata-cube legs")
    p.add_argument("--profile-summary", nargs=2, metavar=("FP64_CSV", "FF_CSV"),
                   help="instead of timing: write profiles/geocode_kernel_medium.json from the raw-page CSV "
                        "exports (ncu -i REPORT --page raw --csv) of the medium captures of the FP64 and "
                        "float-float geocode_kernel launches")
    p.add_argument("--precision-study", action="store_true",
                   help="instead of timing: fp64 and float-float geo2rdr against the oracle over the whole "
                        "workload (error histograms, Newton iteration counts); writes one JSON line")
    return p.parse_args()


def make_scene(workload: str):
    from isce3_gb300 import synth
    if workload == "frame":
        return synth.scene_c2(seed=2)
    if workload == "medium":     # profiling size: 256 MiB SLC, 4000 x 4000 output
        return synth.scene_c2(seed=2, length=8192, width=4096, geo=4000, spacing=10.0)
    return synth.scene_c2(seed=2, length=4096, width=2048, geo=2000, spacing=12.0)


def workload_config(sc, args, world):
    g = sc.geogrid
    return {"workload": f"plain geocode_slc, {sc.radar_grid.length}x{sc.radar_grid.width} c64 SLC -> "
                        f"{g.length}x{g.width} UTM EPSG:{g.epsg} {g.spacing_x:g} m",
            "slc_shape": [sc.radar_grid.length, sc.radar_grid.width], "geogrid_shape": [g.length, g.width],
            "epsg": g.epsg, "dem": f"{sc.dem.length}x{sc.dem.width} EPSG:4326 fBm 0-3000 m",
            "native_doppler": "LUT2d 32x32 quadratic in range +-50 Hz", "az_carrier": "Poly2d linear",
            "geo2rdr": "fp64", "form": "plain", "l2": "inputs larger than L2 (1 GiB SLC, 512 MiB output)",
            "replicas": world, "seed": sc.seed}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None
        self.skip = 0       # samples written before the timed region

    def start(self):
        """Start sampling every 50 ms and return once the first sample is
        written (at most 3 s), so that the samples fall inside the timed
        region that follows."""
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        t_end = time.perf_counter() + 3.0
        while time.perf_counter() < t_end and self.proc.poll() is None:
            if Path(self.path).stat().st_size > 0:
                break
            time.sleep(0.005)
        self.skip = sum(1 for ln in Path(self.path).read_text().splitlines() if ln.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = [ln.split(",") for ln in Path(self.path).read_text().splitlines() if ln.strip()]
        os.unlink(self.path)
        # samples taken before start() returned are not in the timed region,
        # unless they are all there is
        if len(rows) > self.skip:
            rows = rows[self.skip:]
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except ValueError:
                continue
            for name, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------- CPU side
def radar_bbox(az, rg, shape, margin=9):
    """Radar block covering the chips of the given coordinates (the reference
    raster mode pads its block by 5 lines/samples, geocodeSlc.cpp:740-750;
    the sinc chip adds 4)."""
    v = np.isfinite(az) & np.isfinite(rg)
    if not v.any():
        return 0, 1, 0, 1
    a0 = max(int(np.floor(az[v].min())) - margin, 0)
    a1 = min(int(np.ceil(az[v].max())) + margin + 1, shape[0])
    r0 = max(int(np.floor(rg[v].min())) - margin, 0)
    r1 = min(int(np.ceil(rg[v].max())) + margin + 1, shape[1])
    return a0, a1, r0, r1


def sample_rows_block(oracle, sc, row0, nrows):
    """Geogrid rows [row0, row0+nrows) and the radar sub-block they need, the
    way the reference's block generator feeds geocode_slc."""
    g = sc.geogrid[row0:row0 + nrows, 0:sc.geogrid.width]
    coarse = sc.geogrid[row0:row0 + nrows:1, 0:sc.geogrid.width]
    az = np.zeros((coarse.length, coarse.width))
    rg = np.zeros_like(az)
    dummy = np.zeros((16, 16), np.complex64)
    geo = np.zeros((coarse.length, coarse.width), np.complex64)
    oracle.geocode_slc(geo, dummy, sc.dem, sc.radar_grid, coarse, sc.orbit, sc.native_doppler,
                       sc.image_grid_doppler, sc.ellipsoid, sc.threshold, sc.maxiter,
                       az_index_block=az, rg_index_block=rg, az_carrier=sc.az_carrier, rg_carrier=sc.rg_carrier)
    return g, radar_bbox(az, rg, sc.slc.shape)


def run_oracle_sample(oracle, sc, g, box, outputs=False):
    a0, a1, r0, r1 = box
    block = np.ascontiguousarray(sc.slc[a0:a1, r0:r1])
    geo = np.zeros((g.length, g.width), np.complex64)
    mask = np.zeros((g.length, g.width), np.uint8)
    az = np.zeros((g.length, g.width)) if outputs else None
    rg = np.zeros((g.length, g.width)) if outputs else None
    t0 = time.perf_counter()
    phases = oracle.geocode_slc(geo, block, sc.dem, sc.radar_grid, g, sc.orbit, sc.native_doppler,
                                sc.image_grid_doppler, sc.ellipsoid, sc.threshold, sc.maxiter, mask_block=mask,
                                first_azimuth_line=a0, first_range_sample=r0, az_carrier=sc.az_carrier,
                                rg_carrier=sc.rg_carrier, az_index_block=az, rg_index_block=rg,
                                inplace_deramp=True)
    dt = time.perf_counter() - t0
    return dt, phases, dict(geo=geo, mask=mask, az=az, rg=rg)


def fp64_peak_probe() -> float:
    """The DFMA loop's GFLOP/s on this GPU: the FP64 roofline's denominator."""
    import torch
    from isce3_gb300 import _lib as L
    lib = L.lib()
    ctx = L.context(torch.cuda.current_device())
    fp = C_double()
    L.check(lib.gslc_probe_fp64_gflops(ctx, fp), ctx)
    return fp.value


def cpu_sample_rows(sc, steps: int, warmup: int):
    """Geogrid rows of both CPU timings (the cpu_baseline leg and the
    reference arm): the whole geogrid when at most 13 oracle runs are timed
    (the default 10 steps after 3 warm-ups), else its centred half, so that
    the reference arm's warm-up and timed steps end within about two
    minutes on the frame (9.6 s per whole-frame run on 16 cores)."""
    n = sc.geogrid.length
    if steps + warmup <= 13:
        return 0, n
    rows = n // 2
    return (n - rows) // 2, rows


def cpu_baseline(sc, steps: int, warmup: int):
    from oracle import oracle
    oracle.build()
    row0, rows = cpu_sample_rows(sc, steps, warmup)
    g, box = sample_rows_block(oracle, sc, row0, rows)
    dt, phases, out = run_oracle_sample(oracle, sc, g, box, outputs=True)
    npx = g.length * g.width
    info = {"value": npx / dt, "unit": UNIT, "cores": oracle.ncores(), "kind": "port",
            "sample": f"geogrid rows {row0}..{row0 + rows - 1} (x{g.width}) of the frame with their radar "
                      f"sub-block {box[1] - box[0]}x{box[3] - box[2]}; {npx} px in {dt:.2f} s",
            "phase_seconds": {"index": phases[0], "deramp": phases[1], "interpolate": phases[2],
                              "reramp": phases[3]},
            "arch": os.uname().machine}
    if rows < sc.geogrid.length:
        # the whole frame once as well (the DEM window and blocks as one call)
        gw, boxw = sample_rows_block(oracle, sc, 0, sc.geogrid.length)
        dtw = run_oracle_sample(oracle, sc, gw, boxw)[0]
        info["whole_frame"] = {"value": gw.length * gw.width / dtw, "seconds": dtw,
                               "sample": f"all {gw.length} geogrid rows with the radar block they need"}
    return info, (row0, rows, box, out)


# ---------------------------------------------------------------- GPU side
def slc_footprint(az, rg, shape):
    """SLC samples read by the 8x8 sinc chips of all valid pixels, assuming
    each radar line's footprint is one interval (true for a swath)."""
    import torch
    v = torch.isfinite(az) & torch.isfinite(rg)
    ia = torch.floor(az[v]).long().clamp(0, shape[0] - 1)
    ir = torch.floor(rg[v]).long().clamp(0, shape[1] - 1)
    big = torch.iinfo(torch.int64).max
    lo = torch.full((shape[0],), big, dtype=torch.int64, device=az.device)
    hi = torch.full((shape[0],), -1, dtype=torch.int64, device=az.device)
    lo.scatter_reduce_(0, ia, ir, reduce="amin")
    hi.scatter_reduce_(0, ia, ir, reduce="amax")
    lo, hi = lo.cpu().numpy(), hi.cpu().numpy()
    n = 0
    for r in range(shape[0]):
        a, b = max(r - 4, 0), min(r + 4, shape[0])        # chip rows intAz-3 .. intAz+4
        l_, h_ = lo[a:b].min(), hi[a:b].max()
        if h_ >= 0:
            n += min(h_ + 4, shape[1] - 1) - max(l_ - 3, 0) + 1
    return int(n)


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def run_gpu(args, rank, world):
    import torch
    from isce3_gb300 import _lib as L
    from isce3_gb300.geocode import geocode_slc

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    sc = make_scene(args.workload)
    g = sc.geogrid
    npx = g.length * g.width
    lib = L.lib()
    ctx = L.context(dev.index)
    L.check(lib.gslc_ctx_set_timing(ctx, 1), ctx)
    slc_d = torch.from_numpy(sc.slc).to(dev)
    geo_d = torch.empty((g.length, g.width), dtype=torch.complex64, device=dev)
    mask_d = torch.empty((g.length, g.width), dtype=torch.uint8, device=dev)
    common = (sc.dem, sc.radar_grid, g, sc.orbit, sc.native_doppler, sc.image_grid_doppler, sc.ellipsoid,
              sc.threshold, sc.maxiter)
    kw = dict(az_carrier=sc.az_carrier, rg_carrier=sc.rg_carrier)

    # one diagnostic call for radar coordinates (algorithmic bytes, parity sample)
    az_d = torch.empty((g.length, g.width), dtype=torch.float64, device=dev)
    rg_d = torch.empty_like(az_d)
    geocode_slc(geo_d, slc_d, *common, mask_block=mask_d, az_index_block=az_d, rg_index_block=rg_d, **kw)
    n_valid = int(torch.isfinite(az_d).sum())
    n_slc = slc_footprint(az_d, rg_d, sc.slc.shape)
    dem_keep = [v for v in sc.dem.__dict__.get("_gslc_dev", {}).values()]
    dem_bytes = sum(t.numel() * 4 for t in dem_keep)
    alg_bytes = 8 * npx + 1 * npx + 8 * n_slc + dem_bytes

    stream = torch.cuda.current_stream(dev)
    for _ in range(args.warmup):
        geocode_slc(geo_d, slc_d, *common, mask_block=mask_d, **kw)
    sampler = ClockSampler(dev.index)
    kernel_ms, deramp_ms, launches = [], [], 0
    _barrier(world)
    torch.cuda.synchronize()
    sampler.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        geocode_slc(geo_d, slc_d, *common, mask_block=mask_d, **kw)
        a, b = _kernel_ms(lib, ctx)
        kernel_ms.append(a)
        deramp_ms.append(b)
        launches += int(lib.gslc_last_launch_count(ctx))
    e1.record(stream)
    torch.cuda.synchronize()
    _barrier(world)
    clocks = sampler.stop()
    ms = e0.elapsed_time(e1) / args.steps
    ms = _max_over_ranks(ms, world)
    res = dict(npx=npx, n_valid=n_valid, ms=ms, kernel_ms=float(np.mean(kernel_ms)),
               deramp_ms=float(np.mean(deramp_ms)), launches=launches, clocks=clocks, alg_bytes=alg_bytes,
               n_slc=n_slc, dem_bytes=dem_bytes)

    # float-float geo2rdr beside it: same inputs, timed the same way
    geo_f = torch.empty_like(geo_d)
    mask_f = torch.empty_like(mask_d)
    az_f, rg_f = torch.empty_like(az_d), torch.empty_like(rg_d)
    geocode_slc(geo_f, slc_d, *common, mask_block=mask_f, az_index_block=az_f, rg_index_block=rg_f,
                geo2rdr_precision="ff", **kw)
    for _ in range(args.warmup):
        geocode_slc(geo_f, slc_d, *common, mask_block=mask_f, geo2rdr_precision="ff", **kw)
    torch.cuda.synchronize()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    kms = []
    f0.record(stream)
    for _ in range(args.steps):
        geocode_slc(geo_f, slc_d, *common, mask_block=mask_f, geo2rdr_precision="ff", **kw)
        kms.append(_kernel_ms(lib, ctx)[0])
    f1.record(stream)
    torch.cuda.synchronize()
    ms_ff = f0.elapsed_time(f1) / args.steps
    res["ff"] = dict(ms=ms_ff, kernel_ms=float(np.mean(kms)), value=npx * world / (ms_ff * 1e-3),
                     geo_d=geo_f, mask_d=mask_f, az_d=az_f, rg_d=rg_f)
    res["geo_d"], res["mask_d"], res["az_d"], res["rg_d"] = geo_d, mask_d, az_d, rg_d
    res["e2e"] = None if args.no_e2e else run_e2e(args, sc, dev, common, kw)
    return sc, res


PROFILE = ROOT / "profiles" / "geocode_kernel_medium.json"


def profile_per_px() -> dict:
    """Per-output-pixel figures of the committed ncu capture of the fused
    kernel on the medium workload: {"<name>_per_output_px": value}."""
    if not PROFILE.exists():
        return {}
    d = json.loads(PROFILE.read_text())
    return {f"{k}_per_output_px": float(v) for k, v in d.get("per_output_px", {}).items()}


MEDIUM_PX = 4000 * 4000     # output pixels of the medium workload (the captures' launches)


def _ncu_raw(path) -> dict:
    """Metric name -> value of the one launch in an ncu raw-page CSV export."""
    import csv
    rows = list(csv.reader(Path(path).read_text().splitlines()))
    head = next(i for i, r in enumerate(rows) if "gpu__time_duration.sum" in r)
    names, units = rows[head], rows[head + 1]
    vals = rows[head + 2]
    out = {}
    for n, u, v in zip(names, units, vals):
        try:
            x = float(v.replace(",", ""))
        except ValueError:
            continue
        scale = {"Kbyte": 1e3, "Mbyte": 1e6, "Gbyte": 1e9, "byte": 1.0, "msecond": 1e-3, "usecond": 1e-6,
                 "nsecond": 1e-9, "ms": 1e-3, "us": 1e-6, "ns": 1e-9, "s": 1.0, "second": 1.0}.get(u.strip(), 1.0)
        out[n] = x * scale
    return out


def write_profile_summary(fp64_csv, ff_csv) -> dict:
    """profiles/geocode_kernel_medium.json from the two captures."""
    f, g = _ncu_raw(fp64_csv), _ncu_raw(ff_csv)

    def count(m, op):
        # the raw page gives the summed rate; times the elapsed cycles, the count
        return m[f"smsp__sass_thread_inst_executed_op_{op}_pred_on.sum.per_cycle_elapsed"] * \
            m["smsp__cycles_elapsed.avg"]

    def flop(m):
        return (2 * count(m, "dfma") + count(m, "dadd") + count(m, "dmul")) / MEDIUM_PX
    d = {"kernel": "geocode_kernel (fused SLC geocoder)",
         "workload": "medium: 8192 x 4096 c64 SLC -> 4000 x 4000 UTM EPSG:32611 10 m (16,000,000 output px)",
         "command": "M='python bench.py --workload medium --steps 2 --warmup 1 --no-cpu --no-e2e --no-batched "
                    "--no-served --no-geometry'; ncu --set full --clock-control none -k regex:geocode_kernel -s 2 "
                    "-c 1 -o prof_med_fp64 $M; ncu --set full --clock-control none -k regex:geocode_kernel -s 6 "
                    "-c 1 -o prof_med_ff $M; python bench.py --profile-summary fp64.csv ff.csv (the raw-page "
                    "CSV exports)",
         "per_output_px": {
             "dram_bytes": round((f["dram__bytes_read.sum"] + f["dram__bytes_write.sum"]) / MEDIUM_PX, 3),
             "fp64_flop_fp64": round(flop(f), 1),
             "fp64_flop_ff": round(flop(g), 1)},
         "duration_ms": {"fp64": round(f["gpu__time_duration.sum"] * 1e3, 3),
                         "ff": round(g["gpu__time_duration.sum"] * 1e3, 3)},
         "fp64_inst_per_output_px": {v: {op: round(count(m, op) / MEDIUM_PX, 1) for op in ("dfma", "dadd", "dmul")}
                                     for v, m in (("fp64", f), ("ff", g))},
         "definitions": {
             "dram_bytes": "(dram__bytes_read.sum + dram__bytes_write.sum) of the FP64 launch / 16,000,000",
             "fp64_flop_<variant>": "(2 x DFMA + DADD + DMUL thread instructions) / 16,000,000, each count "
                                    "smsp__sass_thread_inst_executed_op_<op>_pred_on.sum.per_cycle_elapsed x "
                                    "smsp__cycles_elapsed.avg"}}
    PROFILE.write_text(json.dumps(d, indent=2) + "\n")
    return d


def fp64_roofline(prof_vals: dict, variant: str, npx: int, kernel_ms: float, peak_gflops: float) -> dict:
    """FP64 roofline of the fused kernel: FP64 FLOP per output pixel counted
    by ncu (2 x DFMA + DADD + DMUL thread instructions of the medium capture)
    times the frame's pixels over the kernel time measured in this run,
    against the DFMA-loop peak measured in this run."""
    out = {"peak_gflops_measured": peak_gflops, "probe": "gslc_probe_fp64_gflops DFMA loop", "unit": "GFLOP/s"}
    f = prof_vals.get(f"fp64_flop_{variant}_per_output_px")
    if f is not None and kernel_ms > 0:
        ach = f * npx / (kernel_ms * 1e-3) / 1e9
        out.update({"achieved": ach, "peak": peak_gflops, "frac": ach / peak_gflops, "flop_per_output_px": f,
                    "flop_source": f"ncu 2*dfma+dadd+dmul of the medium capture ({PROFILE.name})"})
    return out


def C_double():
    import ctypes
    return ctypes.c_double()


def _kernel_ms(lib, ctx):
    import ctypes
    a, b = ctypes.c_float(), ctypes.c_float()
    lib.gslc_last_kernel_ms(ctx, ctypes.byref(a), ctypes.byref(b))
    return a.value, b.value


def run_e2e(args, sc, dev, common, kw):
    """Drop-in call on pinned host buffers; H2D and D2H inside the timing."""
    import torch
    from isce3_gb300.geocode import geocode_slc
    g = sc.geogrid
    from isce3_gb300.io import Raster
    slc_h = torch.empty(sc.slc.shape, dtype=torch.complex64, pin_memory=True)
    slc_h.numpy()[...] = sc.slc
    geo_h = torch.empty((g.length, g.width), dtype=torch.complex64, pin_memory=True)
    mask_h = torch.empty((g.length, g.width), dtype=torch.uint8, pin_memory=True)
    # the DEM raster's samples in page-locked memory too, so that every input
    # of the step comes from pinned host memory
    dem_t = torch.empty(sc.dem.data.shape, dtype=torch.float32, pin_memory=True)
    dem_t.numpy()[...] = sc.dem.data
    dem_h = Raster(dem_t.numpy(), sc.dem.get_geotransform(), sc.dem.get_epsg())
    common_h = (dem_h,) + tuple(common[1:])
    caches = [dem_h, sc.native_doppler, sc.image_grid_doppler]

    def step():
        for c in caches:            # inputs are re-sent every step
            c.__dict__.pop("_gslc_dev", None)
        geocode_slc(geo_h, slc_h, *common_h, mask_block=mask_h, **kw)

    # at least 15 untimed calls (~0.5 s): after the resident legs' seconds of
    # full-rate FP64 the first copy-heavy calls of the next half second ran
    # a few ms slow
    for _ in range(max(15, args.warmup)):
        step()
    torch.cuda.synchronize()
    gc.collect()
    t = []
    for _ in range(max(args.steps, 20)):     # at least 20 drop-in calls: single outliers weigh less
        t0 = time.perf_counter()
        step()
        torch.cuda.synchronize()
        t.append(time.perf_counter() - t0)
    dem_bytes = sum(v.numel() * 4 for v in dem_h.__dict__.get("_gslc_dev", {}).values())
    lut_bytes = sc.native_doppler.data.nbytes
    h2d = slc_h.numel() * 8 + dem_bytes + lut_bytes
    d2h = geo_h.numel() * 8 + mask_h.numel()
    sec = float(np.mean(t))
    # the reference's own call shape: pageable NumPy arrays in and out
    geo_n = np.zeros((g.length, g.width), np.complex64)
    mask_n = np.zeros((g.length, g.width), np.uint8)

    def step_np():
        for c in (sc.dem, sc.native_doppler, sc.image_grid_doppler):
            c.__dict__.pop("_gslc_dev", None)
        geocode_slc(geo_n, sc.slc, *common, mask_block=mask_n, **kw)

    for _ in range(3):
        step_np()
    torch.cuda.synchronize()
    tn = []
    for _ in range(5):
        t0 = time.perf_counter()
        step_np()
        torch.cuda.synchronize()
        tn.append(time.perf_counter() - t0)
    sec_n = float(np.mean(tn))
    return {"value": g.length * g.width / sec, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(d2h), "ms_per_step": sec * 1e3, "p50_ms": float(np.median(t)) * 1e3,
            "ms_steps": [round(x * 1e3, 2) for x in t],
            "timing": "host wall clock around the drop-in call, synchronized; page-locked host buffers",
            "pageable": {"value": g.length * g.width / sec_n, "unit": UNIT, "ms_per_step": sec_n * 1e3,
                         "p50_ms": float(np.median(tn)) * 1e3, "ms_steps": [round(x * 1e3, 2) for x in tn],
                         "timing": "the same call with pageable NumPy inputs and outputs (the reference's call "
                                   "shape), 5 steps"}}


def _barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def _max_over_ranks(x, world):
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([x], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())
    return x


def run_bursts(args):
    """27 uneven TOPS-like bursts onto one 12000 x 12000 UTM grid: plain
    per-burst calls against one batched persistent graph launch."""
    import torch
    from isce3_gb300 import synth
    from isce3_gb300.autotune import time_batch, tune
    from isce3_gb300.batch import GeocodeBatch, GeocodeRequest
    from isce3_gb300.geocode import geocode_slc
    dev = torch.device("cuda", torch.cuda.current_device())
    if args.workload == "frame":
        sc = synth.scene_bursts(seed=4, device=dev)
    else:
        sc = synth.scene_bursts(seed=4, n_az=3, n_sw=3, grid_px=3000, spacing=20.0, lines=(500, 700),
                                samples=(4000, 6000), device=dev)
    outs = [(torch.empty((b.window.length, b.window.width), dtype=torch.complex64, device=dev),
             torch.empty((b.window.length, b.window.width), dtype=torch.uint8, device=dev)) for b in sc.bursts]
    npx = sum(b.window.length * b.window.width for b in sc.bursts)
    common = (sc.dem,)
    res = {"bursts": len(sc.bursts), "output_px": npx, "grid": [sc.geogrid.length, sc.geogrid.width],
           "burst_lines": [min(b.radar_grid.length for b in sc.bursts), max(b.radar_grid.length for b in sc.bursts)],
           "burst_samples": [min(b.radar_grid.width for b in sc.bursts), max(b.radar_grid.width for b in sc.bursts)],
           "prf_hz": sc.prf, "wavelength_m": 0.0555, "range_spacing_m": 2.33,
           "carrier": "Poly2d quadratic in azimuth time (2000 Hz/s)"}
    steps = max(2, min(args.steps, 3))
    for prec in ("fp64", "ff"):
        def plain_pass():
            for b, (g, m) in zip(sc.bursts, outs):
                geocode_slc(g, b.slc, *common, b.radar_grid, b.window, sc.orbit, sc.native_doppler,
                            sc.image_grid_doppler, sc.ellipsoid, sc.threshold, sc.maxiter, mask_block=m,
                            az_carrier=b.az_carrier, rg_carrier=b.rg_carrier, geo2rdr_precision=prec)
        plain_pass()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps):
            plain_pass()
        torch.cuda.synchronize()
        ms_plain = (time.perf_counter() - t0) / steps * 1e3
        ref = [(g.clone(), m.clone()) for g, m in outs]
        valid = sum(int((m == 1).sum()) for _, m in outs)
        reqs = [GeocodeRequest(g, b.slc, sc.dem, b.radar_grid, b.window, sc.orbit, sc.native_doppler,
                               sc.image_grid_doppler, sc.ellipsoid, sc.threshold, sc.maxiter,
                               dict(mask_block=m, az_carrier=b.az_carrier, rg_carrier=b.rg_carrier))
                for b, (g, m) in zip(sc.bursts, outs)]
        best, tried = tune(reqs, prec)
        batch = GeocodeBatch(reqs, prec, best)
        t0 = time.perf_counter()
        ms_batch = time_batch(batch, steps)
        wall_batch = (time.perf_counter() - t0) / (steps + 1) * 1e3
        same = all(torch.equal(m0, m1) and torch.equal(torch.view_as_real(g0).view(torch.int32), torch.view_as_real(g1).view(torch.int32))
                   for (g0, m0), (g1, m1) in zip(ref, outs))
        info = batch.info()
        batch.close()
        res[prec] = {"plain_ms": ms_plain, "plain_px_per_s": npx / (ms_plain * 1e-3),
                     "plain_timing": "host wall clock over sequential synchronous geocode_slc calls",
                     "batched_ms": ms_batch, "batched_px_per_s": npx / (ms_batch * 1e-3),
                     "batched_timing": "CUDA events around graph launches",
                     "batched_wall_ms": wall_batch,
                     "speedup": ms_plain / ms_batch, "valid_px": valid, "batched_equals_plain": bool(same),
                     "tuning": {"form": "per-request kernels" if best.per_request else "persistent queue",
                                "rows_per_thread": best.rows_per_thread, "tiles_per_pop": best.tiles_per_pop,
                                "blocks_per_sm": best.blocks_per_sm,
                                "tried_ms": {"x".join(map(str, k)) if isinstance(k, tuple) else k: v
                                             for k, v in tried.items()},
                                "tried_key": "rows_per_thread x tiles_per_pop x blocks_per_sm of the "
                                             "persistent queue; per-request: each request's own kernel"},
                     "tiles": info["tiles"], "blocks": info["blocks"], "launches_per_run": info["launches_per_run"]}
        del ref
        torch.cuda.empty_cache()
    return res


def run_serving(args):
    """Geocode requests over 8 resident SLCs, continuous-batching server
    against the plain per-request path, on two traces of the same requests:
    Poisson arrivals at 200 req/s (bound by the arrival rate) and every
    request arriving at t = 0 (saturated: throughput is the GPU's)."""
    import torch
    from isce3_gb300 import synth
    from isce3_gb300.serve import GeocodeServer, ResidentStore, ServeRequest, serve_plain
    dev = torch.device("cuda", torch.cuda.current_device())
    if args.workload == "frame":
        sc = synth.scene_serving(seed=5, device=dev)
        n_req = 200
    else:
        sc = synth.scene_serving(seed=5, n_slc=4, lines=(2048, 4096), samples=(2048, 4096), device=dev)
        n_req = 60
    store = ResidentStore(sc.dem, dev)
    for s_ in sc.slcs:
        store.add(s_.key, s_.slc, s_.radar_grid, s_.orbit, native_doppler=s_.native_doppler,
                  az_carrier=s_.az_carrier, rg_carrier=s_.rg_carrier, copy=False)
    torch.cuda.synchronize()
    trace = synth.serving_trace(sc, n_requests=n_req, rate_hz=200.0, seed=6)
    warm = synth.serving_trace(sc, n_requests=16, rate_hz=2000.0, side=(256, 1024), seed=7)
    out = {"slcs": len(sc.slcs), "resident_bytes": store.nbytes, "requests": n_req, "rate_hz": 200.0,
           "side_px": [256, 4096], "spacing_m": [10, 30], "budget_bytes": 150 * 10 ** 9,
           "slc_shapes": [list(s_.radar_grid.shape) for s_ in sc.slcs]}
    traces = {"poisson_200hz": trace, "saturated_t0": [(k, g, 0.0) for k, g, _t in trace]}
    for prec in ("fp64", "ff"):
        warm_server = GeocodeServer(store, geo2rdr_precision=prec)
        warm_server.serve([ServeRequest(k, g, t) for k, g, t in warm])
        warm_server.close()
        serve_plain(store, [ServeRequest(k, g, t) for k, g, t in warm], prec)
        out[prec] = {}
        for name, tr in traces.items():
            server = GeocodeServer(store, budget_bytes=150 * 10 ** 9, max_in_flight=3, max_batch=64,
                                   geo2rdr_precision=prec, per_request_completion=True)
            served = server.serve([ServeRequest(k, g, t) for k, g, t in tr])
            server.close()
            plain = serve_plain(store, [ServeRequest(k, g, t) for k, g, t in tr], prec)
            out[prec][name] = {"served": served, "plain": plain,
                               "px_per_s_ratio": served["px_per_s"] / plain["px_per_s"] if plain["px_per_s"] else None}
    return out


def run_geometry(args, sc):
    """Block planning and metadata cubes around the frame: the GPU call (one
    launch of bounding boxes, the cube passes) against the oracle on the host
    cores, with their agreement."""
    import torch
    from oracle import oracle
    from isce3_gb300 import geometry
    from isce3_gb300.product import GeoGridParameters
    from isce3_gb300.rdr_geo_block_generator import plan_blocks
    oracle.build()
    g = sc.geogrid
    out = {}
    # planner: the frame's geogrid in 500 x 500 blocks (256 blocks), DEM heights
    blocks = [b for _, _, b in plan_blocks(g, 500, 500)]
    dem = geometry.DEMInterpolator(sc.dem)
    mn, mx, _ = dem.compute_min_max_mean_height()
    for _ in range(2):
        geometry.get_radar_bboxes(blocks, sc.radar_grid, sc.orbit, float(mn), float(mx))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    reps = 5
    for _ in range(reps):
        gpu = geometry.get_radar_bboxes(blocks, sc.radar_grid, sc.orbit, float(mn), float(mx))
    gpu_s = (time.perf_counter() - t0) / reps
    t0 = time.perf_counter()
    ref = [oracle.radar_bbox(b, sc.radar_grid, sc.orbit, float(mn), float(mx)) for b in blocks]
    cpu_s = time.perf_counter() - t0
    same = sum(1 for a, r in zip(gpu, ref)
               if (r[4] != 0 and isinstance(a, Exception)) or
               (r[4] == 0 and not isinstance(a, Exception) and
                (a.first_azimuth_line, a.last_azimuth_line, a.first_range_sample, a.last_range_sample) == r[:4]))
    out["planner"] = {"blocks": len(blocks), "block_px": [500, 500], "gpu_ms_per_plan": gpu_s * 1e3,
                      "cpu_ms_per_plan": cpu_s * 1e3, "cpu_threads": 1, "equal_to_oracle": same,
                      "timing": "host wall clock around the synchronous call (H2D, launch, D2H)"}
    # cubes: 20 heights x 200 x 200 at 500 m over the frame (the GSLC workflow's cube)
    h = np.arange(-500.0, 9001.0, 500.0)
    n = 200
    cx, cy = g.start_x + g.spacing_x * g.width / 2, g.start_y + g.spacing_y * g.length / 2
    cube = GeoGridParameters(cx - 250.0 * n, cy + 250.0 * n, 500.0, -500.0, n, n, g.epsg)
    shape = (h.size, n, n)
    names = [k for k, _ in oracle.CUBE_NAMES]
    dts = dict(oracle.CUBE_NAMES)
    arrs = {k: torch.empty(shape, dtype=torch.float64 if dts[k] == np.float64 else torch.float32, device="cuda")
            for k in names}
    kw = {f"{k}_raster": v for k, v in arrs.items()}
    geometry.make_radar_grid_cubes(sc.radar_grid, cube, h, sc.orbit, sc.native_doppler, sc.image_grid_doppler,
                                   numiter_geo2rdr=100, delta_range=1e-8, **kw)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(3):
        geometry.make_radar_grid_cubes(sc.radar_grid, cube, h, sc.orbit, sc.native_doppler,
                                       sc.image_grid_doppler, numiter_geo2rdr=100, delta_range=1e-8, **kw)
    gpu_s = (time.perf_counter() - t0) / 3
    from isce3_gb300 import _lib as L
    passes = int(L.lib().gslc_last_cube_passes(L.context(torch.cuda.current_device())))
    ncpu = oracle.ncores()
    t0 = time.perf_counter()
    ref = oracle.radar_grid_cubes(sc.radar_grid, cube, h, sc.orbit, sc.native_doppler, sc.image_grid_doppler,
                                  maxiter=100, delta_range=1e-8, nthreads=ncpu)
    cpu_s = time.perf_counter() - t0
    par = {}
    for k in names:
        a, r = arrs[k].cpu().numpy(), ref[k]
        v = np.isfinite(r)
        par[k] = {"mask_mismatch": int((np.isfinite(a) != v).sum()),
                  "max_abs_diff": float(np.max(np.abs(a[v].astype(np.float64) - r[v]))) if v.any() else 0.0}
    npts = int(np.prod(shape))
    out["cubes"] = {"points": npts, "shape": list(shape), "spacing_m": 500.0, "gpu_ms": gpu_s * 1e3,
                    "points_per_s": npts / gpu_s, "passes": passes, "cpu_ms": cpu_s * 1e3,
                    "cpu_points_per_s": npts / cpu_s, "cpu_threads": ncpu, "parity": par,
                    "timing": "host wall clock around the synchronous call"}
    return out


def parity_sample(res, row0, rows, box, out):
    """GPU frame rows against the oracle's run on the same rows."""
    from oracle.compare import compare
    sl = slice(row0, row0 + rows)
    geo = res["geo_d"][sl].cpu().numpy()
    mask = res["mask_d"][sl].cpu().numpy()
    az = res["az_d"][sl].cpu().numpy()
    rg = res["rg_d"][sl].cpu().numpy()
    r = compare(geo, out["geo"], az, out["az"], rg, out["rg"], mask, out["mask"])
    r["rows"] = [row0, row0 + rows]
    r["tolerance"] = "|d| <= 1e-5|ref| + 1e-6 rms; phase <= 1e-4 rad; masks exact; flips/splits counted"
    return r


def _abs_stats(x: np.ndarray) -> dict:
    """Quantiles and a decade histogram of |x| (zeros counted apart)."""
    x = np.abs(x[np.isfinite(x)])
    if x.size == 0:
        return {"n": 0}
    q = np.quantile(x, [0.5, 0.9, 0.99, 0.999, 0.9999])
    nz = x[x > 0]
    edges = np.arange(-18, 2)
    hist = np.histogram(np.log10(nz), bins=edges)[0] if nz.size else np.zeros(len(edges) - 1, int)
    return {"n": int(x.size), "zeros": int(x.size - nz.size), "p50": float(q[0]), "p90": float(q[1]),
            "p99": float(q[2]), "p999": float(q[3]), "p9999": float(q[4]), "max": float(x.max()),
            "log10_hist": {f"[1e{int(a)},1e{int(a) + 1})": int(c) for a, c in zip(edges[:-1], hist) if c}}


def run_precision_study(args):
    """fp64 and float-float geo2rdr against the oracle over the whole
    workload: histograms of the azimuth-time, slant-range and phase
    differences and of the relative complex error, and the oracle's Newton
    iteration counts."""
    import torch
    from isce3_gb300.geocode import geocode_slc
    from oracle import oracle
    from oracle.compare import compare
    oracle.build()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    sc = make_scene(args.workload)
    g = sc.geogrid
    rgd = sc.radar_grid
    common = (sc.dem, rgd, g, sc.orbit, sc.native_doppler, sc.image_grid_doppler, sc.ellipsoid, sc.threshold,
              sc.maxiter)
    kw = dict(az_carrier=sc.az_carrier, rg_carrier=sc.rg_carrier)
    slc_d = torch.from_numpy(sc.slc).to(dev)
    gpu = {}
    for prec in ("fp64", "ff"):
        geo = torch.empty((g.length, g.width), dtype=torch.complex64, device=dev)
        mask = torch.empty((g.length, g.width), dtype=torch.uint8, device=dev)
        az = torch.empty((g.length, g.width), dtype=torch.float64, device=dev)
        rg = torch.empty_like(az)
        geocode_slc(geo, slc_d, *common, mask_block=mask, az_index_block=az, rg_index_block=rg,
                    geo2rdr_precision=prec, **kw)
        torch.cuda.synchronize()
        gpu[prec] = {k: v.cpu().numpy() for k, v in dict(geo=geo, mask=mask, az=az, rg=rg).items()}
        del geo, mask, az, rg
    del slc_d
    torch.cuda.empty_cache()
    o = {"geo": np.zeros((g.length, g.width), np.complex64), "mask": np.zeros((g.length, g.width), np.uint8),
         "az": np.zeros((g.length, g.width)), "rg": np.zeros((g.length, g.width)),
         "niter": np.zeros((g.length, g.width), np.uint8)}
    t0 = time.perf_counter()
    oracle.geocode_slc(o["geo"], np.array(sc.slc, copy=True), *common, mask_block=o["mask"],
                       az_index_block=o["az"], rg_index_block=o["rg"], niter_block=o["niter"],
                       inplace_deramp=True, **kw)
    t_oracle = time.perf_counter() - t0
    it = o["niter"][o["niter"] > 0]
    out = {"study": "geo2rdr precision vs oracle", "config": workload_config(sc, args, 1),
           "oracle_seconds": t_oracle, "oracle_cores": oracle.ncores(),
           "newton_iterations": {str(int(k)): int(c) for k, c in zip(*np.unique(it, return_counts=True))},
           "mean_newton_iterations": float(it.mean()) if it.size else None}
    for prec, r in gpu.items():
        both = np.isfinite(r["az"]) & np.isfinite(o["az"])
        dt = (r["az"][both] - o["az"][both]) / rgd.prf
        dr = (r["rg"][both] - o["rg"][both]) * rgd.range_pixel_spacing
        gg, go = r["geo"], o["geo"]
        fin = np.isfinite(gg) & np.isfinite(go) & (np.abs(go) > 0)
        dphi = np.angle(gg[fin] * np.conj(go[fin]))
        rel = np.abs(gg[fin] - go[fin]) / np.abs(go[fin])
        summary = compare(gg, go, r["az"], o["az"], r["rg"], o["rg"], r["mask"], o["mask"])
        out[prec] = {"delta_aztime_s": _abs_stats(dt), "delta_srange_m": _abs_stats(dr),
                     "delta_phase_rad": _abs_stats(dphi), "rel_complex_err": _abs_stats(rel),
                     "parity": {k: v for k, v in summary.items() if not isinstance(v, np.ndarray)}}
    print(json.dumps(out, default=float), flush=True)


def run_reference(args, rank, world):
    """The reference's CPU algorithm (the oracle restatement, OpenMP, all host
    cores) on the same workload: each step one bounded sample of geogrid rows."""
    if rank != 0:
        return
    from oracle import oracle
    oracle.build()
    sc = make_scene(args.workload)
    row0, rows = cpu_sample_rows(sc, args.steps, args.warmup)
    g, box = sample_rows_block(oracle, sc, row0, rows)
    for _ in range(args.warmup):
        run_oracle_sample(oracle, sc, g, box)
    times = [run_oracle_sample(oracle, sc, g, box)[0] for _ in range(args.steps)]
    npx = g.length * g.width
    sec = float(np.mean(times))
    value = npx / sec
    line = {"metric": METRIC, "impl": "reference", "value": value, "unit": UNIT, "n_gpus": 0,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32", "data": "synthetic",
            "config": workload_config(sc, args, 1),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": oracle.ncores(), "kind": "port",
                             "sample": f"geogrid rows {row0}..{row0 + rows - 1} (x{g.width}) with their radar "
                                       f"sub-block per step"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "isce3 itself cannot be built here (Eigen/GDAL/HDF5/pyre absent); the timed CPU code is "
                    "the oracle's C++/OpenMP restatement of geocodeSlc"}
    print(json.dumps(line), flush=True)


def main():
    args = parse_args()
    if args.profile_summary:
        print(json.dumps(write_profile_summary(*args.profile_summary)))
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    import torch
    if not torch.cuda.is_available():
        print(json.dumps({"metric": METRIC, "error": "no CUDA GPU"}))
        sys.exit(1)
    from isce3_gb300 import _lib as L
    L.build()
    if args.precision_study:
        run_precision_study(args)
        return
    sc, res = run_gpu(args, rank, world)
    if rank != 0:
        return
    cpu, par = None, None
    par_ff = None
    if not args.no_cpu:
        cpu, (row0, rows, box, out) = cpu_baseline(sc, args.steps, args.warmup)
        par = parity_sample(res, row0, rows, box, out)
        par_ff = parity_sample(res["ff"], row0, rows, box, out)
    batched = None
    if not args.no_batched:
        batched = run_bursts(args)
    geometry_leg = None
    if not args.no_geometry:
        geometry_leg = run_geometry(args, sc)
    served = None
    if not args.no_served:
        served = run_serving(args)
    # the FP64 peak probe last: right after its seconds of full-rate DFMA the
    # next copy-heavy calls ran 8-50 ms slow for about half a second
    res["fp64_peak_gflops"] = fp64_peak_probe()
    hbm_peak, peak_kind = peaks()
    prof_vals = profile_per_px()
    traffic = prof_vals["dram_bytes_per_output_px"] * res["npx"] if "dram_bytes_per_output_px" in prof_vals else None
    kernel_s = res["kernel_ms"] * 1e-3
    achieved = res["alg_bytes"] / kernel_s / 1e9
    value = res["npx"] * world / (res["ms"] * 1e-3)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": res["ms"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64+f32", "data": "synthetic",
        "config": workload_config(sc, args, world),
        "valid_px_per_s": res["n_valid"] * world / (res["ms"] * 1e-3),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "traffic": traffic,
                     "traffic_source": f"ncu dram bytes/px of the medium capture ({PROFILE.name}) x frame px", "peak_source": f"{peak_kind} hbm_gbs",
                     "kernel": "geocode_kernel (fused)", "kernel_ms": res["kernel_ms"],
                     "alg_bytes_per_launch": res["alg_bytes"],
                     "alg_bytes_terms": {"geo_out": 8 * res["npx"], "mask": res["npx"], "slc": 8 * res["n_slc"],
                                         "dem_window": res["dem_bytes"]},
                     "binding": "fp64 pipe (geo2rdr); see fp64"},
        "fp64": fp64_roofline(prof_vals, "fp64", res["npx"], res["kernel_ms"], res["fp64_peak_gflops"]),
        "deramp_ms": res["deramp_ms"],
        "geo2rdr_ff": {"value": res["ff"]["value"], "unit": UNIT, "ms_per_step": res["ff"]["ms"],
                       "kernel_ms": res["ff"]["kernel_ms"], "parity_sample": par_ff,
                       "fp64": fp64_roofline(prof_vals, "ff", res["npx"], res["ff"]["kernel_ms"],
                                             res["fp64_peak_gflops"]),
                       "note": "float-float (double-word FP32) Newton iterations, FP64 first iterate and range"},
        "batched": batched,
        "served": served,
        "geometry": geometry_leg,
        "e2e": res["e2e"], "gpu_launches": res["launches"], "clocks": res["clocks"],
        "cpu_baseline": cpu, "parity_sample": par,
    }
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
