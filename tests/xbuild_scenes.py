"""Scenes of the cross-build parity study, stored with their inputs.

Two reduced scenes, each written to tests/golden/oracle_xbuild.npz with
every input the geocoder reads except the SLC, and with the outputs of the
oracle built for x86-64 (-ffp-contract=off):

- "c1":  the 1024 x 1024 C1 scene onto a 192 x 192 EPSG:4326 geogrid, zero
  Doppler, a 128 x 128 fBm DEM;
- "c2r": a 2048 x 1024 cut of the frame scene onto a 192 x 192 UTM 32611
  geogrid at 24 m, the frame's native Doppler LUT2d and linear azimuth
  carrier, over a 2-arc-second EPSG:4326 DEM cropped around the geogrid.

Inputs are stored because the scene synthesis runs numpy transcendentals
whose last bits depend on the machine (SIMD kernels differ between x86-64 and
aarch64), while the study compares geocoder builds on identical inputs.  The
SLC is not stored: ``hash_slc`` makes it from a splitmix64 hash of the sample
index with integer arithmetic and exact float conversions, identically on
every machine.
"""
from __future__ import annotations

from pathlib import Path
from types import SimpleNamespace

import numpy as np

from isce3_gb300.core import Ellipsoid, LookSide, LUT2d, Orbit, Poly2d
from isce3_gb300.io import Raster
from isce3_gb300.product import GeoGridParameters, RadarGridParameters

GOLDEN = Path(__file__).resolve().parent / "golden" / "oracle_xbuild.npz"
NAMES = ("c1", "c2r")


def _splitmix64(x: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        z = x + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def hash_slc(length: int, width: int, seed: int) -> np.ndarray:
    """complex64 samples with parts uniform on [-1, 1) in steps of 2^-23."""
    idx = np.arange(length * width, dtype=np.uint64) * np.uint64(2) + np.uint64(seed) * np.uint64(1 << 40)
    re = (_splitmix64(idx) >> np.uint64(40)).astype(np.int64) - (1 << 23)
    im = (_splitmix64(idx + np.uint64(1)) >> np.uint64(40)).astype(np.int64) - (1 << 23)
    out = np.empty(length * width, np.complex64)
    out.real = re.astype(np.float32) * np.float32(2.0 ** -23)
    out.imag = im.astype(np.float32) * np.float32(2.0 ** -23)
    return out.reshape(length, width)


def _crop_dem(dem: Raster, geogrid, margin_px: int) -> Raster:
    """The DEM rows/columns over the geogrid's lon/lat box plus a margin."""
    g = geogrid
    xs = g.start_x + g.spacing_x * np.array([0, g.width, 0, g.width])
    ys = g.start_y + g.spacing_y * np.array([0, 0, g.length, g.length])
    if g.epsg == 4326:
        lon, lat = xs, ys
    else:
        lon, lat = _utm_inverse_deg(g.epsg, xs, ys)
    gt = dem.get_geotransform()
    c0 = max(int(np.floor((lon.min() - gt[0]) / gt[1])) - margin_px, 0)
    c1 = min(int(np.ceil((lon.max() - gt[0]) / gt[1])) + margin_px, dem.data.shape[1])
    r0 = max(int(np.floor((lat.max() - gt[3]) / gt[5])) - margin_px, 0)
    r1 = min(int(np.ceil((lat.min() - gt[3]) / gt[5])) + margin_px, dem.data.shape[0])
    return Raster(np.ascontiguousarray(dem.data[r0:r1, c0:c1]),
                  [gt[0] + c0 * gt[1], gt[1], 0.0, gt[3] + r0 * gt[5], 0.0, gt[5]], dem.get_epsg())


def _utm_inverse_deg(epsg, x, y):
    """Approximate UTM inverse by Newton on the host forward (layout only)."""
    from isce3_gb300 import synth
    zone = epsg - 32600 if epsg < 32700 else epsg - 32700
    lon = np.full_like(np.asarray(x, dtype=np.float64), np.radians((zone - 0.5) * 6 - 180))
    lat = np.full_like(lon, np.radians(35.0))
    for _ in range(30):
        fx, fy = synth.utm_forward_host(epsg, lon, lat)
        ex, ey = fx - x, fy - y
        lon = lon - ex / (6378137.0 * np.cos(lat))
        lat = lat - ey / 6378137.0
    return np.degrees(lon), np.degrees(lat)


def build_scenes() -> dict:
    """The two scenes from the seeded synthesis (run where the fixture is made)."""
    from isce3_gb300 import synth
    c1 = synth.scene_c1(seed=1, length=1024, width=1024, geo=192, dem_px=128, slc=False)
    c2 = synth.scene_c2(seed=2, length=2048, width=1024, geo=192, spacing=24.0, dem_arcsec=2.0, slc=False)
    c2.dem = _crop_dem(c2.dem, c2.geogrid, 80)
    return {"c1": c1, "c2r": c2}


def pack(scenes: dict) -> dict:
    """Flatten the scenes' inputs into arrays for np.savez."""
    out = {}
    for name, sc in scenes.items():
        rg, g, o = sc.radar_grid, sc.geogrid, sc.orbit
        p = name + "/"
        out[p + "radar"] = np.array([rg.sensing_start, rg.wavelength, rg.prf, rg.starting_range,
                                     rg.range_pixel_spacing, int(rg.lookside), rg.length, rg.width], np.float64)
        out[p + "geo"] = np.array([g.start_x, g.start_y, g.spacing_x, g.spacing_y, g.width, g.length, g.epsg],
                                  np.float64)
        out[p + "orbit_t"] = np.array([o.t0, o.spacing], np.float64)
        out[p + "orbit_pos"] = np.asarray(o.position, np.float64)
        out[p + "orbit_vel"] = np.asarray(o.velocity, np.float64)
        out[p + "dem"] = sc.dem.data
        out[p + "dem_gt"] = np.asarray(sc.dem.get_geotransform(), np.float64)
        out[p + "dem_epsg"] = np.array([sc.dem.get_epsg()])
        nd = sc.native_doppler
        if nd.have_data:
            out[p + "dop"] = np.asarray(nd.data, np.float64)
            out[p + "dop_grid"] = np.array([nd.x_start, nd.y_start, nd.x_spacing, nd.y_spacing], np.float64)
        car = sc.az_carrier
        if isinstance(car, Poly2d) and car.x_order >= 0:
            out[p + "az_car"] = car.coeffs
            out[p + "az_car_norm"] = np.array([car.x_mean, car.y_mean, car.x_std, car.y_std], np.float64)
        out[p + "numerics"] = np.array([sc.threshold, sc.maxiter], np.float64)
    return out


def unpack(d, name: str) -> SimpleNamespace:
    """One scene's inputs from the fixture, with its SLC from ``hash_slc``."""
    p = name + "/"
    r = d[p + "radar"]
    from isce3_gb300 import synth
    rg = RadarGridParameters(r[0], r[1], r[2], r[3], r[4], LookSide(int(r[5])), int(r[6]), int(r[7]),
                             synth.EPOCH)
    gv = d[p + "geo"]
    g = GeoGridParameters(gv[0], gv[1], gv[2], gv[3], int(gv[4]), int(gv[5]), int(gv[6]))
    ot = d[p + "orbit_t"]
    orbit = Orbit.from_arrays(ot[0], ot[1], d[p + "orbit_pos"], d[p + "orbit_vel"], reference_epoch=synth.EPOCH)
    dem = Raster(d[p + "dem"], list(d[p + "dem_gt"]), int(d[p + "dem_epsg"][0]))
    native = LUT2d()
    if p + "dop" in d:
        x0, y0, dx, dy = d[p + "dop_grid"]
        native = LUT2d(x0, y0, dx, dy, d[p + "dop"])
    az_car, rg_car = LUT2d(), LUT2d()
    if p + "az_car" in d:
        xm, ym, xs, ys = d[p + "az_car_norm"]
        az_car = Poly2d(d[p + "az_car"], x_mean=xm, y_mean=ym, x_std=xs, y_std=ys)
        rg_car = Poly2d(np.zeros((1, 1)))
    thr, maxiter = d[p + "numerics"]
    seed = 1 if name == "c1" else 2
    return SimpleNamespace(name=name, radar_grid=rg, geogrid=g, orbit=orbit, dem=dem,
                           slc=hash_slc(rg.length, rg.width, seed), native_doppler=native,
                           image_grid_doppler=LUT2d(), az_carrier=az_car, rg_carrier=rg_car,
                           ellipsoid=Ellipsoid(), threshold=float(thr), maxiter=int(maxiter))


def carriers(sc) -> dict:
    return dict(az_carrier=sc.az_carrier, rg_carrier=sc.rg_carrier)


def run_oracle(oracle_mod, sc, variant: str = "") -> dict:
    """The oracle's outputs (geo, mask, az, rg) for one scene and build."""
    g = sc.geogrid
    shape = (g.length, g.width)
    geo = np.zeros(shape, np.complex64)
    mask = np.zeros(shape, np.uint8)
    az = np.zeros(shape)
    rgi = np.zeros(shape)
    oracle_mod.geocode_slc(geo, sc.slc, sc.dem, sc.radar_grid, g, sc.orbit, sc.native_doppler,
                           sc.image_grid_doppler, sc.ellipsoid, sc.threshold, sc.maxiter, mask_block=mask,
                           az_index_block=az, rg_index_block=rgi, build_variant=variant, **carriers(sc))
    return dict(geo=geo, mask=mask, az=az, rg=rgi)


def report(a: dict, b: dict) -> dict:
    """tests' comparison of two outputs (b taken as the reference side)."""
    from oracle.compare import compare
    return compare(a["geo"], b["geo"], a["az"], b["az"], a["rg"], b["rg"], a["mask"], b["mask"])
