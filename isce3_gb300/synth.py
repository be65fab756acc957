"""Seeded synthetic SAR scenes for the geocoding workloads.

No public dataset is named for the SLC geocoding path, so scenes are built
here: a circular near-polar orbit sampled as ECEF state vectors (with Earth
rotation), a zero-Doppler radar grid, a fractal (fBm) DEM, a complex Gaussian
SLC with point targets, Doppler and carrier models, and a geogrid covering
the swath.  Everything is numpy and deterministic in ``seed``.
"""
from __future__ import annotations

from types import SimpleNamespace

import numpy as np

from .core import (DateTime, Ellipsoid, LookSide, LUT2d, Orbit, Poly2d, EARTH_SEMI_MAJOR_AXIS)
from .io import Raster
from .product import GeoGridParameters, RadarGridParameters

GM = 3.986004418e14
EARTH_SPIN = 7.292115024135738e-5     # cxx/isce3/core/Constants.h:47
EPOCH = DateTime(2026, 1, 1, 0, 0, 0.0)


class CircularOrbitModel:
    """Circular orbit in inertial space, expressed in the rotating ECEF frame."""

    def __init__(self, altitude=747e3, inclination_deg=98.0, t_ref=0.0, lat0_deg=35.0, lon0_deg=-121.5,
                 ascending=True):
        self.r = EARTH_SEMI_MAJOR_AXIS + altitude
        self.n = np.sqrt(GM / self.r ** 3)
        self.inc = np.radians(inclination_deg)
        self.t_ref = t_ref
        s = np.sin(np.radians(lat0_deg)) / np.sin(self.inc)
        u0 = np.arcsin(np.clip(s, -1, 1))
        if not ascending:
            u0 = np.pi - u0
        self.u0 = u0
        x, y, _ = self._eci_unit(u0)
        lon_eci = np.arctan2(y, x)
        self.theta0 = lon_eci - np.radians(lon0_deg)

    def _eci_unit(self, u):
        ci, si = np.cos(self.inc), np.sin(self.inc)
        return np.cos(u), np.sin(u) * ci, np.sin(u) * si

    def state(self, t):
        t = np.asarray(t, dtype=np.float64)
        u = self.u0 + self.n * (t - self.t_ref)
        ux, uy, uz = self._eci_unit(u)
        pe = self.r * np.stack([ux, uy, uz], axis=-1)
        ci, si = np.cos(self.inc), np.sin(self.inc)
        ve = self.r * self.n * np.stack([-np.sin(u), np.cos(u) * ci, np.cos(u) * si], axis=-1)
        th = self.theta0 + EARTH_SPIN * (t - self.t_ref)
        c, s = np.cos(th), np.sin(th)
        px = c * pe[..., 0] + s * pe[..., 1]
        py = -s * pe[..., 0] + c * pe[..., 1]
        pz = pe[..., 2]
        vx = c * ve[..., 0] + s * ve[..., 1] + EARTH_SPIN * py
        vy = -s * ve[..., 0] + c * ve[..., 1] - EARTH_SPIN * px
        vz = ve[..., 2]
        return np.stack([px, py, pz], axis=-1), np.stack([vx, vy, vz], axis=-1)

    def orbit(self, t_mid, n=21, spacing=10.0) -> Orbit:
        t0 = t_mid - spacing * (n - 1) / 2
        times = np.array([t0 + i * spacing for i in range(n)])
        pos, vel = self.state(times)
        return Orbit.from_arrays(t0, spacing, pos, vel, reference_epoch=EPOCH)


def rdr2geo(model: CircularOrbitModel, t, r, side: int, height=0.0, ell: Ellipsoid | None = None, iters=12):
    """Ground point at zero Doppler for azimuth time(s) t and slant range(s) r.

    Solves |X - S(t)| = r, (X - S)·V = 0 and h(X) = height by Newton on the
    look angle in the zero-Doppler plane.  Returns lon, lat (rad), h (m).
    """
    ell = ell or Ellipsoid()
    t = np.asarray(t, dtype=np.float64)
    r = np.asarray(r, dtype=np.float64)
    t, r = np.broadcast_arrays(t, r)
    height = np.broadcast_to(np.asarray(height, dtype=np.float64), t.shape)
    S, V = model.state(t)
    vhat = V / np.linalg.norm(V, axis=-1, keepdims=True)
    down = -S / np.linalg.norm(S, axis=-1, keepdims=True)
    e1 = down - np.sum(down * vhat, axis=-1, keepdims=True) * vhat
    e1 /= np.linalg.norm(e1, axis=-1, keepdims=True)
    right = np.cross(e1, vhat)
    e2 = right if side == int(LookSide.Right) else -right
    # initial look angle from a sphere
    Rs = np.linalg.norm(S, axis=-1)
    Re = ell.a
    cosl = np.clip((Rs ** 2 + r ** 2 - (Re + height) ** 2) / (2 * Rs * r), -1, 1)
    th = np.arccos(cosl)
    for _ in range(iters):
        X = S + r[..., None] * (np.cos(th)[..., None] * e1 + np.sin(th)[..., None] * e2)
        h = ell.xyz_to_lon_lat(X)[..., 2]
        dth = 1e-7
        X2 = S + r[..., None] * (np.cos(th + dth)[..., None] * e1 + np.sin(th + dth)[..., None] * e2)
        h2 = ell.xyz_to_lon_lat(X2)[..., 2]
        th = th - (h - height) / ((h2 - h) / dth)
    X = S + r[..., None] * (np.cos(th)[..., None] * e1 + np.sin(th)[..., None] * e2)
    llh = ell.xyz_to_lon_lat(X)
    return llh[..., 0], llh[..., 1], llh[..., 2]


def fbm_surface(shape, hurst, rng: np.random.Generator, lo=0.0, hi=1500.0) -> np.ndarray:
    """Fractional Brownian surface by spectral synthesis, scaled to [lo, hi]."""
    ny, nx = shape
    ky = np.fft.fftfreq(ny)[:, None]
    kx = np.fft.rfftfreq(nx)[None, :]
    k = np.sqrt(kx ** 2 + ky ** 2)
    k[0, 0] = 1.0
    amp = k ** (-(hurst + 1.0))
    amp[0, 0] = 0.0
    phase = rng.uniform(0, 2 * np.pi, size=amp.shape)
    spec = amp * rng.standard_normal(amp.shape) * np.exp(1j * phase)
    z = np.fft.irfft2(spec, s=shape)
    z = (z - z.min()) / (z.max() - z.min())
    return (lo + (hi - lo) * z).astype(np.float32)


def complex_gaussian(shape, rng: np.random.Generator, block_rows=2048) -> np.ndarray:
    """Circular complex Gaussian, unit variance, complex64 (row blocks bound memory)."""
    out = np.empty(shape, dtype=np.complex64)
    s = np.float32(np.sqrt(0.5))
    for i in range(0, shape[0], block_rows):
        n = min(block_rows, shape[0] - i)
        re = rng.standard_normal((n, shape[1]), dtype=np.float32)
        im = rng.standard_normal((n, shape[1]), dtype=np.float32)
        out[i:i + n].real = re * s
        out[i:i + n].imag = im * s
    return out


def _swath_bounds(model, grid: RadarGridParameters, h, n=9):
    ts = np.linspace(grid.sensing_start, grid.sensing_stop, n)
    rs = np.linspace(grid.starting_range, grid.end_range, n)
    T, R = np.meshgrid(ts, rs, indexing="ij")
    lon, lat, _ = rdr2geo(model, T.ravel(), R.ravel(), int(grid.lookside), h)
    return np.degrees(lon), np.degrees(lat)


def lonlat_geogrid(lon_deg, lat_deg, width, length, pad=0.02) -> GeoGridParameters:
    x0, x1 = lon_deg.min(), lon_deg.max()
    y0, y1 = lat_deg.min(), lat_deg.max()
    px, py = pad * (x1 - x0), pad * (y1 - y0)
    x0, x1, y0, y1 = x0 - px, x1 + px, y0 - py, y1 + py
    return GeoGridParameters(x0, y1, (x1 - x0) / width, -(y1 - y0) / length, width, length, 4326)


def lonlat_dem(geogrid_lonlat_bounds, shape, rng, hurst, hmax, margin_px=60) -> Raster:
    """fBm DEM in EPSG:4326 covering the bounds plus ``margin_px`` pixels."""
    x0, x1, y0, y1 = geogrid_lonlat_bounds
    ny, nx = shape
    dx = (x1 - x0) / (nx - 2 * margin_px)
    dy = (y1 - y0) / (ny - 2 * margin_px)
    gt = [x0 - margin_px * dx, dx, 0.0, y1 + margin_px * dy, 0.0, -dy]
    return Raster(fbm_surface(shape, hurst, rng, 0.0, hmax), gt, 4326)


def scene_c1(seed: int = 1, length=1024, width=1024, geo=512, dem_px=256, n_targets=16, slc=True):
    """1024 x 1024 SLC onto a 512 x 512 EPSG:4326 geogrid, zero Doppler."""
    rng = np.random.default_rng(seed)
    model = CircularOrbitModel(lat0_deg=35.0, lon0_deg=-121.5)
    prf, dr, r0, wvl = 1520.0, 6.25, 850e3, 0.24
    t_start = 100.0
    grid = RadarGridParameters(t_start, wvl, prf, r0, dr, LookSide.Right, length, width, EPOCH)
    orbit = model.orbit(grid.sensing_mid, 21, 10.0)
    lon, lat = _swath_bounds(model, grid, 750.0)
    geogrid = lonlat_geogrid(lon, lat, geo, geo)
    bounds = (geogrid.start_x, geogrid.end_x, geogrid.end_y, geogrid.start_y)
    dem = lonlat_dem(bounds, (dem_px, dem_px), rng, 0.8, 1500.0, margin_px=min(60, dem_px // 4))
    data = None
    if slc:
        data = complex_gaussian((length, width), rng)
        ia = rng.integers(8, length - 8, n_targets)
        ir = rng.integers(8, width - 8, n_targets)
        data[ia, ir] += np.complex64(1.0)
    return SimpleNamespace(name="c1", seed=seed, model=model, radar_grid=grid, orbit=orbit, geogrid=geogrid,
                           dem=dem, slc=data, native_doppler=LUT2d(), image_grid_doppler=LUT2d(),
                           az_carrier=LUT2d(), rg_carrier=LUT2d(), ellipsoid=Ellipsoid(),
                           threshold=1e-8, maxiter=25)


def _utm_grid_around(lon_c, lat_c, epsg, width, length, spacing):
    """UTM geogrid of width x length pixels centred on (lon_c, lat_c) in degrees."""
    x, y = utm_forward_host(epsg, np.radians(lon_c), np.radians(lat_c))
    x0 = np.floor((x - spacing * width / 2) / spacing) * spacing
    y1 = np.ceil((y + spacing * length / 2) / spacing) * spacing
    return GeoGridParameters(x0, y1, spacing, -spacing, width, length, epsg)


def utm_forward_host(epsg, lon, lat):
    """UTM forward (Krueger n-series, 6 terms) in numpy, for scene layout only."""
    zone = epsg - 32600 if epsg < 32700 else epsg - 32700
    north = epsg < 32700
    a, e2 = Ellipsoid().a, Ellipsoid().e2
    f = e2 / (1 + np.sqrt(1 - e2))
    n = f / (2 - f)
    lon0 = (zone - 0.5) * (np.pi / 30) - np.pi
    A = a / (1 + n) * (1 + n ** 2 / 4 + n ** 4 / 64)
    al = [n / 2 - 2 * n ** 2 / 3 + 5 * n ** 3 / 16, 13 * n ** 2 / 48 - 3 * n ** 3 / 5, 61 * n ** 3 / 240]
    e = np.sqrt(e2)
    t = np.sinh(np.arctanh(np.sin(lat)) - e * np.arctanh(e * np.sin(lat)))
    xi = np.arctan2(t, np.cos(lon - lon0))
    eta = np.arctanh(np.sin(lon - lon0) / np.sqrt(1 + t ** 2))
    xs = xi + sum(al[j] * np.sin(2 * (j + 1) * xi) * np.cosh(2 * (j + 1) * eta) for j in range(3))
    es = eta + sum(al[j] * np.cos(2 * (j + 1) * xi) * np.sinh(2 * (j + 1) * eta) for j in range(3))
    return 500000 + 0.9996 * A * es, (0 if north else 10000000) + 0.9996 * A * xs


def scene_c2(seed: int = 2, length=16384, width=8192, geo=8000, spacing=10.0, dem_arcsec=1.0, slc=True,
             epsg=32611, geo_length=None, lat0_deg=35.0, lon0_deg=-121.8, ascending=True,
             look_side=LookSide.Right):
    """Frame-scale scene: 16384 x 8192 SLC onto an 8000 x 8000 UTM 10 m grid.

    Native Doppler: 32 x 32 LUT2d, quadratic in range, +-50 Hz; azimuth carrier:
    linear Poly2d; DEM: EPSG:4326 fBm at ``dem_arcsec`` arc-seconds, 0-3000 m.
    The orbit passes (``lat0_deg``, ``lon0_deg``) ascending or descending and
    the radar looks to ``look_side``; ``epsg`` must hold the swath (326zz
    north, 327zz south).
    """
    rng = np.random.default_rng(seed)
    model = CircularOrbitModel(lat0_deg=lat0_deg, lon0_deg=lon0_deg, ascending=ascending)
    prf, dr, r0, wvl = 1520.0, 6.25, 850e3, 0.24
    grid = RadarGridParameters(100.0, wvl, prf, r0, dr, look_side, length, width, EPOCH)
    orbit = model.orbit(grid.sensing_mid, 21, 10.0)
    lon, lat = _swath_bounds(model, grid, 1500.0)
    lon_c, lat_c = lon.mean(), lat.mean()
    geo_length = geo if geo_length is None else geo_length
    geogrid = _utm_grid_around(lon_c, lat_c, epsg, geo, geo_length, spacing)
    # DEM covering the swath footprint (and so the geogrid window) with margin
    d = dem_arcsec / 3600.0
    x0, x1 = lon.min() - 0.15, lon.max() + 0.15
    y0, y1 = lat.min() - 0.15, lat.max() + 0.15
    nx, ny = int(np.ceil((x1 - x0) / d)), int(np.ceil((y1 - y0) / d))
    dem = Raster(fbm_surface((ny, nx), 0.8, rng, 0.0, 3000.0), [x0, d, 0.0, y1, 0.0, -d], 4326)
    # native Doppler: quadratic in range, +-50 Hz, 32 x 32 samples over grid + margin
    rr = np.linspace(grid.starting_range - 200 * dr, grid.end_range + 200 * dr, 32)
    tt = np.linspace(grid.sensing_start - 200 / prf, grid.sensing_stop + 200 / prf, 32)
    u = (rr - rr.mean()) / (rr.max() - rr.mean())
    dop = np.tile(-50.0 + 100.0 * u ** 2, (32, 1))
    native = LUT2d(rr, tt, dop)
    az_carrier = Poly2d([[0.0], [2 * np.pi * 300.0]], x_mean=0.0, y_mean=grid.sensing_mid, x_std=1.0, y_std=1.0)
    rg_carrier = Poly2d(np.zeros((1, 1)))
    data = complex_gaussian((length, width), rng) if slc else None
    return SimpleNamespace(name="c2", seed=seed, model=model, radar_grid=grid, orbit=orbit, geogrid=geogrid,
                           dem=dem, slc=data, native_doppler=native, image_grid_doppler=LUT2d(),
                           az_carrier=az_carrier, rg_carrier=rg_carrier, ellipsoid=Ellipsoid(),
                           threshold=1e-8, maxiter=25)


def kat_slc(scene, axis="x", height=0.0):
    """Known-answer SLC: exp(i * lon) (axis 'x') or exp(i * lat) (axis 'y') of
    each radar pixel's ground point at constant ``height``, the synthetic
    restatement of tests/cxx/isce3/geocode/geocodeSlc.cpp:332-405."""
    g = scene.radar_grid
    t = g.sensing_start + np.arange(g.length) / g.prf
    r = g.starting_range + np.arange(g.width) * g.range_pixel_spacing
    T, R = np.meshgrid(t, r, indexing="ij")
    lon, lat, _ = rdr2geo(scene.model, T, R, int(g.lookside), height)
    ang = lon if axis == "x" else lat
    return np.exp(1j * ang).astype(np.complex64)


def constant_dem_like(raster: Raster, value: float) -> Raster:
    return Raster(np.full_like(raster.data, np.float32(value)), raster.get_geotransform(), raster.get_epsg())


def scene_bursts(seed: int = 4, n_az: int = 9, n_sw: int = 3, grid_px: int = 12000, spacing: float = 10.0,
                 lines=(1200, 1800), samples=(16000, 24000), prf: float = 760.0, dem_arcsec: float = 1.0,
                 device=None, epsg: int = 32611):
    """TOPS-like burst set onto one shared UTM grid.

    ``n_sw`` subswaths x ``n_az`` bursts; burst sizes are seeded uniform in
    ``lines`` x ``samples``; C-band (0.0555 m), 2.33 m range spacing, PRF
    ``prf`` (760 Hz: nine nominal 1500-line bursts then span ~120 km of
    ground track); subswath starting ranges 16 km apart so three 46.6 km
    slant-range swaths cover the grid's width; a quadratic azimuth steering
    carrier per burst (Poly2d, 2000 Hz/s); zero Doppler; fBm DEM.  Each burst
    gets the window of the shared grid its footprint covers (plus margin) and
    complex64 Gaussian samples generated on ``device`` (torch, seeded).
    """
    import torch
    rng = np.random.default_rng(seed)
    model = CircularOrbitModel(lat0_deg=35.0, lon0_deg=-121.8)
    wvl, dr = 0.0555, 2.33
    n = n_az * n_sw
    L_b = rng.integers(lines[0], lines[1] + 1, n)
    W_b = rng.integers(samples[0], samples[1] + 1, n)
    t_burst = 1500.0 / prf
    t_first = 100.0
    mid_t = t_first + 0.5 * n_az * t_burst
    orbit = model.orbit(mid_t, 41, 10.0)
    grids = []
    for s in range(n_sw):
        for k in range(n_az):
            i = s * n_az + k
            grids.append(RadarGridParameters(t_first + k * t_burst, wvl, prf, 800e3 + s * 16e3, dr, LookSide.Right,
                                             int(L_b[i]), int(W_b[i]), EPOCH))
    # shared grid centred on the whole burst set
    corners = [_swath_bounds(model, g, 1500.0, n=3) for g in grids]
    lon_all = np.concatenate([c[0] for c in corners])
    lat_all = np.concatenate([c[1] for c in corners])
    geogrid = _utm_grid_around(lon_all.mean(), lat_all.mean(), epsg, grid_px, grid_px, spacing)
    d = dem_arcsec / 3600.0
    x0, x1 = lon_all.min() - 0.1, lon_all.max() + 0.1
    y0, y1 = lat_all.min() - 0.1, lat_all.max() + 0.1
    nx, ny = int(np.ceil((x1 - x0) / d)), int(np.ceil((y1 - y0) / d))
    dem = Raster(fbm_surface((ny, nx), 0.8, rng, 0.0, 3000.0), [x0, d, 0.0, y1, 0.0, -d], 4326)
    gen = torch.Generator(device=device if device is not None else "cpu")
    gen.manual_seed(seed)
    bursts = []
    for i, g in enumerate(grids):
        lon, lat = _swath_bounds(model, g, 1500.0, n=5)
        lo2, la2 = _swath_bounds(model, g, 0.0, n=5)
        lon, lat = np.concatenate([lon, lo2]), np.concatenate([lat, la2])
        ex, ny_ = utm_forward_host(epsg, np.radians(lon), np.radians(lat))
        c0 = int(np.floor((ex.min() - geogrid.start_x) / spacing)) - 8
        c1 = int(np.ceil((ex.max() - geogrid.start_x) / spacing)) + 8
        r0 = int(np.floor((geogrid.start_y - ny_.max()) / spacing)) - 8
        r1 = int(np.ceil((geogrid.start_y - ny_.min()) / spacing)) + 8
        c0, c1 = max(c0, 0), min(c1, geogrid.width)
        r0, r1 = max(r0, 0), min(r1, geogrid.length)
        if c1 <= c0 or r1 <= r0:
            continue
        window = geogrid[r0:r1, c0:c1]
        tm = g.sensing_mid
        carrier = Poly2d([[0.0], [0.0], [np.pi * 2000.0]], x_mean=0.0, y_mean=tm, x_std=1.0, y_std=1.0)
        slc = None
        if device is not None:
            slc = torch.randn((g.length, g.width), dtype=torch.complex64, device=device, generator=gen)
        bursts.append(SimpleNamespace(radar_grid=g, window=window, window_offset=(r0, c0), az_carrier=carrier,
                                      rg_carrier=Poly2d(np.zeros((1, 1))), slc=slc))
    return SimpleNamespace(name="bursts", seed=seed, model=model, orbit=orbit, geogrid=geogrid, dem=dem,
                           bursts=bursts, native_doppler=LUT2d(), image_grid_doppler=LUT2d(), ellipsoid=Ellipsoid(),
                           threshold=1e-8, maxiter=25, prf=prf)


def scene_serving(seed: int = 5, n_slc: int = 8, lines=(4096, 16384), samples=(4096, 12000), device=None,
                  epsg: int = 32611, dem_arcsec: float = 1.0):
    """Resident SLCs for the serving workload: ``n_slc`` complex64 Gaussian
    SLCs (seeded sizes in ``lines`` x ``samples``), each from its own pass
    (orbit shifted in longitude), with a native-Doppler LUT2d (quadratic in
    range, +-50 Hz) and a linear azimuth carrier, over one shared fBm DEM."""
    import torch
    rng = np.random.default_rng(seed)
    prf, dr, r0, wvl = 1520.0, 6.25, 850e3, 0.24
    slcs = []
    lon_all, lat_all = [], []
    for i in range(n_slc):
        model = CircularOrbitModel(lat0_deg=35.0 + 0.05 * i, lon0_deg=-121.8 + 0.12 * i)
        g = RadarGridParameters(100.0, wvl, prf, r0, dr, LookSide.Right, int(rng.integers(lines[0], lines[1] + 1)),
                                int(rng.integers(samples[0], samples[1] + 1)), EPOCH)
        orbit = model.orbit(g.sensing_mid, 21, 10.0)
        lon, lat = _swath_bounds(model, g, 1500.0, n=5)
        lon_all.append(lon)
        lat_all.append(lat)
        rr = np.linspace(g.starting_range - 200 * dr, g.end_range + 200 * dr, 32)
        tt = np.linspace(g.sensing_start - 200 / prf, g.sensing_stop + 200 / prf, 32)
        u = (rr - rr.mean()) / (rr.max() - rr.mean())
        dop = LUT2d(rr, tt, np.tile(-50.0 + 100.0 * u ** 2, (32, 1)))
        carrier = Poly2d([[0.0], [2 * np.pi * 300.0]], y_mean=g.sensing_mid)
        slcs.append(SimpleNamespace(key=i, model=model, radar_grid=g, orbit=orbit, native_doppler=dop,
                                    az_carrier=carrier, rg_carrier=Poly2d(np.zeros((1, 1))), lon=lon, lat=lat))
    lon_all, lat_all = np.concatenate(lon_all), np.concatenate(lat_all)
    d = dem_arcsec / 3600.0
    x0, x1 = lon_all.min() - 0.25, lon_all.max() + 0.25
    y0, y1 = lat_all.min() - 0.25, lat_all.max() + 0.25
    nx, ny = int(np.ceil((x1 - x0) / d)), int(np.ceil((y1 - y0) / d))
    dem = Raster(fbm_surface((ny, nx), 0.8, rng, 0.0, 3000.0), [x0, d, 0.0, y1, 0.0, -d], 4326)
    if device is not None:
        gen = torch.Generator(device=device)
        gen.manual_seed(seed)
        for s in slcs:
            s.slc = torch.randn(s.radar_grid.shape, dtype=torch.complex64, device=device, generator=gen)
    return SimpleNamespace(slcs=slcs, dem=dem, epsg=epsg, seed=seed)


def serving_trace(scene, n_requests: int = 300, rate_hz: float = 200.0, side=(256, 4096), spacing=(10.0, 30.0),
                  seed: int = 6):
    """Poisson arrivals of geocode requests: each picks a resident SLC, a
    square UTM geogrid of log-uniform side in ``side`` pixels and uniform
    spacing in ``spacing`` metres, centred at a random point of the SLC's
    footprint.  Returns (slc key, GeoGridParameters, arrival s) tuples."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate_hz, n_requests))
    out = []
    for k in range(n_requests):
        s = scene.slcs[int(rng.integers(len(scene.slcs)))]
        n = int(np.exp(rng.uniform(np.log(side[0]), np.log(side[1]))))
        sp = float(np.round(rng.uniform(*spacing), 1))
        f = rng.uniform(0.25, 0.75, 2)
        lon_c = s.lon.min() + f[0] * (s.lon.max() - s.lon.min())
        lat_c = s.lat.min() + f[1] * (s.lat.max() - s.lat.min())
        out.append((s.key, _utm_grid_around(lon_c, lat_c, scene.epsg, n, n, sp), float(t[k] - t[0])))
    return out
