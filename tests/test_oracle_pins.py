"""Pins the CPU oracle against the reference's own known-answer data.

- tests/data/interpolator/data.txt of the reference (golden copy in
  tests/golden/interpolator_data.npz): bilinear to 1e-8, bicubic and
  biquintic MSE < 0.058,
  sinc MSE < 3e-4, nearest exact (tests/cxx/isce3/core/interpolator/
  interpolator.cpp:104-236).
- the circular-orbit Hermite KAT (tests/cxx/isce3/core/orbit/orbit.cpp:495-552),
  1e-8 m and m/s.
"""
from pathlib import Path

import numpy as np
import pytest

from isce3_gb300.core import LUT2d, Orbit, Poly2d

GOLD = Path(__file__).parent / "golden"


@pytest.fixture(scope="module")
def interp_case():
    data = np.load(GOLD / "interpolator_data.npz")["data"]
    idx = np.arange(-5.01, 5.01, 0.25)
    # arange as the reference builds it: repeated addition (interpolator.cpp:26-38)
    v, cur = [], -5.01
    while cur < 5.01:
        v.append(cur)
        cur += 0.25
    idx = np.array(v)
    M = np.sin(idx[:, None] ** 2 + idx[None, :] ** 2)
    return data, M, -5.01, 0.25


def test_bilinear_known_answer(oracle_mod, interp_case):
    data, M, start, delta = interp_case
    err = 0.0
    for row in data:
        x, y = (row[0] - start) / delta, (row[1] - start) / delta
        z = oracle_mod.interp2d(1, M, x, y)
        assert abs(z - row[2]) < 1e-8
        err += (z - row[5]) ** 2
    assert err / len(data) < 0.07


def test_nearest_known_answer(oracle_mod, interp_case):
    data, M, start, delta = interp_case
    for row in data:
        x, y = (row[0] - start) / delta, (row[1] - start) / delta
        assert oracle_mod.interp2d(3, M, x, y) == M[int(round(y)), int(round(x))]


def test_bicubic_known_answer(oracle_mod, interp_case):
    # interpolator.cpp:144-168: points at least one sample inside the left and
    # top edges and two inside the right and bottom ones
    data, M, start, delta = interp_case
    err = 0.0
    for r in data:
        x, y = (r[0] - start) / delta, (r[1] - start) / delta
        if x < 1 or y < 1 or x >= M.shape[1] - 2 or y >= M.shape[0] - 2:
            continue
        err += (oracle_mod.interp2d(2, M, x, y) - r[5]) ** 2
    assert err / len(data) < 0.058


def test_biquintic_known_answer(oracle_mod, interp_case):
    data, M, start, delta = interp_case
    err = sum((oracle_mod.interp2d(4, M, (r[0] - start) / delta, (r[1] - start) / delta) - r[5]) ** 2 for r in data)
    assert err / len(data) < 0.058


def test_sinc_known_answer(oracle_mod, interp_case):
    data, M, start, delta = interp_case
    err, n = 0.0, 0
    for r in data:
        x, y = (r[0] - start) / delta, (r[1] - start) / delta
        if x < 3 or y < 3 or x > M.shape[1] - 5 or y > M.shape[0] - 5:
            continue
        err += (oracle_mod.interp2d(5, M, x, y) - r[5]) ** 2
        n += 1
    assert n > 50 and err / n < 3e-4


def test_spline_float_matches_double_order(oracle_mod, interp_case):
    # the FP32 spline the DEM uses stays within FP32 rounding of the FP64 one
    data, M, start, delta = interp_case
    Mf = M.astype(np.float32)
    for r in data[:50]:
        x, y = (r[0] - start) / delta, (r[1] - start) / delta
        zf = oracle_mod.spline2d_float(Mf, x, y)
        zd = oracle_mod.interp2d(4, Mf.astype(np.float64), x, y)
        assert abs(zf - zd) < 1e-5


class _Circ:
    """tests/cxx/isce3/core/orbit/orbit.cpp CircularOrbit (analytic)."""

    def __init__(self, theta0, phi0, dtheta, dphi, r):
        self.t0, self.p0, self.dt, self.dp, self.r = theta0, phi0, dtheta, dphi, r

    def position(self, t):
        th, ph = self.t0 + t * self.dt, self.p0 + t * self.dp
        return np.array([self.r * np.cos(th), self.r * (np.sin(th) + np.cos(ph)), self.r * np.sin(ph)])

    def velocity(self, t):
        th, ph = self.t0 + t * self.dt, self.p0 + t * self.dp
        return np.array([-self.r * self.dt * np.sin(th), self.r * (self.dt * np.cos(th) - self.dp * np.sin(ph)),
                         self.r * self.dp * np.cos(ph)])


def _circular_orbit():
    ref = _Circ(2 * np.pi / 8, 2 * np.pi / 12, 2 * np.pi / 7000, 2 * np.pi / 4000, 8000000.0)
    t = np.arange(11) * 5.0
    pos = np.array([ref.position(x) for x in t])
    vel = np.array([ref.velocity(x) for x in t])
    return ref, Orbit.from_arrays(0.0, 5.0, pos, vel)


def test_circular_orbit_hermite_known_answer(oracle_mod):
    ref, orbit = _circular_orbit()
    for t in (11.65, 18.35, 27.25, 44.65):
        pos, vel, st = oracle_mod.orbit_interpolate(orbit, t)
        assert st == 0
        assert np.all(np.abs(pos - ref.position(t)) < 1e-8)
        assert np.all(np.abs(vel - ref.velocity(t)) < 1e-8)


def test_orbit_outside_span_is_nan(oracle_mod):
    _, orbit = _circular_orbit()
    pos, vel, st = oracle_mod.orbit_interpolate(orbit, 60.0)
    assert st != 0 and np.all(np.isnan(pos)) and np.all(np.isnan(vel))


def test_lut2d_eval_and_contains(oracle_mod):
    data = np.arange(12, dtype=np.float64).reshape(3, 4) ** 1.5
    lut = LUT2d(10.0, 100.0, 2.0, 0.5, data)
    for y, x in [(100.0, 10.0), (100.3, 13.1), (101.0, 16.0), (99.0, 9.0), (102.0, 20.0)]:
        # clamp + bilinear (core/LUT2d.cpp:139-157)
        xi = min(max((x - 10.0) / 2.0, 0.0), 3.0)
        yi = min(max((y - 100.0) / 0.5, 0.0), 2.0)
        x1, x2, y1, y2 = int(np.floor(xi)), int(np.ceil(xi)), int(np.floor(yi)), int(np.ceil(yi))
        fx, fy = xi - x1, yi - y1
        want = (data[y1, x1] * (1 - fx) * (1 - fy) + data[y1, x2] * fx * (1 - fy) + data[y2, x1] * (1 - fx) * fy
                + data[y2, x2] * fx * fy)
        assert abs(oracle_mod.lut_eval(lut, y, x) - want) < 1e-9
        assert lut.contains(y, x) == (10.0 <= x <= 16.0 and 100.0 <= y <= 101.0)
    assert oracle_mod.lut_eval(LUT2d(), 1.0, 2.0) == 0.0
    assert LUT2d().contains(1e9, -1e9)


def test_poly2d_matches_python(oracle_mod):
    p = Poly2d(np.array([[1.0, 2.0, -0.5], [0.25, 3.0, 0.0]]), x_mean=5.0, y_mean=-1.0, x_std=2.0, y_std=4.0)
    for y, x in [(0.0, 0.0), (3.0, 7.0), (-10.0, 1e3)]:
        assert oracle_mod.poly_eval(p, y, x) == p.eval(y, x)
    assert oracle_mod.poly_eval(Poly2d(), 3.0, 4.0) == 0.0


def test_oracle_regression_golden(oracle_mod):
    """The oracle reproduces its committed output on a small seeded scene."""
    from isce3_gb300 import synth
    gold = np.load(GOLD / "oracle_c1_small.npz")
    sc = synth.scene_c1(seed=7, length=256, width=256, geo=128, dem_px=128)
    g = sc.geogrid
    geo = np.zeros((g.length, g.width), np.complex64)
    mask = np.zeros((g.length, g.width), np.uint8)
    oracle_mod.geocode_slc(geo, sc.slc, sc.dem, sc.radar_grid, g, sc.orbit, sc.native_doppler,
                           sc.image_grid_doppler, sc.ellipsoid, sc.threshold, sc.maxiter, mask_block=mask)
    np.testing.assert_array_equal(mask, gold["mask"])
    np.testing.assert_array_equal(np.isnan(geo), np.isnan(gold["geo"]))
    v = np.isfinite(geo)
    assert np.max(np.abs(geo[v] - gold["geo"][v])) <= 1e-6


@pytest.mark.parametrize("method,code", [("sinc", 0), ("bilinear", 1), ("bicubic", 2), ("nearest", 3),
                                         ("biquintic", 4)])
def test_lut2d_methods_use_their_interpolator(oracle_mod, interp_case, method, code):
    # core/LUT2d.cpp:124-158 and _setInterpolator: the coordinates are
    # clamped to the table, then the method's interpolator runs on them
    _, M, _, _ = interp_case
    lut = LUT2d(-3.0, 7.0, 0.5, 0.25, M, method)
    interp_code = {0: 5, 1: 1, 2: 2, 3: 3, 4: 4}[code]
    rng = np.random.default_rng(5)
    for _ in range(200):
        x = -3.0 + rng.uniform(-2.0, 0.5 * M.shape[1] + 2.0)
        y = 7.0 + rng.uniform(-1.0, 0.25 * M.shape[0] + 1.0)
        xi = min(max((x + 3.0) / 0.5, 0.0), M.shape[1] - 1.0)
        yi = min(max((y - 7.0) / 0.25, 0.0), M.shape[0] - 1.0)
        if code == 2 and not (1 <= xi < M.shape[1] - 2 and 1 <= yi < M.shape[0] - 2):
            continue   # the reference's bicubic reads outside the table there
        assert oracle_mod.lut_eval(lut, y, x) == oracle_mod.interp2d(interp_code, M, xi, yi)
