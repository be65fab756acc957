"""The oracle's geometry against the reference's own source, bit for bit.

oracle/ref.py compiles the reference's geo2rdr (geometry/detail/Geo2Rdr.icc,
called as geometry/geometry.cpp:241-251 does for geocodeSlc.cpp:120-123),
Hermite and Legendre orbit interpolation (core/detail/InterpolateOrbit.icc:
10-155, core/Linspace.icc:77-89), the 2-D interpolators (core/Bilinear,
Bicubic, NearestNeighbor, Spline2d and Sinc2dInterpolator.cpp), Ellipsoid::lonLatToXyz (core/Ellipsoid.h:177-190)
and UTM::inverse / forward (core/Projections.cpp:171-232) where they lie in
the reference checkout.  The oracle's restatement of each must return the
same bits on the same inputs: these are the functions whose rounding decides
the sinc-table rows and Newton stops the parity checker classifies.

Skipped where the reference checkout is not mounted.
"""
import numpy as np
import pytest

from isce3_gb300 import synth
from isce3_gb300.core import LUT2d

from oracle import ref

pytestmark = pytest.mark.skipif(not ref.available(), reason="reference checkout not mounted")


@pytest.fixture(scope="module", params=["c1", "c2"])
def scene(request):
    if request.param == "c1":
        return synth.scene_c1(seed=1, slc=False)
    return synth.scene_c2(seed=2, length=16384, width=8192, geo=64, slc=False, dem_arcsec=30.0)


def _ground_points(sc, m, seed):
    """llh (rad, rad, m) spread over the geogrid's footprint, 0-3000 m high."""
    rng = np.random.default_rng(seed)
    g = sc.geogrid
    x = g.start_x + g.spacing_x * rng.uniform(0, g.width, m)
    y = g.start_y + g.spacing_y * rng.uniform(0, g.length, m)
    if g.epsg == 4326:
        lon, lat = np.radians(x), np.radians(y)
    else:
        ll, bad = ref.utm_inverse(g.epsg, np.stack([x, y], 1))
        assert bad == 0
        lon, lat = ll[:, 0], ll[:, 1]
    return np.stack([lon, lat, rng.uniform(0.0, 3000.0, m)], 1)


def test_orbit_interpolation_bits(oracle_mod, scene):
    o = scene.orbit
    span = o.spacing * (o.size - 1)
    t = np.concatenate([np.linspace(o.t0 - 2.0, o.t0 + span + 2.0, 4001), o.t0 + o.spacing * np.arange(o.size)])
    P, V = ref.orbit_interpolate(o, t)
    for k in range(t.size):
        po, vo, _st = oracle_mod.orbit_interpolate(o, t[k])
        np.testing.assert_array_equal(po, P[k])
        np.testing.assert_array_equal(vo, V[k])


def _legendre(o):
    from isce3_gb300.core import Orbit, OrbitInterpMethod
    return Orbit.from_arrays(o.t0, o.spacing, o.position, o.velocity, o.reference_epoch, OrbitInterpMethod.LEGENDRE)


def test_legendre_orbit_interpolation_bits(oracle_mod, scene):
    """core/detail/InterpolateOrbit.icc:111-155: the 9-point Lagrange form,
    including the state-vector times where it returns the vectors as they
    are."""
    o = _legendre(scene.orbit)
    span = o.spacing * (o.size - 1)
    t = np.concatenate([np.linspace(o.t0 - 2.0, o.t0 + span + 2.0, 4001), o.t0 + o.spacing * np.arange(o.size)])
    P, V = ref.orbit_interpolate(o, t)
    for k in range(t.size):
        po, vo, _st = oracle_mod.orbit_interpolate(o, t[k])
        np.testing.assert_array_equal(po, P[k])
        np.testing.assert_array_equal(vo, V[k])


def test_legendre_geo2rdr_bits(oracle_mod, scene):
    rg = scene.radar_grid
    o = _legendre(scene.orbit)
    llh = _ground_points(scene, 1500, 9)
    t, r, st = ref.geo2rdr(llh, scene.ellipsoid, o, rg.wavelength, int(rg.lookside), rg.sensing_mid,
                           scene.threshold, scene.maxiter, 1e-8)
    assert (st == 0).sum() > 0.9 * len(llh)
    for k in range(len(llh)):
        to, ro, ok = oracle_mod.geo2rdr(llh[k], scene.ellipsoid, o, LUT2d(), rg.wavelength, int(rg.lookside),
                                        rg.sensing_mid, scene.threshold, scene.maxiter, 1e-8)
        assert bool(ok) == (st[k] == 0), k
        if ok:
            assert to == t[k] and ro == r[k], (k, to - t[k], ro - r[k])


def test_lonlat_to_xyz_bits(oracle_mod, scene):
    llh = _ground_points(scene, 2000, 3)
    xyz = ref.lonlat_to_xyz(scene.ellipsoid, llh)
    for k in range(len(llh)):
        out = np.zeros(3)
        oracle_mod.lib().orc_lonlat_to_xyz(scene.ellipsoid.a, scene.ellipsoid.e2, np.ascontiguousarray(llh[k]).ctypes.data,
                                           out.ctypes.data)
        np.testing.assert_array_equal(out, xyz[k])


@pytest.mark.parametrize("doppler", [0.0, 37.5])
def test_geo2rdr_bits(oracle_mod, scene, doppler):
    """t, r and convergence identical, from sensingMid with deltaRange 1e-8
    (geocodeSlc's call), for a zero and a constant image-grid Doppler."""
    rg = scene.radar_grid
    llh = _ground_points(scene, 4000, 5)
    t, r, st = ref.geo2rdr(llh, scene.ellipsoid, scene.orbit, rg.wavelength, int(rg.lookside), rg.sensing_mid,
                           scene.threshold, scene.maxiter, 1e-8, doppler)
    dop = LUT2d()
    dop.ref_value = doppler
    assert (st == 0).sum() > 0.9 * len(llh)
    for k in range(len(llh)):
        to, ro, ok = oracle_mod.geo2rdr(llh[k], scene.ellipsoid, scene.orbit, dop, rg.wavelength, int(rg.lookside),
                                        rg.sensing_mid, scene.threshold, scene.maxiter, 1e-8)
        assert bool(ok) == (st[k] == 0), k
        if ok:
            assert to == t[k] and ro == r[k], (k, to - t[k], ro - r[k])


def test_geo2rdr_outside_orbit_start_bits(oracle_mod):
    """A start guess outside the orbit takes the coarse search
    (Geo2Rdr.icc:50-112) on both sides."""
    sc = synth.scene_c1(seed=1, slc=False)
    rg = sc.radar_grid
    llh = _ground_points(sc, 300, 7)
    t_out = sc.orbit.t0 - 50.0
    t, r, st = ref.geo2rdr(llh, sc.ellipsoid, sc.orbit, rg.wavelength, int(rg.lookside), t_out, 1e-8, 50, 10.0)
    for k in range(len(llh)):
        to, ro, ok = oracle_mod.geo2rdr(llh[k], sc.ellipsoid, sc.orbit, LUT2d(), rg.wavelength, int(rg.lookside),
                                        t_out, 1e-8, 50, 10.0)
        assert bool(ok) == (st[k] == 0)
        if ok:
            assert to == t[k] and ro == r[k]


@pytest.mark.parametrize("epsg", [32611, 32601, 32660, 32733, 32718])
def test_utm_bits(oracle_mod, epsg):
    rng = np.random.default_rng(epsg)
    m = 3000
    xy = np.stack([rng.uniform(2.0e5, 8.0e5, m), rng.uniform(1.0e5, 9.3e6, m)], 1)
    ll, bad = ref.utm_inverse(epsg, xy)
    assert bad == 0
    back, bad = ref.utm_forward(epsg, ll)
    assert bad == 0
    for k in range(m):
        lon, lat, st = oracle_mod.proj_inverse(epsg, xy[k, 0], xy[k, 1])
        assert st == 0 and lon == ll[k, 0] and lat == ll[k, 1]
        x, y, st = oracle_mod.proj_forward(epsg, ll[k, 0], ll[k, 1])
        assert st == 0 and x == back[k, 0] and y == back[k, 1]


# ---- the 2-D interpolators ----
# the oracle's numbering of interp2d (1 bilinear, 2 bicubic, 3 nearest,
# 4 biquintic, 5 sinc) against isce3's dataInterpMethod
_ISCE3_METHOD = {1: 1, 2: 2, 3: 3, 4: 4, 5: 0}


def _points(ny, nx, m, seed, lo=0.0):
    rng = np.random.default_rng(seed)
    x = rng.uniform(lo, nx - 1 - lo, m)
    y = rng.uniform(lo, ny - 1 - lo, m)
    # node coordinates and exact halves as well
    x[:40] = np.floor(x[:40])
    y[40:80] = np.floor(y[40:80]) + 0.5
    return x, y


@pytest.mark.parametrize("ora_method", [1, 2, 3, 4, 5])
def test_interp2d_double_bits(oracle_mod, ora_method):
    """LUT2d's interpolators on doubles, over the interior (the bicubic reads
    one sample outside its cell, so it stays one sample inside the table)."""
    rng = np.random.default_rng(ora_method)
    z = rng.normal(size=(37, 41)) * 50.0 + np.linspace(0, 30, 41)[None, :]
    lo = 1.0 if ora_method == 2 else 0.0
    x, y = _points(37, 41 - (2 if ora_method == 2 else 0), 2000, 11 + ora_method, lo)
    for k in range(x.size):
        want = ref.interp2d(_ISCE3_METHOD[ora_method], z, x[k], y[k])
        assert oracle_mod.interp2d(ora_method, z, x[k], y[k]) == want, (k, x[k], y[k])


def test_dem_spline_float_bits(oracle_mod):
    """Spline2dInterpolator<float> of order 6, the DEM's interpolator, on a
    float table (edges included: its window clamps there)."""
    rng = np.random.default_rng(3)
    z = (rng.normal(size=(48, 52)) * 300.0 + 1500.0).astype(np.float32)
    x, y = _points(48, 52, 3000, 4)
    for k in range(x.size):
        want = ref.spline2d_float(z, x[k], y[k])
        got = oracle_mod.spline2d_float(z, x[k], y[k])
        assert got.view(np.uint32) == want.view(np.uint32), (k, x[k], y[k])


def test_sinc_complex64_bits(oracle_mod):
    """Sinc2dInterpolator<complex<float>>, the SLC interpolator of
    geocodeSlc.cpp:476-494, on 9 x 9 chips and on a larger table."""
    rng = np.random.default_rng(5)
    for shape, m in (((9, 9), 400), ((30, 33), 1500)):
        z = (rng.normal(size=shape) + 1j * rng.normal(size=shape)).astype(np.complex64)
        x, y = _points(shape[0], shape[1], m, 6 + m)
        for k in range(x.size):
            want = ref.sinc2d_cfloat(z, x[k], y[k])
            got = oracle_mod.sinc2d_cfloat(z, x[k], y[k])
            assert np.array([got]).view(np.uint64)[0] == np.array([want]).view(np.uint64)[0], (k, x[k], y[k])


@pytest.mark.parametrize("method", ["sinc", "bilinear", "bicubic", "nearest", "biquintic"])
def test_lut2d_eval_bits(oracle_mod, method):
    """LUT2d<double>::eval (core/LUT2d.cpp:124-158): index, clamp to the
    table, the method's interpolator; points inside and outside the table
    (the bicubic only where its 4 x 4 reads stay in the table)."""
    rng = np.random.default_rng(21)
    data = rng.normal(size=(24, 30)) * 20.0
    lut = LUT2d(-3.0, 7.0, 0.5, 0.25, data, method)
    for _ in range(1500):
        x = -3.0 + rng.uniform(-2.0, 0.5 * 29 + 2.0)
        y = 7.0 + rng.uniform(-1.0, 0.25 * 23 + 1.0)
        if method == "bicubic":
            xi = min(max((x + 3.0) / 0.5, 0.0), 29.0)
            yi = min(max((y - 7.0) / 0.25, 0.0), 23.0)
            if not (1 <= xi < 27 and 1 <= yi < 21):
                continue
        assert oracle_mod.lut_eval(lut, y, x) == ref.lut2d_eval(lut, y, x), (x, y)


def test_poly2d_eval_bits(oracle_mod):
    """Poly2d::eval (core/Poly2d.cpp:8-24): the carriers' polynomials."""
    from isce3_gb300.core import Poly2d
    rng = np.random.default_rng(22)
    for xo, yo in ((0, 0), (1, 0), (0, 1), (2, 3), (4, 2)):
        p = Poly2d(rng.normal(size=(yo + 1, xo + 1)) * 10.0, x_mean=850e3, y_mean=100.0, x_std=3e3, y_std=5.0)
        for _ in range(300):
            x, y = rng.uniform(8.4e5, 8.7e5), rng.uniform(90.0, 110.0)
            assert oracle_mod.poly_eval(p, y, x) == ref.poly2d_eval(p, y, x), (xo, yo, x, y)
