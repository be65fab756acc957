"""Host side of the product: the C ABI loads and exports every declared
symbol, its host-only math matches the oracle, and argument validation raises
the reference's exceptions.  No GPU is used."""
import ctypes as C

import numpy as np
import pytest

from isce3_gb300 import _lib as L, _marshal as M, synth
from isce3_gb300.core import LUT2d, Poly2d
from isce3_gb300.geocode import geocode_slc


@pytest.fixture(scope="module")
def lib():
    L.build()
    return L.load()


def test_library_exports_declared_symbols(lib):
    declared = L.declared_symbols()
    assert len(declared) >= 9
    for name in declared:
        assert hasattr(lib, name), name
    assert b"sm_103a" in lib.gslc_version()


def test_orbit_polynomial_matches_reference_hermite(lib, oracle_mod):
    sc = synth.scene_c1(slc=False)
    o = sc.orbit
    d = M.orbit_desc(o)
    for t in np.linspace(o.start_time, o.end_time, 501):
        p, v = (C.c_double * 3)(), (C.c_double * 3)()
        assert lib.gslc_orbit_interpolate(C.byref(d), t, p, v) == 0
        po, vo, _ = oracle_mod.orbit_interpolate(o, t)
        # the polynomial form is the Hermite interpolant; both differ only by rounding
        assert np.abs(np.array(p[:]) - po).max() < 2e-8
        assert np.abs(np.array(v[:]) - vo).max() < 5e-9
    p, v = (C.c_double * 3)(), (C.c_double * 3)()
    assert lib.gslc_orbit_interpolate(C.byref(d), o.end_time + 1.0, p, v) == L.GSLC_EINVAL


def test_orbit_legendre_matches_oracle_bits(lib, oracle_mod):
    """Legendre orbits (core/detail/InterpolateOrbit.icc:111-155): the
    library interpolates the state vectors in the reference's operation
    order, so position and velocity equal the oracle's bit for bit; fewer
    than 9 state vectors are rejected."""
    from isce3_gb300.core import Orbit, OrbitInterpMethod
    o0 = synth.scene_c1(slc=False).orbit
    o = Orbit.from_arrays(o0.t0, o0.spacing, o0.position, o0.velocity, o0.reference_epoch, OrbitInterpMethod.LEGENDRE)
    d = M.orbit_desc(o)
    assert d.method == 1
    ts = np.concatenate([np.linspace(o.start_time, o.end_time, 701), o.t0 + o.spacing * np.arange(o.size)])
    for t in ts:
        p, v = (C.c_double * 3)(), (C.c_double * 3)()
        assert lib.gslc_orbit_interpolate(C.byref(d), t, p, v) == 0
        po, vo, st = oracle_mod.orbit_interpolate(o, t)
        assert st == 0
        np.testing.assert_array_equal(np.array(p[:]), po)
        np.testing.assert_array_equal(np.array(v[:]), vo)
    short = Orbit.from_arrays(o0.t0, o0.spacing, o0.position[:8], o0.velocity[:8], o0.reference_epoch,
                              OrbitInterpMethod.LEGENDRE)
    ds = M.orbit_desc(short)
    p, v = (C.c_double * 3)(), (C.c_double * 3)()
    assert lib.gslc_orbit_interpolate(C.byref(ds), short.t0 + 1.0, p, v) == L.GSLC_EINVAL


@pytest.mark.parametrize("which", ["c1", "c2"])
def test_zero_doppler_newton_matches_oracle(lib, oracle_mod, which):
    """The kernels' Newton iterations (segment tables: residual D.vel - H,
    step times G = 1/|vel|^2) against the oracle's geo2rdr
    (geometry/detail/Geo2Rdr.icc:114-179) from sensingMid, on random geogrid
    points at random heights: same convergence everywhere, and the same
    iterate except where the last step sits at the threshold."""
    sc = synth.scene_c2(slc=False) if which == "c2" else synth.scene_c1(slc=False)
    o, rg, g, ell = sc.orbit, sc.radar_grid, sc.geogrid, sc.ellipsoid
    d = M.orbit_desc(o)
    t_mid = rg.sensing_start + 0.5 * (rg.length - 1) / rg.prf
    rng = np.random.default_rng(7)
    n, splits, dts, drs = 1500, 0, [], []
    for _ in range(n):
        x = g.start_x + g.spacing_x * rng.uniform(-0.1, 1.1) * g.width
        y = g.start_y + g.spacing_y * rng.uniform(-0.1, 1.1) * g.length
        lon, lat, _h = oracle_mod.proj_inverse(g.epsg, x, y)
        llh = np.array([lon, lat, rng.uniform(0.0, 3000.0)])
        xyz = np.zeros(3)
        oracle_mod.lib().orc_lonlat_to_xyz(ell.a, ell.e2, llh.ctypes.data, xyz.ctypes.data)
        t0, r0, ok0 = oracle_mod.geo2rdr(llh, ell, o, LUT2d(), rg.wavelength, rg.lookside, t_mid, 1e-8, 50, 1e-8)
        t, r, cv = C.c_double(), C.c_double(), C.c_int32()
        assert lib.gslc_geo2rdr_zero_doppler(C.byref(d), xyz.ctypes.data, t_mid, int(rg.lookside), 1e-8, 50,
                                             C.byref(t), C.byref(r), C.byref(cv)) == 0
        assert bool(cv.value) == bool(ok0)
        if not ok0:
            assert np.isnan(t.value) and np.isnan(r.value)
            continue
        if abs(t.value - t0) > 1e-9:      # stopped one iterate apart (|dt| at the threshold)
            splits += 1
            assert abs(t.value - t0) < 1e-8
            continue
        dts.append(abs(t.value - t0))
        drs.append(abs(r.value - r0))
    assert splits <= 0.01 * n
    # the oracle's Hermite formula carries ~1e-11 s / ~4e-9 m of rounding noise
    assert max(dts) < 5e-11 and max(drs) < 2e-8
    t, r, cv = C.c_double(), C.c_double(), C.c_int32()
    assert lib.gslc_geo2rdr_zero_doppler(C.byref(d), np.zeros(3).ctypes.data, t_mid, 0, 1e-8, 50,
                                         C.byref(t), C.byref(r), C.byref(cv)) == L.GSLC_EINVAL


def test_sinc_table_identical_to_oracle(lib, oracle_mod):
    tab = np.zeros((8192, 8), np.float32)
    assert lib.gslc_sinc_table(tab.ctypes.data) == 0
    np.testing.assert_array_equal(tab, oracle_mod.sinc_table())
    np.testing.assert_allclose(tab.astype(np.float64).sum(axis=1), 1.0, atol=1e-6)


@pytest.mark.parametrize("which", ["c1", "c2", "c1_tight"])
def test_dem_window_identical_to_oracle(lib, oracle_mod, which):
    sc = synth.scene_c2(slc=False) if which == "c2" else synth.scene_c1(slc=False)
    margin = 3 if which == "c1_tight" else 50
    d = L.DemRaster()
    d.width, d.length = sc.dem.width, sc.dem.length
    for i, v in enumerate(sc.dem.get_geotransform()):
        d.gt[i] = v
    d.epsg = sc.dem.get_epsg()
    w, g = L.DemWindow(), M.geo_grid_desc(sc.geogrid)
    assert lib.gslc_compute_dem_window(C.byref(d), C.byref(g), margin, C.byref(w)) == 0
    keep = oracle_mod._Keep()
    out = [C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64(), C.c_double(), C.c_double()]
    st = oracle_mod.lib().orc_dem_subset(C.byref(oracle_mod.dem_struct(sc.dem, keep)),
                                         C.byref(oracle_mod.geo_struct(sc.geogrid)), margin,
                                         *[C.addressof(x) for x in out])
    assert st == 0
    assert (w.x_off, w.y_off, w.width, w.length) == tuple(x.value for x in out[:4])
    assert w.x_start == out[4].value and w.y_start == out[5].value   # bit-exact


def _args(sc):
    return (sc.dem, sc.radar_grid, sc.geogrid, sc.orbit, LUT2d(), LUT2d(), sc.ellipsoid, 1e-8, 25)


def test_list_validation_errors():
    """geocode_slc.py:61-92: mismatched inputs raise ValueError before any GPU work."""
    sc = synth.scene_c1(length=64, width=64, geo=16, dem_px=64, slc=True)
    g = sc.geogrid
    geo = np.zeros((g.length, g.width), np.complex64)
    with pytest.raises(ValueError, match="not the same type"):
        geocode_slc([geo], sc.slc, *_args(sc))
    with pytest.raises(ValueError, match="do not match"):
        geocode_slc([geo, geo.copy()], [sc.slc], *_args(sc))
    with pytest.raises(ValueError, match="radar input is invalid"):
        geocode_slc([geo], [], *_args(sc))
    with pytest.raises(ValueError, match="radar input is invalid"):
        geocode_slc([geo], [sc.slc, sc.slc[:10]], *_args(sc))
    with pytest.raises(ValueError, match="mask output array shape"):
        geocode_slc(geo, sc.slc, *_args(sc), mask_block=np.zeros((3, 3), np.uint8))
    with pytest.raises(ValueError, match="carrier output array shape"):
        geocode_slc(geo, sc.slc, *_args(sc), carrier_phase_block=np.zeros((3, 3)))
    with pytest.raises(TypeError):
        geocode_slc(geo, sc.slc, *_args(sc), az_carrier=LUT2d(), rg_carrier=Poly2d())
    with pytest.raises(TypeError):
        geocode_slc(geo.astype(np.complex128), sc.slc, *_args(sc))


def test_lut2d_constructors():
    x = np.linspace(0, 10, 5)
    y = np.linspace(100, 102, 3)
    z = np.arange(15, dtype=float).reshape(3, 5)
    a = LUT2d(x, y, z, "nearest")
    b = LUT2d(0.0, 100.0, 2.5, 1.0, z, "nearest")
    for lut in (a, b):
        assert lut.have_data and lut.width == 5 and lut.length == 3 and lut.ref_value == 0.0
        assert lut.x_spacing == 2.5 and lut.y_spacing == 1.0
    one = LUT2d(np.array([1.0]), np.array([2.0]), np.array([[7.5]]))
    assert not one.have_data and one.ref_value == 7.5
    with pytest.raises(ValueError):
        LUT2d(np.array([0.0, 1.0, 3.0]), y, np.zeros((3, 3)))
