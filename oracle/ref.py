"""ctypes front end of the reference's own geometry code — TEST INFRASTRUCTURE.

oracle/Makefile's "ref" target compiles the reference's geo2rdr
(geometry/detail/Geo2Rdr.icc), Hermite orbit interpolation
(core/detail/InterpolateOrbit.icc, core/Linspace.icc), Ellipsoid::lonLatToXyz
(core/Ellipsoid.h) and UTM projection (core/Projections.cpp) from the
reference checkout, behind oracle/ref_geo.cpp's C ABI, into oracle/_ref/.
Tests use it to pin the oracle's restatement of those functions bit for bit.
The checkout exists only where the reference is mounted; elsewhere
``available()`` is False and the pins are skipped.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REF = Path(os.environ.get("ISCE3_REFERENCE", "/root/reference"))
LIBS = {"": HERE / "_ref" / "libref_geo.so", "fma": HERE / "_ref" / "libref_geo_fma.so"}
INTERP_LIB = HERE / "_ref" / "libref_interp.so"
_SRC = [HERE / "ref_geo.cpp", HERE / "ref_interp.cpp", HERE / "ref_shim" / "Eigen" / "Dense",
        HERE / "ref_shim" / "pyre" / "journal.h"]
_libs: dict = {}


def available() -> bool:
    return (REF / "cxx" / "isce3" / "geometry" / "detail" / "Geo2Rdr.icc").exists()


def build(force: bool = False) -> bool:
    """Compile both builds (plain and contracting) if the checkout is present."""
    if not available():
        return False
    newest = max(p.stat().st_mtime for p in _SRC)
    if force or any(not p.exists() or p.stat().st_mtime < newest for p in [*LIBS.values(), INTERP_LIB]):
        cmd = ["make", "-C", str(HERE)] + (["-B"] if force else []) + ["ref", f"REF={REF}"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference build failed:\n{r.stdout}\n{r.stderr}")
    return True


def lib(variant: str = "") -> C.CDLL:
    L = _libs.get(variant)
    if L is None:
        if not build():
            raise RuntimeError("the reference checkout is not available")
        L = C.CDLL(str(LIBS[variant]))
        L.ref_orbit_interpolate.restype = C.c_int64
        L.ref_orbit_interpolate.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_int,
                                            C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]
        L.ref_lonlat_to_xyz.restype = None
        L.ref_lonlat_to_xyz.argtypes = [C.c_double, C.c_double, C.c_void_p, C.c_int64, C.c_void_p]
        L.ref_geo2rdr.restype = None
        L.ref_geo2rdr.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_int, C.c_double,
                                  C.c_double,
                                  C.c_void_p, C.c_int64, C.c_double, C.c_int, C.c_double, C.c_double, C.c_int,
                                  C.c_double, C.c_double, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        L.ref_utm_inverse.restype = C.c_int64
        L.ref_utm_inverse.argtypes = [C.c_int, C.c_void_p, C.c_int64, C.c_void_p]
        L.ref_utm_forward.restype = C.c_int64
        L.ref_utm_forward.argtypes = [C.c_int, C.c_void_p, C.c_int64, C.c_void_p]
        _libs[variant] = L
    return L


def _orbit_arrays(orbit):
    return (np.ascontiguousarray(orbit.position, np.float64), np.ascontiguousarray(orbit.velocity, np.float64))


def orbit_interpolate(orbit, t, variant: str = ""):
    """Orbit::interpolate (FillNaN, the orbit's interpolation method) at the
    times t: (pos, vel) of shape (m, 3)."""
    pos, vel = _orbit_arrays(orbit)
    t = np.ascontiguousarray(t, np.float64)
    P, V = np.zeros((t.size, 3)), np.zeros((t.size, 3))
    lib(variant).ref_orbit_interpolate(pos.ctypes.data, vel.ctypes.data, orbit.size, orbit.t0, orbit.spacing,
                                       int(orbit.interp_method), t.ctypes.data, t.size, P.ctypes.data, V.ctypes.data)
    return P, V


def lonlat_to_xyz(ellipsoid, llh, variant: str = ""):
    llh = np.ascontiguousarray(llh, np.float64).reshape(-1, 3)
    xyz = np.zeros_like(llh)
    lib(variant).ref_lonlat_to_xyz(ellipsoid.a, ellipsoid.e2, llh.ctypes.data, len(llh), xyz.ctypes.data)
    return xyz


def geo2rdr(llh, ellipsoid, orbit, wavelength, side, t_guess, threshold, maxiter, delta_range,
            doppler_ref_value=0.0, bounds_error=True, variant: str = ""):
    """isce3::geometry::geo2rdr at m points with an image-grid Doppler table
    without data (reference value ``doppler_ref_value``): (t, r, status)."""
    pos, vel = _orbit_arrays(orbit)
    llh = np.ascontiguousarray(llh, np.float64).reshape(-1, 3)
    m = len(llh)
    t, r, st = np.zeros(m), np.zeros(m), np.zeros(m, np.int32)
    lib(variant).ref_geo2rdr(pos.ctypes.data, vel.ctypes.data, orbit.size, orbit.t0, orbit.spacing,
                             int(orbit.interp_method), ellipsoid.a,
                             ellipsoid.e2, llh.ctypes.data, m, wavelength, int(side), t_guess, threshold,
                             int(maxiter), delta_range, doppler_ref_value, int(bounds_error), t.ctypes.data,
                             r.ctypes.data, st.ctypes.data)
    return t, r, st


def utm_inverse(epsg, xy, variant: str = ""):
    xy = np.ascontiguousarray(xy, np.float64).reshape(-1, 2)
    out = np.zeros_like(xy)
    bad = lib(variant).ref_utm_inverse(int(epsg), xy.ctypes.data, len(xy), out.ctypes.data)
    return out, int(bad)


def utm_forward(epsg, lonlat, variant: str = ""):
    ll = np.ascontiguousarray(lonlat, np.float64).reshape(-1, 2)
    out = np.zeros_like(ll)
    bad = lib(variant).ref_utm_forward(int(epsg), ll.ctypes.data, len(ll), out.ctypes.data)
    return out, int(bad)


_interp = None


def interp_lib() -> C.CDLL:
    """The reference's interpolators (ref_interp.cpp)."""
    global _interp
    if _interp is None:
        if not build():
            raise RuntimeError("the reference checkout is not available")
        L = C.CDLL(str(INTERP_LIB))
        L.ref_interp2d_double.restype = C.c_double
        L.ref_interp2d_double.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_double]
        L.ref_spline2d_float.restype = C.c_float
        L.ref_spline2d_float.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_double]
        L.ref_sinc2d_cfloat.restype = None
        L.ref_sinc2d_cfloat.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_double, C.c_void_p]
        L.ref_lut2d_eval.restype = C.c_double
        L.ref_lut2d_eval.argtypes = [C.c_double, C.c_double, C.c_double, C.c_double, C.c_void_p, C.c_int, C.c_int,
                                     C.c_int, C.c_int, C.c_double, C.c_double]
        L.ref_poly2d_eval.restype = C.c_double
        L.ref_poly2d_eval.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_void_p,
                                      C.c_double, C.c_double]
        _interp = L
    return _interp


def interp2d(method: int, z, x: float, y: float) -> float:
    """createInterpolator<double>(method) at (x, y); method: isce3 dataInterpMethod
    (0 sinc, 1 bilinear, 2 bicubic, 3 nearest, 4 biquintic)."""
    z = np.ascontiguousarray(z, np.float64)
    return interp_lib().ref_interp2d_double(int(method), z.ctypes.data, z.shape[0], z.shape[1], x, y)


def spline2d_float(z, x: float, y: float) -> np.float32:
    z = np.ascontiguousarray(z, np.float32)
    return np.float32(interp_lib().ref_spline2d_float(z.ctypes.data, z.shape[0], z.shape[1], x, y))


def sinc2d_cfloat(z, x: float, y: float) -> np.complex64:
    z = np.ascontiguousarray(z, np.complex64)
    out = np.zeros(2, np.float32)
    interp_lib().ref_sinc2d_cfloat(z.ctypes.data, z.shape[0], z.shape[1], x, y, out.ctypes.data)
    return np.complex64(out[0] + 1j * out[1])


def lut2d_eval(lut, y: float, x: float) -> float:
    """LUT2d<double>::eval of a table with data (core/LUT2d.cpp:124-158)."""
    z = np.ascontiguousarray(lut.data, np.float64)
    return interp_lib().ref_lut2d_eval(lut.x_start, lut.y_start, lut.x_spacing, lut.y_spacing, z.ctypes.data,
                                       z.shape[0], z.shape[1], int(lut.interp_method), int(lut.bounds_error), y, x)


def poly2d_eval(p, y: float, x: float) -> float:
    """Poly2d::eval (core/Poly2d.cpp:8-24)."""
    c = np.ascontiguousarray(p.coeffs, np.float64).reshape(-1)
    return interp_lib().ref_poly2d_eval(p.x_order, p.y_order, p.x_mean, p.y_mean, p.x_std, p.y_std, c.ctypes.data,
                                        y, x)
