"""Core value types of the SLC geocoding call surface.

These mirror the Python surface of isce3's ``isce3.core`` objects that
``isce3.geocode.geocode_slc`` accepts (pybind bindings in
python/extensions/pybind_isce3/core/{Orbit,LUT2d,Poly2d,Ellipsoid,
StateVector,DateTime}.cpp).  They are plain host-side containers: the numeric
work happens in the CUDA library, which receives them as POD descriptors.
"""
from __future__ import annotations

import datetime as _dt
import enum
from dataclasses import dataclass
from typing import Iterable, Sequence

import numpy as np

# WGS84, cxx/isce3/core/Constants.h:41-44
EARTH_SEMI_MAJOR_AXIS = 6378137.0
EARTH_ECCENTRICITY_SQUARED = 0.006694379990141317
# cxx/isce3/core/Constants.h:32-35
SINC_HALF, SINC_LEN, SINC_ONE, SINC_SUB = 4, 8, 9, 8192


class LookSide(enum.IntEnum):
    """cxx/isce3/core/LookSide.h: Right = -1, Left = 1."""
    Right = -1
    Left = 1


class DataInterpMethod(enum.IntEnum):
    """cxx/isce3/core/Constants.h:23-28 (dataInterpMethod)."""
    SINC = 0
    BILINEAR = 1
    BICUBIC = 2
    NEAREST = 3
    BIQUINTIC = 4


class OrbitInterpMethod(enum.IntEnum):
    """cxx/isce3/core/Orbit.h (OrbitInterpMethod)."""
    HERMITE = 0
    LEGENDRE = 1


_METHOD_NAMES = {
    "sinc": DataInterpMethod.SINC,
    "bilinear": DataInterpMethod.BILINEAR,
    "bicubic": DataInterpMethod.BICUBIC,
    "nearest": DataInterpMethod.NEAREST,
    "biquintic": DataInterpMethod.BIQUINTIC,
}


def _duck_method(method) -> DataInterpMethod:
    """python/extensions/pybind_isce3/core/LUT2d.cpp duck_method: str or enum."""
    if isinstance(method, str):
        try:
            return _METHOD_NAMES[method.lower()]
        except KeyError:
            raise ValueError(f"unknown interpolation method {method!r}") from None
    return DataInterpMethod(int(method))


class DateTime:
    """UTC date-time with sub-nanosecond seconds (cxx/isce3/core/DateTime.h).

    Stored as an integer count of whole seconds since 1970-01-01 plus a float
    fraction, which is what time tags relative to a reference epoch need.
    """

    def __init__(self, *args):
        if len(args) == 1 and isinstance(args[0], str):
            s = args[0].strip().replace("T", " ")
            whole, _, frac = s.partition(".")
            base = _dt.datetime.strptime(whole, "%Y-%m-%d %H:%M:%S")
            self._sec = int(base.replace(tzinfo=_dt.timezone.utc).timestamp())
            self._frac = float("0." + frac) if frac else 0.0
        elif len(args) == 1 and isinstance(args[0], DateTime):
            self._sec, self._frac = args[0]._sec, args[0]._frac
        else:
            y, mo, d = args[:3]
            h, mi = (args[3:5] + (0, 0))[:2] if len(args) > 3 else (0, 0)
            s = args[5] if len(args) > 5 else 0.0
            base = _dt.datetime(y, mo, d, h, mi, tzinfo=_dt.timezone.utc)
            whole = int(np.floor(s))
            self._sec = int(base.timestamp()) + whole
            self._frac = float(s - whole)

    def __add__(self, seconds: float) -> "DateTime":
        out = DateTime(self)
        whole = int(np.floor(seconds))
        out._sec += whole
        out._frac += float(seconds) - whole
        if out._frac >= 1.0:
            out._sec += 1
            out._frac -= 1.0
        return out

    def __sub__(self, other: "DateTime") -> float:
        return float(self._sec - other._sec) + (self._frac - other._frac)

    def __eq__(self, other) -> bool:
        return isinstance(other, DateTime) and self._sec == other._sec and self._frac == other._frac

    def isoformat(self) -> str:
        base = _dt.datetime.fromtimestamp(self._sec, tz=_dt.timezone.utc)
        return base.strftime("%Y-%m-%dT%H:%M:%S") + f"{self._frac:.9f}"[1:]

    def __repr__(self) -> str:
        return f"DateTime({self.isoformat()!r})"


@dataclass
class StateVector:
    """python/extensions/pybind_isce3/core/StateVector.cpp:15-16."""
    datetime: DateTime
    position: Sequence[float]
    velocity: Sequence[float]


class Orbit:
    """Uniformly sampled platform state vectors (cxx/isce3/core/Orbit.h).

    Time tags are ``t0 + i * spacing`` seconds after ``reference_epoch``
    (core/Linspace.h:56), exactly as the reference stores them.
    """

    def __init__(self, state_vectors: Iterable[StateVector], reference_epoch: DateTime | None = None,
                 interp_method=OrbitInterpMethod.HERMITE, type: str = ""):
        svs = list(state_vectors)
        if len(svs) < 2:
            raise ValueError("Orbit requires at least 2 state vectors")
        if reference_epoch is None:
            reference_epoch = svs[0].datetime
        self.reference_epoch = reference_epoch
        t = np.array([sv.datetime - reference_epoch for sv in svs], dtype=np.float64)
        spacing = (t[-1] - t[0]) / (len(t) - 1)
        if np.any(np.abs(np.diff(t) - spacing) > 1e-6 * max(abs(spacing), 1.0)):
            raise ValueError("non-uniform state vector time spacing")
        self._init(t[0], spacing, np.array([sv.position for sv in svs], dtype=np.float64),
                   np.array([sv.velocity for sv in svs], dtype=np.float64), interp_method, type)

    @classmethod
    def from_arrays(cls, t0: float, spacing: float, position, velocity, reference_epoch=None,
                    interp_method=OrbitInterpMethod.HERMITE, type: str = "") -> "Orbit":
        self = cls.__new__(cls)
        self.reference_epoch = reference_epoch if reference_epoch is not None else DateTime(2000, 1, 1)
        self._init(float(t0), float(spacing), np.asarray(position, dtype=np.float64),
                   np.asarray(velocity, dtype=np.float64), interp_method, type)
        return self

    def _init(self, t0, spacing, pos, vel, interp_method, type_):
        if pos.shape != vel.shape or pos.ndim != 2 or pos.shape[1] != 3:
            raise ValueError("position and velocity must be (n, 3)")
        self.t0 = float(t0)
        self.spacing = float(spacing)
        self._pos = np.ascontiguousarray(pos)
        self._vel = np.ascontiguousarray(vel)
        if isinstance(interp_method, str):
            interp_method = OrbitInterpMethod[interp_method.upper()]
        self.interp_method = OrbitInterpMethod(int(interp_method))
        self.type = type_

    @property
    def size(self) -> int:
        return self._pos.shape[0]

    @property
    def time(self) -> np.ndarray:
        # core/Linspace.h:56 — first + i * spacing, evaluated in double
        return np.array([self.t0 + i * self.spacing for i in range(self.size)])

    @property
    def position(self) -> np.ndarray:
        return self._pos

    @property
    def velocity(self) -> np.ndarray:
        return self._vel

    @property
    def start_time(self) -> float:
        return self.t0

    @property
    def end_time(self) -> float:
        return self.t0 + (self.size - 1) * self.spacing

    @property
    def mid_time(self) -> float:
        return 0.5 * (self.start_time + self.end_time)

    def contains(self, t: float) -> bool:
        return self.start_time <= t <= self.end_time

    def copy(self) -> "Orbit":
        return Orbit.from_arrays(self.t0, self.spacing, self._pos.copy(), self._vel.copy(),
                                 self.reference_epoch, self.interp_method, self.type)


class LUT2d:
    """2-D look-up table z = f(y, x) (cxx/isce3/core/LUT2d.{h,cpp}).

    Constructors follow python/extensions/pybind_isce3/core/LUT2d.cpp:39-92:
    ``LUT2d()``, ``LUT2d(xstart, ystart, dx, dy, data, method, b_error)`` and
    ``LUT2d(xcoord, ycoord, data, method, b_error)``.  A default LUT has no
    data, contains every point and evaluates to ``ref_value`` (0).
    """

    def __init__(self, *args, method="bilinear", b_error: bool = True, **kw):
        self.have_data = False
        self.bounds_error = True
        self.ref_value = 0.0
        self.x_start = self.y_start = 0.0
        self.x_spacing = self.y_spacing = 1.0
        self._data = np.zeros((0, 0))
        if "data" in kw or len(args) >= 3:
            names = ("xstart", "ystart", "dx", "dy", "data", "method", "b_error")
            if len(args) in (3, 4, 5) and np.ndim(args[0]) == 1 and len(args) < 6 and np.ndim(args[2]) == 2 \
                    and np.ndim(args[1]) == 1:
                # (xcoord, ycoord, data[, method[, b_error]])
                xcoord = np.asarray(args[0], dtype=np.float64)
                ycoord = np.asarray(args[1], dtype=np.float64)
                data = np.asarray(args[2], dtype=np.float64)
                if len(args) > 3:
                    method = args[3]
                if len(args) > 4:
                    b_error = args[4]
                self._set_from_coords(xcoord, ycoord, data)
            else:
                vals = dict(zip(names, args))
                vals.update(kw)
                data = np.asarray(vals["data"], dtype=np.float64)
                if data.ndim != 2:
                    raise RuntimeError("buffer object must be 2-D")
                method = vals.get("method", method)
                b_error = vals.get("b_error", b_error)
                self.x_start, self.y_start = float(vals["xstart"]), float(vals["ystart"])
                self.x_spacing, self.y_spacing = float(vals["dx"]), float(vals["dy"])
                self._data = np.ascontiguousarray(data)
                self.have_data = True
                self.ref_value = float(data[0, 0])
            self.bounds_error = bool(b_error)
        elif len(args) == 1:
            method = args[0]
        self.interp_method = _duck_method(method)

    def _set_from_coords(self, xcoord, ycoord, data):
        """core/LUT2d.cpp:50-119 (setFromData)."""
        if data.ndim != 2:
            raise RuntimeError("buffer object must be 2-D")
        if xcoord.size == 0 and ycoord.size == 0:
            self.have_data = False
            return
        if xcoord.size == 1 and ycoord.size == 1:
            self.have_data = False
            self.ref_value = float(data[0, 0])
            return
        if xcoord.size != data.shape[1] or ycoord.size != data.shape[0]:
            raise ValueError("Inconsistent shapes between data and coordinates")
        dy = ycoord[1] - ycoord[0]
        dx = xcoord[1] - xcoord[0]
        if np.any(np.abs(np.diff(ycoord) - dy) > 1e-8):
            raise ValueError("Detected non-regular Y-coordinates for LUT2d grid.")
        if np.any(np.abs(np.diff(xcoord) - dx) > 1e-8):
            raise ValueError("Detected non-regular X-coordinates for LUT2d grid.")
        self.x_start, self.y_start = float(xcoord[0]), float(ycoord[0])
        self.x_spacing, self.y_spacing = float(dx), float(dy)
        self._data = np.ascontiguousarray(data)
        self.have_data = True
        self.ref_value = float(data[0, 0])

    @property
    def data(self) -> np.ndarray:
        return self._data

    @property
    def length(self) -> int:
        return int(self._data.shape[0])

    @property
    def width(self) -> int:
        return int(self._data.shape[1]) if self._data.ndim == 2 else 0

    def contains(self, y: float, x: float) -> bool:
        """core/LUT2d.h:84-95."""
        if not self.have_data:
            return True
        i = (x - self.x_start) / self.x_spacing
        j = (y - self.y_start) / self.y_spacing
        return (0.0 <= i <= self.width - 1.0) and (0.0 <= j <= self.length - 1.0)


class Poly2d:
    """Normalised 2-D polynomial (cxx/isce3/core/Poly2d.{h,cpp}).

    ``coeffs[i, j]`` multiplies ``((y - y_mean)/y_std)**i * ((x - x_mean)/x_std)**j``
    (python/extensions/pybind_isce3/core/Poly2d.cpp:51-70).  ``Poly2d()``
    has order -1 and evaluates to 0 (core/Poly2d.h:56).
    """

    def __init__(self, coeffs=None, x_mean: float = 0.0, y_mean: float = 0.0,
                 x_std: float = 1.0, y_std: float = 1.0):
        if coeffs is None:
            self.coeffs = np.zeros((0, 0))
            self.x_order = self.y_order = -1
        else:
            c = np.ascontiguousarray(np.atleast_2d(np.asarray(coeffs, dtype=np.float64)))
            self.coeffs = c
            self.y_order, self.x_order = c.shape[0] - 1, c.shape[1] - 1
        self.x_mean, self.y_mean = float(x_mean), float(y_mean)
        self.x_std, self.y_std = float(x_std), float(y_std)

    def eval(self, y: float, x: float) -> float:
        """core/Poly2d.cpp:8-24, evaluated in the same order."""
        xval = (x - self.x_mean) / self.x_std
        yval = (y - self.y_mean) / self.y_std
        val = 0.0
        scaley = 1.0
        for i in range(self.y_order + 1):
            scalex = 1.0
            for j in range(self.x_order + 1):
                val += scalex * scaley * float(self.coeffs[i, j])
                scalex *= xval
            scaley *= yval
        return val


class Ellipsoid:
    """Reference ellipsoid (cxx/isce3/core/Ellipsoid.h), WGS84 by default."""

    def __init__(self, a: float = EARTH_SEMI_MAJOR_AXIS, e2: float = EARTH_ECCENTRICITY_SQUARED):
        self.a = float(a)
        self.e2 = float(e2)

    @property
    def b(self) -> float:
        return self.a * np.sqrt(1.0 - self.e2)

    def lon_lat_to_xyz(self, llh) -> np.ndarray:
        """core/Ellipsoid.h:177-190 (vectorised over the last axis)."""
        llh = np.asarray(llh, dtype=np.float64)
        lon, lat, h = llh[..., 0], llh[..., 1], llh[..., 2]
        re = self.a / np.sqrt(1.0 - (self.e2 * np.sin(lat) ** 2))
        return np.stack([(re + h) * np.cos(lat) * np.cos(lon),
                         (re + h) * np.cos(lat) * np.sin(lon),
                         ((re * (1.0 - self.e2)) + h) * np.sin(lat)], axis=-1)

    def xyz_to_lon_lat(self, xyz) -> np.ndarray:
        """ECEF -> lon/lat/height by fixed-point iteration (vectorised)."""
        xyz = np.asarray(xyz, dtype=np.float64)
        x, y, z = xyz[..., 0], xyz[..., 1], xyz[..., 2]
        lon = np.arctan2(y, x)
        p = np.hypot(x, y)
        lat = np.arctan2(z, p * (1.0 - self.e2))
        h = np.zeros_like(lat)
        for _ in range(8):
            n = self.a / np.sqrt(1.0 - self.e2 * np.sin(lat) ** 2)
            h = p / np.cos(lat) - n
            lat = np.arctan2(z, p * (1.0 - self.e2 * n / (n + h)))
        return np.stack([lon, lat, h], axis=-1)
