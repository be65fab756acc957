"""Grid descriptions of the SLC geocoding call surface.

Mirrors isce3's ``RadarGridParameters`` (cxx/isce3/product/
RadarGridParameters.{h,cpp}), ``GeoGridParameters`` (cxx/isce3/product/
GeoGridParameters.h) and ``SubSwaths`` (cxx/isce3/product/SubSwaths.{h,cpp})
with the Python keyword names of their pybind bindings.
"""
from __future__ import annotations

import numpy as np

from .core import DateTime, LookSide


class RadarGridParameters:
    """python/extensions/pybind_isce3/product/RadarGridParameters.cpp:18-53."""

    def __init__(self, sensing_start: float, wavelength: float, prf: float, starting_range: float,
                 range_pixel_spacing: float, lookside, length: int, width: int,
                 ref_epoch: DateTime | None = None):
        self.sensing_start = float(sensing_start)
        self.wavelength = float(wavelength)
        self.prf = float(prf)
        self.starting_range = float(starting_range)
        self.range_pixel_spacing = float(range_pixel_spacing)
        if isinstance(lookside, str):
            lookside = LookSide[lookside.capitalize()]
        self.lookside = LookSide(int(lookside))
        self.length = int(length)
        self.width = int(width)
        self.ref_epoch = ref_epoch if ref_epoch is not None else DateTime(2000, 1, 1)

    # cxx/isce3/product/RadarGridParameters.h:96-160
    @property
    def az_time_interval(self) -> float:
        return 1.0 / self.prf

    @property
    def sensing_stop(self) -> float:
        return self.sensing_start + (self.length - 1.0) / self.prf

    @property
    def sensing_mid(self) -> float:
        return 0.5 * (self.sensing_start + self.sensing_stop)

    @property
    def end_range(self) -> float:
        return self.starting_range + (self.width - 1.0) * self.range_pixel_spacing

    @property
    def mid_range(self) -> float:
        return 0.5 * (self.starting_range + self.end_range)

    @property
    def shape(self):
        return (self.length, self.width)

    def sensing_time(self, line: float) -> float:
        return self.sensing_start + line / self.prf

    def slant_range(self, sample: float) -> float:
        return self.starting_range + sample * self.range_pixel_spacing

    def contains(self, aztime: float, srange: float) -> bool:
        """product/RadarGridParameters.cpp:27-35 (half-pixel margins)."""
        half_az = self.az_time_interval / 2
        half_rg = self.range_pixel_spacing / 2
        return (aztime >= self.sensing_start - half_az and srange >= self.starting_range - half_rg
                and aztime <= self.sensing_stop + half_az and srange <= self.end_range + half_rg)

    def offset_and_resize(self, yoff: float, xoff: float, ysize: int, xsize: int) -> "RadarGridParameters":
        """RadarGridParameters.h offsetAndResize."""
        return RadarGridParameters(self.sensing_time(yoff), self.wavelength, self.prf, self.slant_range(xoff),
                                   self.range_pixel_spacing, self.lookside, ysize, xsize, self.ref_epoch)

    def copy(self) -> "RadarGridParameters":
        return RadarGridParameters(self.sensing_start, self.wavelength, self.prf, self.starting_range,
                                   self.range_pixel_spacing, self.lookside, self.length, self.width,
                                   self.ref_epoch)


class GeoGridParameters:
    """python/extensions/pybind_isce3/product/GeoGridParameters.cpp:16-20.

    ``start_x``/``start_y`` are the outer corner of the first pixel; pixel
    centres are at ``start + spacing * (index + 0.5)``.
    """

    def __init__(self, start_x: float = 0.0, start_y: float = 0.0, spacing_x: float = 0.0,
                 spacing_y: float = 0.0, width: int = 0, length: int = 0, epsg: int = 4326):
        self.start_x = float(start_x)
        self.start_y = float(start_y)
        self.spacing_x = float(spacing_x)
        self.spacing_y = float(spacing_y)
        self.width = int(width)
        self.length = int(length)
        self.epsg = int(epsg)

    @property
    def end_x(self) -> float:
        return self.start_x + self.spacing_x * self.width

    @property
    def end_y(self) -> float:
        return self.start_y + self.spacing_y * self.length

    @property
    def shape(self):
        return (self.length, self.width)

    def __getitem__(self, key):
        """Sub-grid by (row slice, column slice) like the pybind __getitem__."""
        islice, jslice = key
        i0, i1, istep = islice.indices(self.length)
        j0, j1, jstep = jslice.indices(self.width)
        if istep != 1 or jstep != 1:
            raise ValueError("only unit-step slices are supported")
        return GeoGridParameters(self.start_x + j0 * self.spacing_x, self.start_y + i0 * self.spacing_y,
                                 self.spacing_x, self.spacing_y, j1 - j0, i1 - i0, self.epsg)

    def __repr__(self):
        return (f"GeoGridParameters(start_x={self.start_x}, start_y={self.start_y}, spacing_x={self.spacing_x}, "
                f"spacing_y={self.spacing_y}, width={self.width}, length={self.length}, epsg={self.epsg})")


class SubSwaths:
    """Valid-sample intervals per radar line (product/SubSwaths.{h,cpp}).

    ``set_valid_samples_array(n, arr)`` stores an (length, 2) int array of
    half-open [start, stop) range-sample intervals for subswath ``n``
    (1-based).  ``get_sample_sub_swath`` restates SubSwaths.cpp:58-96.
    """

    def __init__(self, length: int = 0, width: int = 0, num_sub_swaths: int = 1):
        self.length = int(length)
        self.width = int(width)
        self._arrays = [np.zeros((0, 2), dtype=np.int32) for _ in range(int(num_sub_swaths))]

    @property
    def num_sub_swaths(self) -> int:
        return len(self._arrays)

    def set_valid_samples_array(self, sub_swath_number: int, valid_samples_array) -> None:
        arr = np.ascontiguousarray(np.asarray(valid_samples_array), dtype=np.int32)
        if arr.shape != (self.length, 2):
            raise ValueError(f"valid samples array must have shape ({self.length}, 2)")
        n = int(sub_swath_number)
        while len(self._arrays) < n:
            self._arrays.append(np.zeros((0, 2), dtype=np.int32))
        self._arrays[n - 1] = arr

    def get_valid_samples_array(self, sub_swath_number: int) -> np.ndarray:
        return self._arrays[int(sub_swath_number) - 1]

    def get_sample_sub_swath(self, azimuth_index: int, range_index: int) -> int:
        if range_index < 0 or range_index >= self.width or azimuth_index < 0 or azimuth_index >= self.length:
            return 0
        if len(self._arrays) == 0:
            return 1
        for s, arr in enumerate(self._arrays, start=1):
            if arr.size == 0:
                return s
            if arr[azimuth_index, 0] <= range_index < arr[azimuth_index, 1]:
                return s
        return 0

    def packed(self) -> np.ndarray:
        """(n, length, 2) int32 array; an empty subswath covers the whole line."""
        out = np.zeros((len(self._arrays), self.length, 2), dtype=np.int32)
        for k, arr in enumerate(self._arrays):
            if arr.size == 0:
                out[k, :, 0] = np.iinfo(np.int32).min
                out[k, :, 1] = np.iinfo(np.int32).max
            else:
                out[k] = arr
        return out
