"""``isce3.container.RadarGeometry``: a radar grid with its orbit and Doppler.

cxx/isce3/container/RadarGeometry.h:14-82 — the radar grid, the orbit and
the Doppler centroid LUT of the image grid that geo2rdr solves against.
"""
from __future__ import annotations

from .core import LUT2d, LookSide, Orbit
from .product import RadarGridParameters


class RadarGeometry:
    """Radar grid + orbit + Doppler (the geo2rdr Doppler of the image grid)."""

    def __init__(self, radar_grid: RadarGridParameters, orbit: Orbit, doppler: LUT2d | None = None):
        if not isinstance(radar_grid, RadarGridParameters):
            raise TypeError("radar_grid must be a RadarGridParameters")
        self._radar_grid = radar_grid
        self._orbit = orbit
        self._doppler = doppler if doppler is not None else LUT2d()

    @property
    def radar_grid(self) -> RadarGridParameters:
        return self._radar_grid

    @property
    def orbit(self) -> Orbit:
        return self._orbit

    @property
    def doppler(self) -> LUT2d:
        return self._doppler

    @property
    def lookside(self) -> LookSide:
        return self._radar_grid.lookside

    @property
    def wavelength(self) -> float:
        return self._radar_grid.wavelength

    @property
    def grid_length(self) -> int:
        return self._radar_grid.length

    @property
    def grid_width(self) -> int:
        return self._radar_grid.width
