"""GB300-native SLC geocoding with isce3's ``geocode_slc`` call surface.

Modules mirror the reference's Python packages on this path:
``core`` (Orbit, LUT2d, Poly2d, Ellipsoid, DateTime, StateVector, LookSide),
``product`` (RadarGridParameters, GeoGridParameters, SubSwaths), ``io``
(Raster), ``container`` (RadarGeometry), ``geocode`` (geocode_slc) and
``cuda.geocode`` (Geocode, the block raster geocoder).  The compute is
one CUDA library, libgslc.so, reached through the C ABI in include/gslc.h.
"""
from . import core, product, io, container  # noqa: F401
from .core import (DataInterpMethod, DateTime, Ellipsoid, LookSide, LUT2d, Orbit, OrbitInterpMethod,  # noqa: F401
                   Poly2d, StateVector)
from .product import GeoGridParameters, RadarGridParameters, SubSwaths  # noqa: F401

__version__ = "0.1.0"


def build(force: bool = False) -> None:
    """Compile libgslc.so for sm_103a in-tree."""
    from . import _lib
    _lib.build(force=force)
