"""``isce3.cuda`` surface on this path: ``isce3_gb300.cuda.geocode.Geocode``."""
from . import geocode  # noqa: F401
