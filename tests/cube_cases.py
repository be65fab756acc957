"""Cube geogrids for the radar-grid metadata cube tests
(geometry/metadataCubes.cpp:276-489): a coarse grid around each synthetic
scene's swath, larger than the radar grid so that native-Doppler LUT bounds
and the orbit span make some points fail, and a heights vector like the GSLC
workflow's (-500 m to 9000 m)."""
import numpy as np

from isce3_gb300.product import GeoGridParameters

HEIGHTS = np.arange(-500.0, 9001.0, 500.0)


def utm_cube(sc, spacing=500.0, n=90):
    g = sc.geogrid
    cx = g.start_x + g.spacing_x * g.width / 2
    cy = g.start_y + g.spacing_y * g.length / 2
    return GeoGridParameters(cx - spacing * n / 2, cy + spacing * n / 2, spacing, -spacing, n, n, g.epsg)


def lonlat_cube(sc, n=64):
    g = sc.geogrid
    w = g.spacing_x * g.width * 1.6
    l = g.spacing_y * g.length * 1.6
    cx = g.start_x + g.spacing_x * g.width / 2
    cy = g.start_y + g.spacing_y * g.length / 2
    return GeoGridParameters(cx - w / 2, cy - l / 2, w / n, l / n, n, n, 4326)
