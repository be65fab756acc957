"""Geogrid blocks for the block-planning tests (radar bounding boxes).

Cases around the synthetic scenes: blocks inside the swath, blocks partly
or wholly outside the radar grid (no overlap), a geogrid far beyond the
orbit's time span (geo2rdr leaves the orbit: no convergence), and a geogrid
on the other side of the ground track (wrong look side).
"""
import numpy as np

from isce3_gb300 import synth
from isce3_gb300.product import GeoGridParameters
from isce3_gb300.rdr_geo_block_generator import plan_blocks


def lonlat_scene(seed=11):
    return synth.scene_c1(seed=seed, slc=False)


def utm_scene(seed=12):
    return synth.scene_c2(seed=seed, length=4096, width=2048, geo=600, spacing=20.0, dem_arcsec=12.0, slc=False)


def enlarged(g: GeoGridParameters, factor: float, blocks_px: int):
    """g grown by `factor` about its centre, in blocks_px-pixel blocks."""
    w, l = int(g.width * factor), int(g.length * factor)
    x0 = g.start_x - g.spacing_x * (w - g.width) / 2
    y0 = g.start_y - g.spacing_y * (l - g.length) / 2
    big = GeoGridParameters(x0, y0, g.spacing_x, g.spacing_y, w, l, g.epsg)
    return big, [b for _, _, b in plan_blocks(big, blocks_px, blocks_px)]


def shifted(g: GeoGridParameters, dx: float, dy: float):
    return GeoGridParameters(g.start_x + dx, g.start_y + dy, g.spacing_x, g.spacing_y, g.width, g.length, g.epsg)


def mirrored_lonlat(sc):
    """The geogrid reflected across the ground track at sensing mid."""
    g = sc.geogrid
    pos, _ = sc.model.state(sc.radar_grid.sensing_mid)
    nadir_lon = np.degrees(np.arctan2(pos[1], pos[0]))
    cx = g.start_x + g.spacing_x * g.width / 2
    return shifted(g, 2 * (nadir_lon - cx), 0.0)


def lonlat_blocks(sc):
    g = sc.geogrid
    _, blocks = enlarged(g, 2.0, 128)
    return [g, shifted(g, 0.0, 12.0), mirrored_lonlat(sc)] + blocks


def utm_blocks(sc):
    g = sc.geogrid
    _, blocks = enlarged(g, 2.0, 200)
    return [g, shifted(g, 0.0, 1.3e6)] + blocks
