"""Geo-block -> radar-block planning of the GSLC workflow on the GPU.

``block_generator`` keeps the call surface and the yielded tuples of
``isce3.core.rdr_geo_block_generator.block_generator``
(python/packages/isce3/core/rdr_geo_block_generator.py:7-117): the geogrid is
cut into blocks of ``geo_lines_per_block`` x ``geo_cols_per_block`` pixels,
each block's radar bounding box comes from ``get_radar_bbox`` at the DEM's
min/max heights, and blocks without radar data are skipped.  The reference
plans block by block on the host (eight geo2rdr solves per block); here the
DEM statistics are one GPU reduction and all blocks' bounding boxes one
kernel launch, computed before the first block is yielded.
"""
from __future__ import annotations

import numpy as np

from .geometry import DEMInterpolator, get_radar_bboxes
from .product import GeoGridParameters


def plan_blocks(geo_grid: GeoGridParameters, geo_lines_per_block: int, geo_cols_per_block: int):
    """The block geogrids in the reference's order (y blocks outer, x inner),
    with their start coordinates formed as there (rdr_geo_block_generator.py:49-96)."""
    n_y = int(np.ceil(geo_grid.length / geo_lines_per_block))
    n_x = int(np.ceil(geo_grid.width / geo_cols_per_block))
    block_length = geo_lines_per_block * geo_grid.spacing_y
    block_width = geo_cols_per_block * geo_grid.spacing_x
    out = []
    for i_y in range(n_y):
        y0 = i_y * geo_lines_per_block
        y1 = min(y0 + geo_lines_per_block, geo_grid.length)
        y_start = geo_grid.start_y + i_y * block_length
        for i_x in range(n_x):
            x0 = i_x * geo_cols_per_block
            x1 = min(x0 + geo_cols_per_block, geo_grid.width)
            x_start = geo_grid.start_x + i_x * block_width
            g = GeoGridParameters(x_start, y_start, geo_grid.spacing_x, geo_grid.spacing_y, x1 - x0, y1 - y0,
                                  geo_grid.epsg)
            out.append((np.s_[y0:y1, x0:x1], (y1 - y0, x1 - x0), g))
    return out


def block_generator(geo_grid, radar_grid, orbit, dem_raster, geo_lines_per_block, geo_cols_per_block,
                    geogrid_expansion_threshold=1, device=None):
    """Yield ``(radar_slice, geo_slice, geo_block_shape, blk_geo_grid)`` for
    every geogrid block with radar data, in the reference's order."""
    dem = dem_raster if isinstance(dem_raster, DEMInterpolator) else DEMInterpolator(dem_raster)
    min_h, max_h, _ = dem.compute_min_max_mean_height(device)
    blocks = plan_blocks(geo_grid, geo_lines_per_block, geo_cols_per_block)
    boxes = get_radar_bboxes([g for _, _, g in blocks], radar_grid, orbit, float(min_h), float(max_h),
                             geogrid_expansion_threshold=geogrid_expansion_threshold, device=device)
    for (geo_slice, shape, g), bbox in zip(blocks, boxes):
        if isinstance(bbox, Exception):
            continue        # no radar data for this block
        radar_slice = np.s_[bbox.first_azimuth_line:bbox.last_azimuth_line,
                            bbox.first_range_sample:bbox.last_range_sample]
        yield radar_slice, geo_slice, shape, g


__all__ = ["block_generator", "plan_blocks"]
