"""DEM raster stand-in for ``isce3.io.Raster`` on the geocoding path.

The reference reads the DEM through GDAL (cxx/isce3/io/Raster.h; used by
geometry/loadDem.cpp:22-133).  The geocoder only needs the raster's samples,
geotransform and EPSG code, so this class carries exactly those.  It also
reads and writes a small self-describing file format (``.npy`` samples plus
a ``.json`` sidecar with the geotransform and EPSG) for the examples.
"""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np


class Raster:
    """A single-band float32 raster with a GDAL-style geotransform.

    ``geotransform = [x0, dx, 0, y0, 0, dy]`` gives the outer corner of pixel
    (0, 0) and the pixel spacing, as ``GDALGetGeoTransform`` would.
    """

    def __init__(self, path_or_data, geotransform=None, epsg: int | None = None):
        if isinstance(path_or_data, (str, Path)):
            p = Path(path_or_data)
            meta = json.loads(p.with_suffix(".json").read_text())
            data = np.load(p.with_suffix(".npy"))
            geotransform = meta["geotransform"]
            epsg = meta["epsg"]
        else:
            data = path_or_data
        if geotransform is None or epsg is None:
            raise ValueError("Raster needs a geotransform and an EPSG code")
        self.data = np.ascontiguousarray(np.asarray(data, dtype=np.float32))
        if self.data.ndim != 2:
            raise ValueError("Raster data must be 2-D")
        gt = [float(v) for v in geotransform]
        if len(gt) != 6:
            raise ValueError("geotransform must have 6 terms")
        if gt[2] != 0.0 or gt[4] != 0.0:
            raise NotImplementedError("rotated geotransforms are not supported")
        self._gt = gt
        self._epsg = int(epsg)
        self._device_cache = {}

    # isce3.io.Raster-like accessors
    @property
    def width(self) -> int:
        return int(self.data.shape[1])

    @property
    def length(self) -> int:
        return int(self.data.shape[0])

    def get_geotransform(self):
        return list(self._gt)

    def get_epsg(self) -> int:
        return self._epsg

    @property
    def dx(self) -> float:
        return self._gt[1]

    @property
    def dy(self) -> float:
        return self._gt[5]

    def to_device(self, device) -> "Raster":
        """Keep the whole raster resident on ``device``; geocode calls then
        index it in place instead of uploading their DEM window."""
        import torch
        self.resident = torch.from_numpy(self.data).to(device)
        return self

    def save(self, path) -> None:
        p = Path(path)
        np.save(p.with_suffix(".npy"), self.data)
        p.with_suffix(".json").write_text(json.dumps({"geotransform": self._gt, "epsg": self._epsg}))
