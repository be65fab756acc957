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
from types import SimpleNamespace

import numpy as np

# GDALDataType codes (gdal.h), as isce3.io.gdal exposes them
gdal = SimpleNamespace(GDT_Unknown=0, GDT_Byte=1, GDT_UInt16=2, GDT_Int16=3, GDT_UInt32=4, GDT_Int32=5,
                       GDT_Float32=6, GDT_Float64=7, GDT_CInt16=8, GDT_CInt32=9, GDT_CFloat32=10,
                       GDT_CFloat64=11)

_NP_TO_GDT = {np.dtype(np.uint8): gdal.GDT_Byte, np.dtype(np.uint16): gdal.GDT_UInt16,
              np.dtype(np.int16): gdal.GDT_Int16, np.dtype(np.uint32): gdal.GDT_UInt32,
              np.dtype(np.int32): gdal.GDT_Int32, np.dtype(np.float32): gdal.GDT_Float32,
              np.dtype(np.float64): gdal.GDT_Float64, np.dtype(np.complex64): gdal.GDT_CFloat32,
              np.dtype(np.complex128): gdal.GDT_CFloat64}


def gdal_type_of(arr) -> int:
    """GDALDataType of a NumPy array or torch tensor (GDT_Unknown if none)."""
    dt = getattr(arr, "dtype", None)
    try:
        import torch
        if isinstance(arr, torch.Tensor):
            dt = torch.empty(0, dtype=arr.dtype).numpy().dtype
    except (ImportError, TypeError):
        pass
    return _NP_TO_GDT.get(np.dtype(dt), gdal.GDT_Unknown) if dt is not None else gdal.GDT_Unknown


class Raster:
    """A raster of one or more bands with a GDAL-style geotransform.

    ``geotransform = [x0, dx, 0, y0, 0, dy]`` gives the outer corner of pixel
    (0, 0) and the pixel spacing, as ``GDALGetGeoTransform`` would.  Samples
    are ``(length, width)`` for one band or ``(bands, length, width)``.  Real
    samples are held as float32 (a DEM, which has one band) or float64 (a
    phase raster), complex ones as complex64 (an SLC); the geotransform and
    EPSG code are needed only where the raster is used as a DEM.
    """

    def __init__(self, path_or_data, geotransform=None, epsg: int | None = None):
        if isinstance(path_or_data, (str, Path)):
            p = Path(path_or_data)
            meta = json.loads(p.with_suffix(".json").read_text())
            data = np.load(p.with_suffix(".npy"))
            geotransform = meta.get("geotransform")
            epsg = meta.get("epsg")
        else:
            data = path_or_data
        arr = np.asarray(data)
        if np.iscomplexobj(arr):
            dt = np.complex64
        elif arr.dtype == np.float64:
            dt = np.float64
        else:
            dt = np.float32
        self.data = np.ascontiguousarray(arr.astype(dt, copy=False))
        if self.data.ndim not in (2, 3):
            raise ValueError("Raster data must be 2-D, or 3-D with the bands first")
        self._gt = None
        if geotransform is not None:
            gt = [float(v) for v in geotransform]
            if len(gt) != 6:
                raise ValueError("geotransform must have 6 terms")
            if gt[2] != 0.0 or gt[4] != 0.0:
                raise NotImplementedError("rotated geotransforms are not supported")
            self._gt = gt
        self._epsg = int(epsg) if epsg is not None else None
        self._device_cache = {}

    @classmethod
    def empty(cls, width: int, length: int, datatype: int = gdal.GDT_CFloat32, geotransform=None, epsg=None,
              bands: int = 1):
        """A zero-filled raster to write into (isce3.io.Raster(path, width,
        length, bands, datatype, driver) without the file)."""
        inv = {v: k for k, v in _NP_TO_GDT.items()}
        if datatype not in (gdal.GDT_Float32, gdal.GDT_Float64, gdal.GDT_CFloat32):
            raise NotImplementedError("only GDT_Float32, GDT_Float64 and GDT_CFloat32 rasters are held")
        shape = (int(length), int(width)) if bands == 1 else (int(bands), int(length), int(width))
        return cls(np.zeros(shape, inv[datatype]), geotransform, epsg)

    def datatype(self) -> int:
        """GDALDataType of the samples (isce3.io.Raster.datatype())."""
        return gdal_type_of(self.data)

    # isce3.io.Raster-like accessors
    @property
    def width(self) -> int:
        return int(self.data.shape[-1])

    @property
    def length(self) -> int:
        return int(self.data.shape[-2])

    def num_bands(self) -> int:
        """Number of bands (isce3.io.Raster.num_bands)."""
        return 1 if self.data.ndim == 2 else int(self.data.shape[0])

    def band(self, i: int) -> np.ndarray:
        """Samples of band i (0-based; GDAL numbers bands from 1), a view."""
        if self.data.ndim == 2:
            if i != 0:
                raise IndexError("single-band raster")
            return self.data
        return self.data[i]

    def get_geotransform(self):
        if self._gt is None:
            raise ValueError("raster has no geotransform")
        return list(self._gt)

    def set_geotransform(self, geotransform) -> None:
        self._gt = [float(v) for v in geotransform]

    def get_epsg(self) -> int:
        if self._epsg is None:
            raise ValueError("raster has no EPSG code")
        return self._epsg

    @property
    def dx(self) -> float:
        return self.get_geotransform()[1]

    @property
    def dy(self) -> float:
        return self.get_geotransform()[5]

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
