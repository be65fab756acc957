"""Comparison of product output against the oracle — TEST INFRASTRUCTURE.

Used by tests/ and by bench.py's CPU-baseline leg.  Tolerances of the parity
contract:

- masks and the valid/invalid pattern: bit-exact;
- complex values: |gpu - oracle| <= 1e-5 |oracle| + 1e-6 rms(oracle);
- phase: |arg(gpu * conj(oracle))| <= 1e-4 rad where |oracle| >= 1e-2 rms.

Three kinds of pixel are counted separately, because two correct
implementations of the reference (its own x86 and Arm builds included) split
there; they are bounded, not hidden:

- geometry splits: the azimuth coordinate differs by more than 1e-6 pixel
  or the range coordinate by more than 1e-8 pixel.  Either the geo2rdr
  Newton stops one iterate apart (the last |dt| sits at the threshold,
  Geo2Rdr.icc:172), which moves azimuth time by up to the threshold, or the
  FP32 DEM spline rounds the height to a neighbouring float because lon/lat
  differ by an ulp (different libm), which moves slant range by about one
  float ulp of the height: 1e-7 m near sea level to 2e-4 m at 3000 m.
  Normal differences are below 1e-10 s in azimuth time and 1e-8 m in slant
  range; the range limit is finer because the flattening phase turns range
  into phase at 4 pi / wavelength (about 3e-4 rad per 1e-6 pixel at L-band).
- sinc-table flips: the coordinate selects a different row of the 8192-phase
  sinc table (Sinc2dInterpolator.cpp:82-83); the reference's own orbit
  interpolation carries ~1e-9 m rounding noise, so a fraction ~1e-4 of pixels
  whose fractional index sits at a 1/8192 boundary flips.
"""
import numpy as np

SINC_SUB = 8192


def table_index(coord, first=0):
    a = np.asarray(coord, dtype=np.float64) - first
    with np.errstate(invalid="ignore"):
        ia = np.trunc(a)
        y = 4.0 + (a - ia)
        iy = np.floor(y)
        fy = y - iy
        idx = np.clip(np.nan_to_num(fy * SINC_SUB).astype(np.int64), 0, SINC_SUB - 1)
    return idx + SINC_SUB * np.nan_to_num(iy - 4).astype(np.int64)


def compare(geo_g, geo_o, az_g, az_o, rg_g, rg_o, mask_g=None, mask_o=None, az_first=0, rg_first=0,
            rtol=1e-5, atol_rms=1e-6, phase_tol=1e-4, split_px=1e-6, split_rg_px=1e-8):
    geo_g = np.asarray(geo_g)
    geo_o = np.asarray(geo_o)
    r = {}
    r["mask_mismatch"] = int(np.sum(mask_g != mask_o)) if mask_g is not None else 0
    vg, vo = np.isfinite(az_g), np.isfinite(az_o)
    r["coord_validity_mismatch"] = int(np.sum(vg != vo))
    r["value_nan_mismatch"] = int(np.sum(np.isnan(geo_g) != np.isnan(geo_o)))
    both = vg & vo
    with np.errstate(invalid="ignore"):
        split = both & ((np.abs(az_g - az_o) > split_px) | (np.abs(rg_g - rg_o) > split_rg_px))
    flips = both & ~split & ((table_index(az_g, az_first) != table_index(az_o, az_first)) |
                             (table_index(rg_g, rg_first) != table_index(rg_o, rg_first)))
    r["n_geometry_splits"] = int(split.sum())
    flips = flips | split
    fin = both & np.isfinite(geo_o) & np.isfinite(geo_g)
    ok = fin & ~flips
    r["n_valid"] = int(fin.sum())
    r["n_flips"] = int((flips & fin).sum())
    r["flip_fraction"] = r["n_flips"] / max(r["n_valid"], 1)
    if ok.any():
        rms = float(np.sqrt(np.mean(np.abs(geo_o[ok]) ** 2)))
        err = np.abs(geo_g[ok] - geo_o[ok])
        tol = rtol * np.abs(geo_o[ok]) + atol_rms * rms
        r["n_out_of_tol"] = int(np.sum(err > tol))
        big = np.abs(geo_o[ok]) >= 1e-2 * rms
        ph = np.abs(np.angle(geo_g[ok][big] * np.conj(geo_o[ok][big])))
        r["max_phase_err"] = float(ph.max()) if ph.size else 0.0
        r["n_phase_out_of_tol"] = int(np.sum(ph > phase_tol))
        rel = err / np.maximum(np.abs(geo_o[ok]), 1e-2 * rms)
        r["max_rel_err"] = float(rel.max())
        r["p99_rel_err"] = float(np.percentile(rel, 99))
    else:
        r.update(n_out_of_tol=0, max_phase_err=0.0, n_phase_out_of_tol=0, max_rel_err=0.0, p99_rel_err=0.0)
    # invalid pixels carry the same fill on both sides
    inv = ~both
    r["invalid_fill_mismatch"] = int(np.sum(~((geo_g[inv] == geo_o[inv]) |
                                              (np.isnan(geo_g[inv]) & np.isnan(geo_o[inv])))))
    quiet = both & ~split
    if quiet.any():
        # coordinate agreement away from geometry splits (noise level)
        r["max_az_coord_diff"] = float(np.max(np.abs(az_g[quiet] - az_o[quiet])))
        r["max_rg_coord_diff"] = float(np.max(np.abs(rg_g[quiet] - rg_o[quiet])))
    return r


def assert_parity(r, max_flip_fraction=2e-3):
    assert r["mask_mismatch"] == 0, r
    assert r["coord_validity_mismatch"] == 0, r
    assert r["value_nan_mismatch"] == 0, r
    assert r["invalid_fill_mismatch"] == 0, r
    assert r["n_out_of_tol"] == 0, r
    assert r["n_phase_out_of_tol"] == 0, r
    assert r["flip_fraction"] <= max_flip_fraction, r
