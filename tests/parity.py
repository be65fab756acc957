"""Comparison of product output against the oracle, with the tolerances the
parity contract states:

- masks and the valid/invalid pattern: bit-exact;
- complex values: |gpu - oracle| <= 1e-5 |oracle| + 1e-6 rms(oracle);
- phase: |arg(gpu * conj(oracle))| <= 1e-4 rad where |oracle| >= 1e-2 rms.

A pixel whose radar coordinate selects a different row of the 8192-phase sinc
table on the two sides (its fractional index sits within ~1e-8 pixel of a
1/8192 boundary) is a "table flip": two correct implementations of the
reference disagree there by up to ~1e-3 relative, because the reference's own
orbit interpolation carries ~1e-9 m rounding noise.  Flips are counted and
bounded, not hidden.
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
            rtol=1e-5, atol_rms=1e-6, phase_tol=1e-4):
    geo_g = np.asarray(geo_g)
    geo_o = np.asarray(geo_o)
    r = {}
    r["mask_mismatch"] = int(np.sum(mask_g != mask_o)) if mask_g is not None else 0
    vg, vo = np.isfinite(az_g), np.isfinite(az_o)
    r["coord_validity_mismatch"] = int(np.sum(vg != vo))
    r["value_nan_mismatch"] = int(np.sum(np.isnan(geo_g) != np.isnan(geo_o)))
    both = vg & vo
    flips = both & ((table_index(az_g, az_first) != table_index(az_o, az_first)) |
                    (table_index(rg_g, rg_first) != table_index(rg_o, rg_first)))
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
    if both.any():
        r["max_az_coord_diff"] = float(np.max(np.abs(az_g[both] - az_o[both])))
        r["max_rg_coord_diff"] = float(np.max(np.abs(rg_g[both] - rg_o[both])))
    return r


def assert_parity(r, max_flip_fraction=1e-3):
    assert r["mask_mismatch"] == 0, r
    assert r["coord_validity_mismatch"] == 0, r
    assert r["value_nan_mismatch"] == 0, r
    assert r["invalid_fill_mismatch"] == 0, r
    assert r["n_out_of_tol"] == 0, r
    assert r["n_phase_out_of_tol"] == 0, r
    assert r["flip_fraction"] <= max_flip_fraction, r
