"""Block planning on the GPU against the oracle: radar bounding boxes of many
geogrid blocks in one launch (geometry/boundingbox.cpp:434-641), the DEM
statistics (DEMInterpolator.cpp:515-560) and block_generator
(python/packages/isce3/core/rdr_geo_block_generator.py:7-117).

Bounding boxes are integers: they must equal the oracle's exactly, status and
failure detail included, for blocks inside the swath, outside the radar grid,
beyond the orbit's span and on the wrong side of the track."""
import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import plan_cases  # noqa: E402
from isce3_gb300 import geometry  # noqa: E402
from isce3_gb300.core import LUT2d  # noqa: E402
from isce3_gb300.rdr_geo_block_generator import block_generator, plan_blocks  # noqa: E402

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)


def _gpu(blocks, sc, **kw):
    out = []
    for r in geometry.get_radar_bboxes(blocks, sc.radar_grid, sc.orbit, **kw):
        if isinstance(r, Exception):
            out.append(str(r))
        else:
            out.append((r.first_azimuth_line, r.last_azimuth_line, r.first_range_sample, r.last_range_sample))
    return out


def _oracle(oracle_mod, blocks, sc, min_height=-500.0, max_height=9000.0, doppler=None, margin=50,
            geo2rdr_params=None, geogrid_expansion_threshold=100):
    p = geo2rdr_params or geometry.Geo2RdrParams()
    out = []
    for b in blocks:
        r = oracle_mod.radar_bbox(b, sc.radar_grid, sc.orbit, min_height, max_height, doppler, margin, p.threshold,
                                  p.maxiter, p.delta_range, geogrid_expansion_threshold)
        out.append(r[:4] if r[4] == 0 else geometry._bbox_error(r[4], r[5]))
    return out


@pytest.mark.parametrize("kw", [dict(min_height=0.0, max_height=1500.0),
                                dict(min_height=-500.0, max_height=9000.0, margin=0),
                                dict(min_height=200.0, max_height=300.0, margin=5, geogrid_expansion_threshold=1),
                                dict(min_height=0.0, max_height=1500.0, geogrid_expansion_threshold=0)])
def test_bboxes_lonlat_match_oracle(oracle_mod, kw):
    sc = plan_cases.lonlat_scene()
    blocks = plan_cases.lonlat_blocks(sc)
    got, ref = _gpu(blocks, sc, **kw), _oracle(oracle_mod, blocks, sc, **kw)
    assert got == ref
    kinds = {type(r) for r in ref}
    if kw.get("geogrid_expansion_threshold", 100):
        assert kinds == {tuple, str}          # the cases cover success and failure


def test_bboxes_utm_match_oracle(oracle_mod):
    sc = plan_cases.utm_scene()
    blocks = plan_cases.utm_blocks(sc)
    for kw in (dict(min_height=0.0, max_height=3000.0), dict(min_height=0.0, max_height=3000.0, margin=0)):
        got, ref = _gpu(blocks, sc, **kw), _oracle(oracle_mod, blocks, sc, **kw)
        assert got == ref
    assert sum(isinstance(r, tuple) for r in ref) > 2


def test_bboxes_with_doppler_match_oracle(oracle_mod):
    """Non-zero image-grid Doppler (bilinear LUT2d, bounds checked) enters the
    Newton derivative with delta_range."""
    sc = plan_cases.utm_scene()
    blocks = plan_cases.utm_blocks(sc)
    d = sc.native_doppler
    kw = dict(min_height=0.0, max_height=3000.0, doppler=d,
              geo2rdr_params=geometry.Geo2RdrParams(1e-8, 50, 10.0))
    got, ref = _gpu(blocks, sc, **kw), _oracle(oracle_mod, blocks, sc, **kw)
    assert got == ref


def test_get_radar_bbox_overloads(oracle_mod):
    sc = plan_cases.lonlat_scene()
    rg = sc.radar_grid
    b = geometry.get_radar_bbox(sc.geogrid, rg, sc.orbit, 0.0, 1500.0)
    # the reference test's properties (tests/python/extensions/pybind/geometry/bbox.py:30-58)
    assert b.first_azimuth_line < b.last_azimuth_line and b.first_range_sample < b.last_range_sample
    assert 0 <= b.first_azimuth_line < rg.length and 0 <= b.last_azimuth_line < rg.length
    assert 0 <= b.first_range_sample < rg.width and 0 <= b.last_range_sample < rg.width
    dem = geometry.DEMInterpolator(sc.dem)
    mn, mx, _ = dem.compute_min_max_mean_height()
    b2 = geometry.get_radar_bbox(sc.geogrid, rg, sc.orbit, dem)          # margin 5 by default
    r = oracle_mod.radar_bbox(sc.geogrid, rg, sc.orbit, float(mn), float(mx), margin=5)
    assert (b2.first_azimuth_line, b2.last_azimuth_line, b2.first_range_sample, b2.last_range_sample) == r[:4]
    with pytest.raises(RuntimeError, match="did not converge"):
        geometry.get_radar_bbox(plan_cases.shifted(sc.geogrid, 0.0, 12.0), rg, sc.orbit)
    with pytest.raises(ValueError):
        geometry.get_radar_bbox(sc.geogrid, rg, sc.orbit, 10.0, 0.0)
    with pytest.raises(ValueError):
        geometry.get_radar_bbox(sc.geogrid, rg, sc.orbit, 0.0, 10.0, margin=-1)


def test_dem_stats_match_oracle(oracle_mod):
    rng = np.random.default_rng(7)
    z = rng.uniform(-30.0, 4000.0, (1031, 777)).astype(np.float32)
    z[rng.integers(0, 1031, 2000), rng.integers(0, 777, 2000)] = np.nan
    big = torch.full((1031, 800), 1e9, dtype=torch.float32, device="cuda")
    big[:, :777] = torch.from_numpy(z).cuda()
    view = big[:, :777]                          # a row stride beyond the width
    from isce3_gb300 import _lib as L
    import ctypes as C
    lib, ctx = L.lib(), L.context(0)
    mn, mx, mean, nv = C.c_float(), C.c_float(), C.c_double(), C.c_int64()
    for _ in range(2):                           # the same bits on every call
        L.check(lib.gslc_dem_stats(ctx, C.c_void_p(view.data_ptr()), 1031, 777, view.stride(0), C.byref(mn),
                                   C.byref(mx), C.byref(mean), C.byref(nv), None), ctx)
        omn, omx, omean, on = oracle_mod.dem_stats(z)
        assert np.float32(mn.value) == omn and np.float32(mx.value) == omx and nv.value == on
        assert abs(mean.value - omean) <= 1e-12 * abs(omean)
    allnan = torch.full((3, 5), float("nan"), device="cuda")
    L.check(lib.gslc_dem_stats(ctx, C.c_void_p(allnan.data_ptr()), 3, 5, 5, C.byref(mn), C.byref(mx),
                               C.byref(mean), C.byref(nv), None), ctx)
    assert nv.value == 0 and math.isnan(mean.value) and mn.value == np.finfo(np.float32).max


def _reference_block_generator(oracle_mod, geo_grid, sc, lines, cols, expansion):
    """rdr_geo_block_generator.py:7-117 over the oracle's bbox and DEM stats."""
    mn, mx, _, _ = oracle_mod.dem_stats(sc.dem.data)
    for geo_slice, shape, g in plan_blocks(geo_grid, lines, cols):
        r = oracle_mod.radar_bbox(g, sc.radar_grid, sc.orbit, float(mn), float(mx), None, 50, 1e-8, 50, 10.0,
                                  expansion)
        if r[4] != 0:
            continue
        yield np.s_[r[0]:r[1], r[2]:r[3]], geo_slice, shape, g


@pytest.mark.parametrize("lines,cols", [(128, 128), (100, 300), (512, 64)])
def test_block_generator_matches_reference_loop(oracle_mod, lines, cols):
    sc = plan_cases.lonlat_scene()
    big, _ = plan_cases.enlarged(sc.geogrid, 1.6, 64)
    got = list(block_generator(big, sc.radar_grid, sc.orbit, sc.dem, lines, cols))
    ref = list(_reference_block_generator(oracle_mod, big, sc, lines, cols, 1))
    assert len(got) == len(ref) > 0
    for (ra, ga, sa, ba), (rb, gb, sb, bb) in zip(got, ref):
        assert ra == rb and ga == gb and sa == sb
        assert (ba.start_x, ba.start_y, ba.width, ba.length) == (bb.start_x, bb.start_y, bb.width, bb.length)
    n_blocks = len(plan_blocks(big, lines, cols))
    assert len(got) < n_blocks            # some blocks have no radar data and are skipped
