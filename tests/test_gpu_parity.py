"""GPU parity: the sm_103a kernel (through the C ABI) against the CPU oracle.

Every case runs the same seeded inputs through isce3_gb300.geocode.geocode_slc
(which calls gslc_geocode_slc in libgslc.so) and through the oracle, then
applies tests/parity.py: masks and validity bit-exact, complex values within
1e-5 relative (+1e-6 rms), phase within 1e-4 rad, sinc-table flips counted
and bounded.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from isce3_gb300 import synth  # noqa: E402
from isce3_gb300.core import DataInterpMethod, LUT2d, Poly2d  # noqa: E402
from isce3_gb300.geocode import geocode_slc  # noqa: E402
from isce3_gb300.product import SubSwaths  # noqa: E402

from oracle.compare import assert_parity, compare  # noqa: E402

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)


def _run_both(oracle_mod, sc, slc_blocks, rg=None, geogrid=None, dem=None, n_out=1, **kw):
    """Run product and oracle with identical arguments; return both outputs."""
    rg = rg or sc.radar_grid
    g = geogrid or sc.geogrid
    dem = dem or sc.dem
    shape = (g.length, g.width)
    nd = kw.pop("native_doppler", sc.native_doppler)
    igd = kw.pop("image_grid_doppler", sc.image_grid_doppler)
    out = {}
    for side in ("gpu", "ora"):
        geo = [np.zeros(shape, np.complex64) for _ in range(n_out)]
        mask = np.zeros(shape, np.uint8)
        az = np.zeros(shape)
        rgi = np.zeros(shape)
        carrier = np.full(shape, -7.0)
        flat = np.full(shape, -7.0)
        blocks = [b.copy() for b in slc_blocks]
        args = (geo if n_out > 1 else geo[0], blocks if n_out > 1 else blocks[0], dem, rg, g, sc.orbit, nd, igd,
                sc.ellipsoid, kw.get("threshold", sc.threshold), kw.get("maxiter", sc.maxiter))
        extra = {k: v for k, v in kw.items() if k not in ("threshold", "maxiter")}
        if side == "gpu":
            geocode_slc(*args, mask_block=mask, carrier_phase_block=carrier, flatten_phase_block=flat,
                        az_index_block=az, rg_index_block=rgi, **extra)
        else:
            extra.pop("geo2rdr_precision", None)
            oracle_mod.geocode_slc(*args, mask_block=mask, carrier_phase_block=carrier, flatten_phase_block=flat,
                                   az_index_block=az, rg_index_block=rgi, **extra)
        out[side] = dict(geo=geo, mask=mask, az=az, rg=rgi, carrier=carrier, flat=flat)
    return out["gpu"], out["ora"]


def _check(gpu, ora, az_first=0, rg_first=0, max_flip=1e-3):
    reports = []
    for gg, go in zip(gpu["geo"], ora["geo"]):
        r = compare(gg, go, gpu["az"], ora["az"], gpu["rg"], ora["rg"], gpu["mask"], ora["mask"],
                    az_first, rg_first)
        print(r)
        assert_parity(r, max_flip)
        reports.append(r)
    # carrier / flattening phase outputs: written on the same pixels, FP64;
    # compared away from geometry splits
    with np.errstate(invalid="ignore"):
        split = (np.abs(gpu["az"] - ora["az"]) > 1e-6) | (np.abs(gpu["rg"] - ora["rg"]) > 1e-6)
    for k in ("carrier", "flat"):
        wg, wo = gpu[k] != -7.0, ora[k] != -7.0
        np.testing.assert_array_equal(wg, wo)
        w = wg & ~split
        if w.any():
            assert np.abs(gpu[k][w] - ora[k][w]).max() <= 1e-6, k
    return reports


@pytest.fixture(scope="module")
def c1():
    return synth.scene_c1()


@pytest.mark.parametrize("precision", ["fp64", "ff"])
def test_c1_plain(oracle_mod, c1, precision):
    gpu, ora = _run_both(oracle_mod, c1, [c1.slc], geo2rdr_precision=precision)
    r = _check(gpu, ora)[0]
    assert r["n_valid"] > 100000
    assert r["max_rel_err"] < 1e-5


def test_c1_device_tensors_match_host_arrays(c1):
    """Device-resident torch inputs give the same bits as the host path."""
    g = c1.geogrid
    host = np.zeros((g.length, g.width), np.complex64)
    geocode_slc(host, c1.slc, c1.dem, c1.radar_grid, g, c1.orbit, LUT2d(), LUT2d(), c1.ellipsoid, 1e-8, 25)
    dev_out = torch.zeros((g.length, g.width), dtype=torch.complex64, device="cuda")
    dev_in = torch.from_numpy(c1.slc).cuda()
    geocode_slc(dev_out, dev_in, c1.dem, c1.radar_grid, g, c1.orbit, LUT2d(), LUT2d(), c1.ellipsoid, 1e-8, 25)
    np.testing.assert_array_equal(dev_out.cpu().numpy().view(np.uint64), host.view(np.uint64))
    np.testing.assert_array_equal(dev_in.cpu().numpy(), c1.slc)   # input not mutated


@pytest.mark.parametrize("pinned", [False, True])
def test_utm_host_outputs_equal_device_outputs(pinned):
    """Host geo blocks and mask, copied back by the library in row bands while
    later bands compute (gslc_geocode_slc_to_host), equal the device outputs
    of one launch bit for bit: a ragged last band, two blocks, carriers."""
    sc = synth.scene_c2(length=2048, width=1024, geo=600, spacing=12.0)
    g = sc.geogrid
    shape = (g.length, g.width)
    common = (sc.dem, sc.radar_grid, g, sc.orbit, sc.native_doppler, sc.image_grid_doppler, sc.ellipsoid,
              sc.threshold, sc.maxiter)
    kw = dict(az_carrier=sc.az_carrier, rg_carrier=sc.rg_carrier)
    slc2 = (sc.slc * np.complex64(0.5 - 0.25j)).astype(np.complex64)
    if pinned:
        host = [torch.zeros(shape, dtype=torch.complex64).pin_memory() for _ in range(2)]
        hmask = torch.zeros(shape, dtype=torch.uint8).pin_memory()
    else:
        host = [np.zeros(shape, np.complex64) for _ in range(2)]
        hmask = np.zeros(shape, np.uint8)
    geocode_slc(host, [sc.slc, slc2], *common, mask_block=hmask, **kw)
    dev = [torch.zeros(shape, dtype=torch.complex64, device="cuda") for _ in range(2)]
    dmask = torch.zeros(shape, dtype=torch.uint8, device="cuda")
    geocode_slc(dev, [torch.from_numpy(sc.slc).cuda(), torch.from_numpy(slc2).cuda()], *common,
                mask_block=dmask, **kw)
    dm = dmask.cpu().numpy()
    assert (dm == 1).sum() > 100000
    for h, d in zip(host, dev):
        hn = h.numpy() if pinned else h
        np.testing.assert_array_equal(d.cpu().numpy().view(np.uint64), hn.view(np.uint64))
    np.testing.assert_array_equal(dm, hmask.numpy() if pinned else hmask)


def test_c1_doppler_carriers_corrections_blocks(oracle_mod, c1):
    """Squinted grid (image-grid Doppler = native), Poly2d carriers, correction
    LUTs, two blocks of a radar sub-block with offsets, flatten with the
    corrected range, custom invalid value."""
    rg = c1.radar_grid
    rr = np.linspace(rg.starting_range - 50 * rg.range_pixel_spacing, rg.end_range + 50 * rg.range_pixel_spacing, 16)
    tt = np.linspace(rg.sensing_start - 50 / rg.prf, rg.sensing_stop + 50 / rg.prf, 12)
    u = (rr - rr.mean()) / (rr.max() - rr.mean())
    dop = LUT2d(rr, tt, np.tile(-40.0 + 80.0 * u ** 2, (12, 1)) + 3.0 * np.linspace(-1, 1, 12)[:, None])
    az_car = Poly2d([[0.0, 1e-4], [2 * np.pi * 250.0, 0.0]], x_mean=rg.mid_range, y_mean=rg.sensing_mid)
    rg_car = Poly2d([[0.5, 2e-3, 1e-7]], x_mean=rg.mid_range, y_mean=0.0)
    s_vec = np.linspace(rg.starting_range, rg.end_range, 9)
    t_vec = np.linspace(rg.sensing_start, rg.sensing_stop, 7)
    corr_r = LUT2d(s_vec, t_vec, 0.37 + 0.01 * np.arange(63).reshape(7, 9), DataInterpMethod.BILINEAR)
    corr_t = LUT2d(s_vec, t_vec, np.full((7, 9), 2.1e-5), DataInterpMethod.NEAREST)
    a0, r0 = 100, 150
    sub = [c1.slc[a0:a0 + 800, r0:r0 + 700], (c1.slc[a0:a0 + 800, r0:r0 + 700] * np.complex64(0.3 - 0.7j))]
    gpu, ora = _run_both(oracle_mod, c1, sub, n_out=2, native_doppler=dop, image_grid_doppler=dop,
                         az_carrier=az_car, rg_carrier=rg_car, az_time_correction=corr_t,
                         srange_correction=corr_r, first_azimuth_line=a0, first_range_sample=r0,
                         flatten_with_corrected_srange=True, invalid_value=np.complex64(-1 + 2j))
    _check(gpu, ora, az_first=a0, rg_first=r0)


def test_more_blocks_than_one_launch(oracle_mod, c1):
    """17 radar/geo block pairs: more than one launch's 16 (the call runs its
    blocks in groups of 16 with the same geometry)."""
    scales = [np.complex64(np.exp(0.3j * k) * (1.0 + 0.05 * k)) for k in range(17)]
    blocks = [c1.slc * s_ for s_ in scales]
    az_car = Poly2d([[0.0], [2 * np.pi * 100.0]], y_mean=c1.radar_grid.sensing_mid)
    gpu, ora = _run_both(oracle_mod, c1, blocks, n_out=17, az_carrier=az_car, rg_carrier=Poly2d())
    reports = _check(gpu, ora)
    assert len(reports) == 17 and all(r["n_valid"] > 10000 for r in reports)


@pytest.mark.parametrize("flatten,reramp,precision", [(False, True, "fp64"), (True, False, "fp64"),
                                                     (False, False, "fp64"), (True, True, "ff")])
def test_c1_flags(oracle_mod, c1, flatten, reramp, precision):
    az_car = Poly2d([[0.0], [2 * np.pi * 100.0]], y_mean=c1.radar_grid.sensing_mid)
    gpu, ora = _run_both(oracle_mod, c1, [c1.slc], flatten=flatten, reramp=reramp, az_carrier=az_car,
                         rg_carrier=Poly2d(), geo2rdr_precision=precision)
    _check(gpu, ora)


def test_sliced_grid_and_subswaths(oracle_mod, c1):
    rg = c1.radar_grid
    sliced = rg.offset_and_resize(100, 80, 700, 800)
    sw = SubSwaths(rg.length, rg.width, 2)
    lo = (100 + 50 * np.sin(np.arange(rg.length) / 90.0)).astype(np.int32)
    sw.set_valid_samples_array(1, np.stack([lo, np.full(rg.length, 500, np.int32)], axis=1))
    sw.set_valid_samples_array(2, np.stack([np.full(rg.length, 520, np.int32), np.full(rg.length, 990, np.int32)],
                                           axis=1))
    gpu, ora = _run_both(oracle_mod, c1, [c1.slc], sliced_radargrid=sliced, subswaths=sw)
    _check(gpu, ora)
    assert set(np.unique(gpu["mask"])) >= {0, 1, 2, 255}


@pytest.mark.parametrize("precision", ["fp64", "ff"])
def test_utm_geogrid_and_lut_doppler(oracle_mod, precision):
    """Reduced frame scene: UTM 32611 geogrid over an EPSG:4326 DEM, native
    Doppler LUT2d (quadratic in range) and a linear azimuth carrier."""
    sc = synth.scene_c2(length=2048, width=1024, geo=600, spacing=12.0)
    gpu, ora = _run_both(oracle_mod, sc, [sc.slc], az_carrier=sc.az_carrier, rg_carrier=sc.rg_carrier,
                         geo2rdr_precision=precision)
    r = _check(gpu, ora)[0]
    assert r["n_valid"] > 10000


@pytest.mark.parametrize("precision", ["fp64", "ff"])
def test_partial_native_doppler(oracle_mod, c1, precision):
    """A native Doppler table covering part of the swath, its edges running
    through the geogrid in range and azimuth: pixels whose zero-Doppler time
    and range (geocodeSlc.cpp:200-206), or whose chip's az and rng
    (geocodeSlc.cpp:457-467), fall outside it are left as the reference's
    LUT2d::contains decides, and the chips inside are demodulated with the
    table's Doppler."""
    rg = c1.radar_grid
    span_r = rg.end_range - rg.starting_range
    span_t = rg.sensing_stop - rg.sensing_start
    rr = np.linspace(rg.starting_range + 0.2 * span_r, rg.starting_range + 0.75 * span_r, 13)
    tt = np.linspace(rg.sensing_start + 0.15 * span_t, rg.sensing_start + 0.8 * span_t, 9)
    u = np.linspace(-1.0, 1.0, 13)
    dop = LUT2d(rr, tt, np.tile(30.0 - 55.0 * u ** 2, (9, 1)) + 8.0 * np.linspace(-1, 1, 9)[:, None])
    gpu, ora = _run_both(oracle_mod, c1, [c1.slc], native_doppler=dop, geo2rdr_precision=precision)
    r = _check(gpu, ora)[0]
    m = gpu["mask"]
    inside, outside = (m != 255).mean(), (m == 255).mean()
    assert inside > 0.2 and outside > 0.2, (inside, outside)
    assert r["n_valid"] > 10000


@pytest.mark.parametrize("precision", ["fp64", "ff"])
def test_native_doppler_table_beyond_index_range(oracle_mod, c1, precision):
    """A bilinear native Doppler table spanning more than 2^21 range samples
    (1000 km cells): the chip's Doppler takes the FP64-coordinate form
    instead of the one from the radar indices, with the same results."""
    rg = c1.radar_grid
    rr = rg.starting_range - 8.0e6 + 1.0e6 * np.arange(17)
    tt = np.linspace(rg.sensing_start - 1.0, rg.sensing_stop + 1.0, 5)
    dop = LUT2d(rr, tt, np.tile(20.0 + 3.0e-6 * (rr - rg.starting_range), (5, 1)) + 4.0 * np.arange(5)[:, None])
    gpu, ora = _run_both(oracle_mod, c1, [c1.slc], native_doppler=dop, geo2rdr_precision=precision)
    r = _check(gpu, ora)[0]
    assert r["n_valid"] > 10000


@pytest.mark.parametrize("where", ["south_32734", "descending_32610", "left_32609"])
def test_utm_south_and_descending_pass(oracle_mod, where):
    """The reduced frame scene moved to the southern hemisphere (UTM zone 34
    south, false northing 10,000 km: Projections.cpp's south branch), to a
    descending pass (the swath crossing the UTM rows the other way) and to
    a left-looking radar (the first iterate's look-side test,
    geometry/detail/Geo2Rdr.icc:156-161, with the other sign)."""
    if where == "left_32609":
        sc = synth.scene_c2(length=2048, width=1024, geo=600, spacing=12.0, epsg=32609,
                            look_side=synth.LookSide.Left)
    elif where == "south_32734":
        sc = synth.scene_c2(length=2048, width=1024, geo=600, spacing=12.0, epsg=32734, lat0_deg=-33.9,
                            lon0_deg=19.5)
    else:
        sc = synth.scene_c2(length=2048, width=1024, geo=600, spacing=12.0, epsg=32610, lat0_deg=47.5,
                            lon0_deg=-114.0, ascending=False)
    for precision in ("fp64", "ff"):
        gpu, ora = _run_both(oracle_mod, sc, [sc.slc], az_carrier=sc.az_carrier, rg_carrier=sc.rg_carrier,
                             geo2rdr_precision=precision)
        r = _check(gpu, ora)[0]
        assert r["n_valid"] > 10000


@pytest.mark.parametrize("case", ["coarse_exact", "dem_west_edge", "utm_dem"])
def test_utm_tile_fit_and_exact_paths(oracle_mod, case):
    """UTM geogrids through both ground-point paths of the kernel: the tile
    fit of the projection inverse (tiles up to 1 km), the exact per-pixel
    inverse (40 m spacing: 1.2 km tiles), tiles straddling the DEM's west
    edge (nodes disagree on the reference-height branch, so those tiles fall
    back to the exact path), and a UTM DEM (forward projection at the
    nodes)."""
    from isce3_gb300.io import Raster
    spacing = 40.0 if case == "coarse_exact" else 12.0
    sc = synth.scene_c2(length=2048, width=1024, geo=200 if case == "coarse_exact" else 600, spacing=spacing)
    g, dem = sc.geogrid, sc.dem
    if case == "dem_west_edge":
        gt = list(dem.get_geotransform())
        lon_c, _lat, _h = oracle_mod.proj_inverse(g.epsg, g.start_x + 0.5 * g.width * g.spacing_x,
                                                  g.start_y + 0.5 * g.length * g.spacing_y)
        k = int((np.degrees(lon_c) - gt[0]) / gt[1])
        dem = Raster(np.ascontiguousarray(dem.data[:, k:]), [gt[0] + k * gt[1]] + gt[1:], 4326)
    elif case == "utm_dem":
        rng = np.random.default_rng(11)
        n = 400
        x0 = g.start_x - 0.25 * g.width * g.spacing_x
        y0 = g.start_y + 0.25 * g.length * abs(g.spacing_y)
        dem = Raster(synth.fbm_surface((n, n), 0.8, rng, 0.0, 2000.0), [x0, 30.0, 0.0, y0, 0.0, -30.0], g.epsg)
    gpu, ora = _run_both(oracle_mod, sc, [sc.slc], dem=dem, az_carrier=sc.az_carrier, rg_carrier=sc.rg_carrier)
    r = _check(gpu, ora)[0]
    assert r["n_valid"] > 10000


def test_known_answer_lonlat_phase_gpu(c1):
    """The lon-as-phase KAT run through the GPU path (1e-6 rad)."""
    g = c1.geogrid
    slc = synth.kat_slc(c1, "x", 0.0)
    dem = synth.constant_dem_like(c1.dem, 0.0)
    geo = np.zeros((g.length, g.width), np.complex64)
    geocode_slc(geo, slc, dem, c1.radar_grid, g, c1.orbit, LUT2d(), LUT2d(), c1.ellipsoid, 1e-9, 25, flatten=False)
    truth = np.radians(g.start_x + g.spacing_x * (np.arange(g.width) + 0.5))[None, :]
    v = np.isfinite(geo)
    assert v.sum() > 0.4 * v.size
    err = np.angle(geo * np.exp(-1j * truth))[v]
    assert np.abs(err).max() < 1e-6


def test_edge_cases(oracle_mod, c1):
    g = c1.geogrid
    # geogrid entirely outside the swath: all invalid, mask 255
    far = g[0:32, 0:32]
    far.start_x += 5.0
    gpu, ora = _run_both(oracle_mod, c1, [c1.slc], geogrid=far, dem=synth.constant_dem_like(c1.dem, 0.0))
    assert np.all(gpu["mask"] == 255) and np.all(np.isnan(gpu["geo"][0]))
    _check(gpu, ora)
    # NaN and inf samples in the SLC propagate like the reference
    bad = c1.slc.copy()
    bad[500:503, 500:540] = np.complex64(complex(np.nan, 1.0))
    bad[600, 600] = np.complex64(complex(np.inf, 0.0))
    gpu, ora = _run_both(oracle_mod, c1, [bad])
    _check(gpu, ora)
    # radar block smaller than one sinc chip: nothing interpolated
    gpu, ora = _run_both(oracle_mod, c1, [c1.slc[:6, :6].copy()])
    assert np.all(~np.isfinite(gpu["geo"][0]))
    _check(gpu, ora)
    # empty geogrid is a no-op
    empty = np.zeros((0, g.width), np.complex64)
    geocode_slc(empty, c1.slc, c1.dem, c1.radar_grid, g[0:0, 0:g.width], c1.orbit, LUT2d(), LUT2d(),
                c1.ellipsoid, 1e-8, 25)


def test_projection_failure_raises(c1):
    """A UTM geogrid far outside its zone fails the inverse projection; the
    reference throws (Projections.h ProjectionBase::inverse), so do we."""
    from isce3_gb300.product import GeoGridParameters
    g = GeoGridParameters(-2.0e7, 4.0e6, 10.0, -10.0, 8, 8, 32611)
    geo = np.zeros((8, 8), np.complex64)
    with pytest.raises(ValueError):
        geocode_slc(geo, c1.slc, c1.dem, c1.radar_grid, g, c1.orbit, LUT2d(), LUT2d(), c1.ellipsoid, 1e-8, 25)


@pytest.mark.parametrize("precision", ["fp64", "ff"])
@pytest.mark.parametrize("name", ["c1", "c2r"])
def test_split_flip_fraction_within_cross_build(oracle_mod, name, precision):
    """On the stored cross-build scenes (tests/xbuild_scenes.py) the GPU's
    geometry splits and sinc-table flips against the oracle are at most 1.5x
    the fraction by which the oracle's own contracting build (the reference's
    aarch64 arithmetic, tests/test_oracle_cross_build.py) departs from it,
    and at most 1e-3 of valid pixels; everything else within tolerance."""
    import xbuild_scenes as xs
    sc = xs.unpack(dict(np.load(xs.GOLDEN)), name)
    plain = xs.run_oracle(oracle_mod, sc, "")
    fused = xs.run_oracle(oracle_mod, sc, "fma")
    r_x = xs.report(fused, plain)
    g = sc.geogrid
    shape = (g.length, g.width)
    gpu = dict(geo=np.zeros(shape, np.complex64), mask=np.zeros(shape, np.uint8), az=np.zeros(shape),
               rg=np.zeros(shape))
    geocode_slc(gpu["geo"], sc.slc, sc.dem, sc.radar_grid, g, sc.orbit, sc.native_doppler, sc.image_grid_doppler,
                sc.ellipsoid, sc.threshold, sc.maxiter, mask_block=gpu["mask"], az_index_block=gpu["az"],
                rg_index_block=gpu["rg"], geo2rdr_precision=precision, **xs.carriers(sc))
    r_g = xs.report(gpu, plain)
    print(name, precision, "gpu:", r_g, "fused build:", r_x)
    assert_parity(r_g, max_flip_fraction=1e-3)
    assert r_g["flip_fraction"] <= 1.5 * r_x["flip_fraction"], (r_g["flip_fraction"], r_x["flip_fraction"])


@pytest.mark.parametrize("method,precision", [("bilinear", "fp64"), ("bilinear", "ff"), ("nearest", "fp64")])
def test_lut2d_carriers(oracle_mod, c1, method, precision):
    """Data-bearing LUT2d azimuth and range carriers (the pybind overload for
    AzRgFunc = LUT2d<double>, GeocodeSlc.cpp:337): the deramp evaluates them
    at every radar sample (geocodeSlc.cpp:240-274) and the reramp at every
    output pixel (:298-394).  The tables cover the radar grid with a margin;
    the azimuth carrier is a TOPS-like quadratic in time, the range carrier
    a slow ramp in range."""
    rg = c1.radar_grid
    rr = np.linspace(rg.starting_range - 20 * rg.range_pixel_spacing, rg.end_range + 20 * rg.range_pixel_spacing, 24)
    tt = np.linspace(rg.sensing_start - 20 / rg.prf, rg.sensing_stop + 20 / rg.prf, 20)
    T, R = np.meshgrid(tt - rg.sensing_mid, rr - rg.mid_range, indexing="ij")
    az_car = LUT2d(rr, tt, 2 * np.pi * 180.0 * T + np.pi * 900.0 * T ** 2 + 1e-5 * R, method)
    rg_car = LUT2d(rr, tt, 2e-3 * R + 0.3 * T, method)
    gpu, ora = _run_both(oracle_mod, c1, [c1.slc], az_carrier=az_car, rg_carrier=rg_car,
                         geo2rdr_precision=precision)
    r = _check(gpu, ora)[0]
    assert r["n_valid"] > 100000
    # the carrier output holds the table values at the pixels' radar positions
    w = np.isfinite(gpu["az"]) & (gpu["carrier"] != -7.0)
    assert np.abs(gpu["carrier"][w]).max() > 1.0


@pytest.mark.parametrize("method,precision", [("sinc", "fp64"), ("bicubic", "fp64"), ("biquintic", "fp64"),
                                              ("biquintic", "ff")])
def test_lut2d_methods(oracle_mod, c1, method, precision):
    """LUT2d tables with the reference's other interpolators
    (core/LUT2d.cpp _setInterpolator: sinc 8 x 8, bicubic, biquintic order
    6) as the image-grid and native Doppler of a squinted grid (geo2rdr's
    Newton and the sinc chip's demodulation), as the slant-range correction
    and as the azimuth and range carriers.  The tables reach 12 samples past
    the radar grid on every side, so that the points the kernels evaluate
    lie where the sinc interpolator is non-zero and the bicubic reads stay
    inside the table."""
    rg = c1.radar_grid
    nr, nt = 40, 36
    pad_r, pad_t = 12, 12
    dr = (rg.end_range - rg.starting_range) / (nr - 1 - 2 * pad_r)
    dt = (rg.sensing_stop - rg.sensing_start) / (nt - 1 - 2 * pad_t)
    rr = rg.starting_range + dr * (np.arange(nr) - pad_r)
    tt = rg.sensing_start + dt * (np.arange(nt) - pad_t)
    T, R = np.meshgrid((tt - rg.sensing_mid) / (tt[-1] - tt[0]), (rr - rg.mid_range) / (rr[-1] - rr[0]),
                       indexing="ij")
    dop = LUT2d(rr, tt, -30.0 + 120.0 * R ** 2 + 25.0 * np.sin(3.0 * T) + 8.0 * R * T, method)
    corr_r = LUT2d(rr, tt, 0.4 + 0.2 * np.cos(2.0 * R + T), method)
    az_car = LUT2d(rr, tt, 2 * np.pi * 40.0 * T + 3.0 * T ** 2 + 0.5 * R, method)
    rg_car = LUT2d(rr, tt, 0.8 * R + 0.2 * T * R, method)
    gpu, ora = _run_both(oracle_mod, c1, [c1.slc], native_doppler=dop, image_grid_doppler=dop,
                         srange_correction=corr_r, az_carrier=az_car, rg_carrier=rg_car,
                         geo2rdr_precision=precision)
    r = _check(gpu, ora)[0]
    assert r["n_valid"] > 100000


@pytest.mark.parametrize("precision", ["fp64", "ff"])
@pytest.mark.parametrize("which", ["c1", "c2"])
def test_legendre_orbit(oracle_mod, c1, which, precision):
    """Legendre orbit interpolation (core/detail/InterpolateOrbit.icc:111-155):
    every Newton iterate interpolates the state vectors in the reference's
    operation order (the segment tables hold Hermite pieces); a float-float
    request takes the same FP64 path.  EPSG:4326 and UTM geogrids."""
    import copy
    from isce3_gb300.core import Orbit, OrbitInterpMethod
    sc = copy.copy(c1 if which == "c1" else synth.scene_c2(length=2048, width=1024, geo=400, spacing=15.0))
    o = sc.orbit
    sc.orbit = Orbit.from_arrays(o.t0, o.spacing, o.position, o.velocity, o.reference_epoch,
                                 OrbitInterpMethod.LEGENDRE)
    kw = {} if which == "c1" else dict(az_carrier=sc.az_carrier, rg_carrier=sc.rg_carrier)
    gpu, ora = _run_both(oracle_mod, sc, [sc.slc], geo2rdr_precision=precision, **kw)
    r = _check(gpu, ora)[0]
    assert r["n_valid"] > 10000


def test_context_orbit_tables_follow_the_orbit(c1):
    """A context keeps the host tables of the last orbits it used, keyed by
    their state vectors: calls alternating between two orbits, and one whose
    state vectors are changed in place, each give the bits of a call with
    that orbit alone."""
    from isce3_gb300.core import Orbit
    g = c1.geogrid

    def run(orbit):
        out = np.zeros((g.length, g.width), np.complex64)
        geocode_slc(out, c1.slc, c1.dem, c1.radar_grid, g, orbit, LUT2d(), LUT2d(), c1.ellipsoid, 1e-8, 25)
        return out.view(np.uint64).copy()

    o = c1.orbit
    a = Orbit.from_arrays(o.t0, o.spacing, o.position.copy(), o.velocity.copy(), o.reference_epoch)
    b = Orbit.from_arrays(o.t0, o.spacing, o.position + np.array([0.0, 0.0, 40.0]), o.velocity.copy(),
                          o.reference_epoch)
    ra = run(a)
    rb = run(b)
    assert not np.array_equal(ra, rb)
    np.testing.assert_array_equal(run(a), ra)
    saved = a.position.copy()
    a.position[:, 2] += 40.0               # the same bytes as b now
    np.testing.assert_array_equal(run(a), rb)
    a.position[...] = saved
    np.testing.assert_array_equal(run(a), ra)
