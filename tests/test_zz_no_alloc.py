"""The allocation-free entry point gslc_geocode_slc_noalloc, called through
the C ABI, gives the same result as gslc_geocode_slc.

It exists for callers that must not allocate device memory while they run
(serving loops with a fixed HBM budget, hosts that forbid allocation after
start-up, frameworks that own the memory pool); its scratch is static device
memory shared by every call.  The test makes two calls in a row that both use
that scratch (carrier deramp) with different sizes, so a second call that
inherited stale scratch contents would show.  It runs alone in a fresh
process as well as after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from isce3_gb300 import _lib as L, _marshal as M, synth  # noqa: E402
from isce3_gb300.core import LUT2d, Poly2d  # noqa: E402

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)


def _args(sc, slc, geo, mask, az_carrier, rg_carrier, dev, keep, orbit=None, c32=False):
    """GeocodeArgs for device tensors, as isce3_gb300.geocode builds them."""
    holder = M.AzRgHolder()
    a = L.GeocodeArgs()
    a.radar_grid = M.radar_grid_desc(sc.radar_grid)
    a.sliced_radar_grid = M.radar_grid_desc(sc.radar_grid)
    a.geo_grid = M.geo_grid_desc(sc.geogrid)
    a.orbit = M.orbit_desc(orbit if orbit is not None else sc.orbit)
    a.native_doppler = M.lut_desc(sc.native_doppler, dev)
    a.image_grid_doppler = M.lut_desc(sc.image_grid_doppler, dev)
    a.az_time_correction = M.lut_desc(LUT2d(), dev)
    a.srange_correction = M.lut_desc(LUT2d(), dev)
    a.az_carrier = M.azrg_desc(az_carrier, dev, holder)
    a.rg_carrier = M.azrg_desc(rg_carrier, dev, holder)
    a.ellipsoid_a, a.ellipsoid_e2 = sc.ellipsoid.a, sc.ellipsoid.e2
    a.threshold_geo2rdr, a.numiter_geo2rdr = sc.threshold, sc.maxiter
    a.flatten, a.reramp = 1, 1
    a.invalid_re, a.invalid_im = np.float32(np.nan), np.float32(np.nan)
    a.n_blocks = 1
    a.rdr_length, a.rdr_width = slc.shape
    rp = (C.c_void_p * 1)(slc.data_ptr())
    gp = (C.c_void_p * 1)(geo.data_ptr())
    a.rdr_blocks = C.cast(rp, C.POINTER(C.c_void_p))
    a.geo_blocks = C.cast(gp, C.POINTER(C.c_void_p))
    a.mask = mask.data_ptr()
    a.dem, dem_t = M.dem_raster_desc(sc.dem, sc.geogrid, 50, dev)
    a.dem_margin = 50
    a.rdr_format = 1 if c32 else 0
    keep.extend([holder, rp, gp, dem_t])
    return a


def _run(sc, az_carrier, rg_carrier, noalloc, c32=False, inplace=False, measure=False):
    """One call through the C ABI; returns (geo, mask[, radar block after])."""
    dev = torch.device("cuda", torch.cuda.current_device())
    g = sc.geogrid
    stream = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    lib = L.lib()
    slc = torch.from_numpy(sc.slc).to(dev)
    if c32:
        # complex32 samples (float16 pairs) as 32-bit words, by the library's codec
        words = torch.empty(slc.shape, dtype=torch.int32, device=dev)
        ctx = L.context(dev.index)
        L.check(lib.gslc_complex64_to_complex32(ctx, C.c_void_p(slc.data_ptr()), C.c_void_p(words.data_ptr()),
                                                 slc.numel(), stream), ctx)
        slc = words
    before = slc.clone()
    geo = torch.zeros((g.length, g.width), dtype=torch.complex64, device=dev)
    mask = torch.zeros((g.length, g.width), dtype=torch.uint8, device=dev)
    keep = []
    a = _args(sc, slc, geo, mask, az_carrier, rg_carrier, dev, keep, c32=c32)
    a.inplace_deramp = int(inplace)
    torch.cuda.synchronize()
    mem0 = _memory(dev.index) if measure else None
    if noalloc:
        err = C.create_string_buffer(512)
        st = lib.gslc_geocode_slc_noalloc(C.byref(a), stream, err, len(err))
        assert st == 0, err.value.decode()
    else:
        ctx = L.context(dev.index)
        L.check(lib.gslc_geocode_slc(ctx, C.byref(a), stream), ctx)
    torch.cuda.synchronize()
    if measure:
        mem1 = _memory(dev.index)
        # nothing was allocated: device free memory, the default pool's use and
        # reservation, and the pool's high-water mark (reset before the call)
        assert mem1 == dict(mem0, used_high=mem0["used"]), (mem0, mem1)
    if not inplace:
        assert torch.equal(slc, before), "radar input modified"
    return geo.cpu().numpy(), mask.cpu().numpy(), slc.cpu().numpy()


def _memory(device: int) -> dict:
    """cudaMemGetInfo's free bytes and the default memory pool's use (the
    pool serves cudaMallocAsync), with the pool's used high-water mark reset
    so that a transient allocation inside a call would show."""
    cu = C.CDLL("libcuda.so.1")
    d, pool = C.c_int(), C.c_void_p()
    assert cu.cuDeviceGet(C.byref(d), device) == 0
    assert cu.cuDeviceGetDefaultMemPool(C.byref(pool), d) == 0
    vals = {}
    for name, attr in (("reserved", 5), ("used", 7), ("used_high", 8)):
        v = C.c_uint64()
        assert cu.cuMemPoolGetAttribute(pool, attr, C.byref(v)) == 0
        vals[name] = v.value
    zero = C.c_uint64(0)
    assert cu.cuMemPoolSetAttribute(pool, 8, C.byref(zero)) == 0     # reset the high-water mark
    vals["used_high"] = vals["used"]
    vals["free"] = torch.cuda.mem_get_info(device)[0]
    return vals


def _compare(ref, got):
    (g0, m0), (g1, m1) = ref, got
    np.testing.assert_array_equal(m0, m1)
    v = np.isfinite(g0)
    np.testing.assert_array_equal(v, np.isfinite(g1))
    assert v.sum() > 1000
    rms = np.sqrt(np.mean(np.abs(g0[v]) ** 2))
    # tolerance of the parity tests: 1e-5 relative + 1e-6 rms
    assert np.all(np.abs(g1[v] - g0[v]) <= 1e-5 * np.abs(g0[v]) + 1e-6 * rms)


def test_noalloc_matches_regular_entry_point_twice():
    sc1 = synth.scene_c1(seed=11, length=1024, width=1024, geo=256, dem_px=128)
    sc2 = synth.scene_c1(seed=12, length=768, width=640, geo=192, dem_px=96)
    mid1, mid2 = sc1.radar_grid.sensing_mid, sc2.radar_grid.sensing_mid
    cases = [
        (sc1, Poly2d([[0.0], [2 * np.pi * 200.0]], y_mean=mid1), Poly2d([[0.3, 1e-3]], x_mean=sc1.radar_grid.mid_range)),
        (sc2, Poly2d([[0.1], [-2 * np.pi * 90.0]], y_mean=mid2), Poly2d([[0.0, -2e-3]], x_mean=sc2.radar_grid.mid_range)),
    ]
    for sc, azc, rgc in cases:             # two calls in a row, different sizes
        ref = _run(sc, azc, rgc, noalloc=False)
        got = _run(sc, azc, rgc, noalloc=True)
        _compare(ref[:2], got[:2])


def test_noalloc_allocates_nothing():
    """A call that is not the first on the device (the first one uploads the
    sinc table, and the first launch of each kernel loads its code) changes
    neither the device's free memory nor the default pool's use, reservation
    or high-water mark."""
    sc = synth.scene_c1(seed=14, length=768, width=768, geo=192, dem_px=96)
    azc = Poly2d([[0.0], [2 * np.pi * 150.0]], y_mean=sc.radar_grid.sensing_mid)
    rgc = Poly2d([[0.2, 1e-3]], x_mean=sc.radar_grid.mid_range)
    _run(sc, azc, rgc, noalloc=True)
    got = _run(sc, azc, rgc, noalloc=True, measure=True)
    ref = _run(sc, azc, rgc, noalloc=False)
    _compare(ref[:2], got[:2])


def test_noalloc_complex32_blocks_with_carriers():
    """complex32 radar blocks with carriers: the deramp reads them and writes
    complex64 copies into the static scratch, as gslc_geocode_slc does into
    its stream-ordered scratch."""
    sc = synth.scene_c1(seed=15, length=640, width=704, geo=160, dem_px=96)
    azc = Poly2d([[0.0], [2 * np.pi * 120.0]], y_mean=sc.radar_grid.sensing_mid)
    rgc = Poly2d([[0.1, -1e-3]], x_mean=sc.radar_grid.mid_range)
    ref = _run(sc, azc, rgc, noalloc=False, c32=True)
    got = _run(sc, azc, rgc, noalloc=True, c32=True)
    _compare(ref[:2], got[:2])


def test_noalloc_inplace_deramp():
    """inplace_deramp=1 deramps the caller's block itself (the reference's
    behaviour) and uses no scratch: same outputs and same deramped block as
    the regular entry point."""
    sc = synth.scene_c1(seed=16, length=512, width=512, geo=128, dem_px=96)
    azc = Poly2d([[0.0], [2 * np.pi * 80.0]], y_mean=sc.radar_grid.sensing_mid)
    rgc = Poly2d([[0.0]])
    ref = _run(sc, azc, rgc, noalloc=False, inplace=True)
    got = _run(sc, azc, rgc, noalloc=True, inplace=True)
    _compare(ref[:2], got[:2])
    np.testing.assert_array_equal(ref[2], got[2])
    assert not np.array_equal(got[2], sc.slc)


def test_noalloc_sinc_lut_carriers():
    """Carriers given as LUT2d tables with the sinc method: their double sinc
    table is static scratch too, uploaded with the float one at set-up."""
    sc = synth.scene_c1(seed=17, length=512, width=576, geo=128, dem_px=96)
    rg = sc.radar_grid
    rr = rg.starting_range + (rg.end_range - rg.starting_range) / 11 * (np.arange(36) - 12)
    tt = rg.sensing_start + (rg.sensing_stop - rg.sensing_start) / 11 * (np.arange(36) - 12)
    T, R = np.meshgrid((tt - rg.sensing_mid) / (tt[-1] - tt[0]), (rr - rg.mid_range) / (rr[-1] - rr[0]),
                       indexing="ij")
    azc = LUT2d(rr, tt, 2 * np.pi * 30.0 * T + 0.4 * R, "sinc")
    rgc = LUT2d(rr, tt, 0.6 * R - 0.1 * T, "sinc")
    ref = _run(sc, azc, rgc, noalloc=False)
    got = _run(sc, azc, rgc, noalloc=True)
    _compare(ref[:2], got[:2])


def test_noalloc_rejects_long_orbit():
    """More state vectors than the static orbit table holds (256)."""
    sc = synth.scene_c1(seed=17, length=256, width=256, geo=64, dem_px=96)
    orbit = sc.model.orbit(sc.radar_grid.sensing_mid, 257, 2.0)
    dev = torch.device("cuda", torch.cuda.current_device())
    g = sc.geogrid
    slc = torch.from_numpy(sc.slc).to(dev)
    geo = torch.zeros((g.length, g.width), dtype=torch.complex64, device=dev)
    mask = torch.zeros((g.length, g.width), dtype=torch.uint8, device=dev)
    keep = []
    a = _args(sc, slc, geo, mask, Poly2d(), Poly2d(), dev, keep, orbit=orbit)
    err = C.create_string_buffer(512)
    st = L.lib().gslc_geocode_slc_noalloc(C.byref(a), C.c_void_p(torch.cuda.current_stream().cuda_stream), err,
                                          len(err))
    assert st == L.GSLC_EINVAL
    assert b"256 state vectors" in err.value


def test_noalloc_rejects_oversized_input():
    sc = synth.scene_c1(seed=13, length=2048, width=2100, geo=64, dem_px=96)   # 4.3M samples > 4194304
    dev = torch.device("cuda", torch.cuda.current_device())
    g = sc.geogrid
    slc = torch.from_numpy(sc.slc).to(dev)
    geo = torch.zeros((g.length, g.width), dtype=torch.complex64, device=dev)
    mask = torch.zeros((g.length, g.width), dtype=torch.uint8, device=dev)
    keep = []
    a = _args(sc, slc, geo, mask, Poly2d([[0.0], [1.0]]), Poly2d([[0.0]]), dev, keep)
    err = C.create_string_buffer(512)
    st = L.lib().gslc_geocode_slc_noalloc(C.byref(a), C.c_void_p(torch.cuda.current_stream().cuda_stream), err,
                                          len(err))
    assert st == L.GSLC_EINVAL
    assert b"allocation-free deramp scratch" in err.value
