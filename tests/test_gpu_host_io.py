"""Host radar blocks through the pipelined call (gslc_geocode_slc_host_io):
the SLC and DEM window upload band by band while earlier bands compute, and
the results equal the device-resident call's bit for bit, for complex64 and
complex32 blocks, a radar sub-block with offsets and two blocks, page-locked
and pageable buffers, and when a plan too small makes the kernel flag reads
beyond what had arrived (every band then runs again)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import isce3_gb300.geocode as G  # noqa: E402
from isce3_gb300 import _lib as L  # noqa: E402
from isce3_gb300 import synth  # noqa: E402
from isce3_gb300.core import Poly2d  # noqa: E402
from isce3_gb300.types import to_complex32  # noqa: E402

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)


@pytest.fixture(scope="module")
def scene():
    return synth.scene_c2(length=3072, width=1536, geo=700, spacing=12.0)


def _run(sc, blocks, device_in, host_out, pinned=False, **kw):
    g = sc.geogrid
    shape = (g.length, g.width)
    common = (sc.dem, sc.radar_grid, g, sc.orbit, sc.native_doppler, sc.image_grid_doppler, sc.ellipsoid,
              sc.threshold, sc.maxiter)
    rdr = [torch.from_numpy(b).cuda() if device_in else b for b in blocks]
    if pinned:
        rdr = [torch.from_numpy(b).pin_memory() for b in blocks]
    if host_out:
        mk = (lambda sh, dt: torch.zeros(sh, dtype=dt).pin_memory()) if pinned else \
            (lambda sh, dt: torch.zeros(sh, dtype=dt).numpy())
    else:
        def mk(sh, dt):
            return torch.zeros(sh, dtype=dt, device="cuda")
    geo = [mk(shape, torch.complex64) for _ in blocks]
    mask = mk(shape, torch.uint8)
    az, rg = mk(shape, torch.float64), mk(shape, torch.float64)
    G.geocode_slc(geo if len(blocks) > 1 else geo[0], rdr if len(blocks) > 1 else rdr[0], *common, mask_block=mask,
                  az_index_block=az, rg_index_block=rg, az_carrier=sc.az_carrier,
                  rg_carrier=Poly2d([[0.1, 1e-3]], x_mean=sc.radar_grid.mid_range), **kw)

    def host(x):
        return x.cpu().numpy() if isinstance(x, torch.Tensor) else x
    return [host(x) for x in geo], host(mask), host(az), host(rg)


def _same(a, b):
    for x, y in zip(a[0], b[0]):
        np.testing.assert_array_equal(x.view(np.uint64), y.view(np.uint64))
    for x, y in zip(a[1:], b[1:]):
        np.testing.assert_array_equal(x.view(np.uint8), y.view(np.uint8))


@pytest.mark.parametrize("pinned", [False, True])
def test_host_inputs_equal_device_inputs(scene, pinned):
    sc = scene
    dev = _run(sc, [sc.slc], device_in=True, host_out=False)
    assert (dev[1] == 1).sum() > 200000
    for k in list(sc.dem.__dict__.get("_gslc_dev", {})):
        sc.dem.__dict__["_gslc_dev"].pop(k)        # the call uploads the DEM window too
    host = _run(sc, [sc.slc], device_in=False, host_out=True, pinned=pinned)
    assert G.L.lib().gslc_last_io_reruns(L.context(0)) == 0
    _same(dev, host)
    again = _run(sc, [sc.slc], device_in=False, host_out=False)     # DEM window cached now
    _same(dev, again)


def test_complex32_blocks_and_sub_block_offsets(scene):
    sc = scene
    a0, r0 = 300, 100
    sub = np.ascontiguousarray(sc.slc[a0:a0 + 2400, r0:r0 + 1300])
    b2 = (sub * np.complex64(0.5 + 0.5j)).astype(np.complex64)
    kw = dict(first_azimuth_line=a0, first_range_sample=r0)
    dev = _run(sc, [sub, b2], device_in=True, host_out=False, **kw)
    host = _run(sc, [sub, b2], device_in=False, host_out=True, **kw)
    _same(dev, host)
    c32 = to_complex32(sub)
    dev32 = _run(sc, [c32], device_in=False, host_out=False, **kw)
    t32 = torch.from_numpy(c32.view(np.int32)).cuda().view(torch.complex32)
    g = sc.geogrid
    ref = [torch.zeros((g.length, g.width), dtype=torch.complex64, device="cuda")]
    G.geocode_slc(ref[0], t32, sc.dem, sc.radar_grid, g, sc.orbit, sc.native_doppler, sc.image_grid_doppler,
                  sc.ellipsoid, sc.threshold, sc.maxiter, az_carrier=sc.az_carrier,
                  rg_carrier=Poly2d([[0.1, 1e-3]], x_mean=sc.radar_grid.mid_range), **kw)
    np.testing.assert_array_equal(dev32[0][0].view(np.uint64), ref[0].cpu().numpy().view(np.uint64))


def test_plan_too_small_runs_again(scene, monkeypatch):
    """A plan shrunk by 400 lines and rows: chips and splines reach beyond
    what had arrived, the kernel flags it and every band runs again."""
    sc = scene
    dev = _run(sc, [sc.slc], device_in=True, host_out=False)
    for k in list(sc.dem.__dict__.get("_gslc_dev", {})):
        sc.dem.__dict__["_gslc_dev"].pop(k)
    monkeypatch.setattr(G, "HOST_IO_MARGIN", -400)
    host = _run(sc, [sc.slc], device_in=False, host_out=True)
    assert G.L.lib().gslc_last_io_reruns(L.context(0)) == 1
    _same(dev, host)
