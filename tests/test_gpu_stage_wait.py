"""The one device-side wait, made to run out (gslc_ctx_set_stage_wait).

Each block of the fused and persistent kernels copies the orbit's Newton
tables into shared memory and waits for them with a deadline.  With a
deadline of one SM clock after the copy's issue every wait runs out before
its first poll: the threads read the global tables instead, the call returns
GSLC_ETIMEOUT (GslcError with that status), the outputs equal a normal run's
bit for bit, and the context stays usable.  Nothing faults or hangs: the copy
is an ordinary 12 KB bulk copy that lands, and each block waits for it
(bounded) before it finishes.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from isce3_gb300 import _lib as L  # noqa: E402
from isce3_gb300 import synth  # noqa: E402
from isce3_gb300.batch import BatchTuning, GeocodeBatch, GeocodeRequest  # noqa: E402
from isce3_gb300.geocode import geocode_slc  # noqa: E402

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)


@pytest.fixture(scope="module")
def scene():
    sc = synth.scene_c2(length=2048, width=1024, geo=256, spacing=12.0)
    sc.slc_dev = torch.from_numpy(sc.slc).cuda()
    return sc


def _outputs(sc):
    g = sc.geogrid
    return (torch.full((g.length, g.width), complex(7.0, 7.0), dtype=torch.complex64, device="cuda"),
            torch.full((g.length, g.width), 9, dtype=torch.uint8, device="cuda"))


def _plain(sc, geo, mask):
    geocode_slc(geo, sc.slc_dev, sc.dem, sc.radar_grid, sc.geogrid, sc.orbit, sc.native_doppler,
                sc.image_grid_doppler, sc.ellipsoid, sc.threshold, sc.maxiter, mask_block=mask,
                az_carrier=sc.az_carrier, rg_carrier=sc.rg_carrier)


def _same(a, b):
    assert torch.equal(a[1], b[1])
    assert torch.equal(torch.view_as_real(a[0]).view(torch.int32), torch.view_as_real(b[0]).view(torch.int32))


def test_plain_call_wait_runs_out(scene):
    ref = _outputs(scene)
    _plain(scene, *ref)
    assert (ref[1] == 1).sum().item() > 30000
    out = _outputs(scene)
    L.set_stage_wait(1)
    try:
        with pytest.raises(L.GslcError) as ei:
            _plain(scene, *out)
    finally:
        L.set_stage_wait(0)
    assert ei.value.status == L.GSLC_ETIMEOUT
    _same(out, ref)
    again = _outputs(scene)
    _plain(scene, *again)          # default deadline: no error
    _same(again, ref)


def test_persistent_batch_wait_runs_out(scene):
    ref = _outputs(scene)
    _plain(scene, *ref)

    def batch_run():
        out = _outputs(scene)
        req = GeocodeRequest(out[0], scene.slc_dev, scene.dem, scene.radar_grid, scene.geogrid, scene.orbit,
                             scene.native_doppler, scene.image_grid_doppler, scene.ellipsoid, scene.threshold,
                             scene.maxiter, dict(mask_block=out[1], az_carrier=scene.az_carrier,
                                                 rg_carrier=scene.rg_carrier))
        b = GeocodeBatch([req], "fp64", BatchTuning(tiles_per_pop=1, use_graph=False))
        return b, out

    L.set_stage_wait(1)      # read when the batch binds its requests
    try:
        b, out = batch_run()
    finally:
        L.set_stage_wait(0)
    b.launch()
    with pytest.raises(L.GslcError) as ei:
        b.wait()
    b.close()
    assert ei.value.status == L.GSLC_ETIMEOUT
    _same(out, ref)
    b, out = batch_run()
    b.launch()
    b.wait()
    b.close()
    _same(out, ref)
