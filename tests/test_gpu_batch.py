"""Batched form: one persistent, graph-captured launch over uneven bursts
gives, for every burst, exactly the output of its plain geocode_slc call."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from isce3_gb300 import synth  # noqa: E402
from isce3_gb300.batch import BatchTuning, GeocodeBatch, GeocodeRequest, HostFlags  # noqa: E402
from isce3_gb300.geocode import geocode_slc  # noqa: E402

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)


@pytest.fixture(scope="module")
def bursts():
    return synth.scene_bursts(seed=5, n_az=3, n_sw=2, grid_px=1500, spacing=30.0, lines=(300, 420),
                              samples=(2400, 3000), device="cuda")


def _outputs(sc):
    outs = []
    for b in sc.bursts:
        w = b.window
        outs.append((torch.empty((w.length, w.width), dtype=torch.complex64, device="cuda"),
                     torch.empty((w.length, w.width), dtype=torch.uint8, device="cuda")))
    return outs


def _requests(sc, outs):
    return [GeocodeRequest(o[0], b.slc, sc.dem, b.radar_grid, b.window, sc.orbit, sc.native_doppler,
                           sc.image_grid_doppler, sc.ellipsoid, sc.threshold, sc.maxiter,
                           dict(mask_block=o[1], az_carrier=b.az_carrier, rg_carrier=b.rg_carrier))
            for b, o in zip(sc.bursts, outs)]


def _plain(sc, precision):
    outs = _outputs(sc)
    for b, (g, m) in zip(sc.bursts, outs):
        geocode_slc(g, b.slc, sc.dem, b.radar_grid, b.window, sc.orbit, sc.native_doppler, sc.image_grid_doppler,
                    sc.ellipsoid, sc.threshold, sc.maxiter, mask_block=m, az_carrier=b.az_carrier,
                    rg_carrier=b.rg_carrier, geo2rdr_precision=precision)
    return outs


def _same(a, b):
    for (g0, m0), (g1, m1) in zip(a, b):
        assert torch.equal(m0, m1)
        assert torch.equal(torch.view_as_real(g0).view(torch.int32), torch.view_as_real(g1).view(torch.int32))


@pytest.mark.parametrize("precision,graph,pop,per_request", [("fp64", True, 2, False), ("ff", True, 4, False),
                                                              ("fp64", False, 1, False), ("fp64", True, 0, True),
                                                              ("ff", False, 0, True)])
def test_batch_equals_plain_calls(bursts, precision, graph, pop, per_request):
    ref = _plain(bursts, precision)
    outs = _outputs(bursts)
    batch = GeocodeBatch(_requests(bursts, outs), precision,
                         BatchTuning(tiles_per_pop=pop or 2, use_graph=graph, per_request=per_request))
    info = batch.info()
    n = len(bursts.bursts)
    assert info["tiles"] > 0 and info["launches_per_run"] == (2 * n if per_request else n + 1)
    for _ in range(2):                       # a replay recomputes the same bits
        for g, m in outs:
            g.fill_(0)
            m.fill_(0)
        batch.run()
        _same(ref, outs)
    valid = sum(int((m == 1).sum()) for _, m in outs)
    assert valid > 0.2 * sum(m.numel() for _, m in outs)
    batch.close()


def test_batch_legendre_orbit_equals_plain_calls(bursts):
    """A Legendre orbit in the persistent kernel: its tables are the state
    vectors (no segment tables to stage), every iterate interpolates them;
    each burst equals its plain call."""
    import copy
    from isce3_gb300.core import Orbit, OrbitInterpMethod
    sc = copy.copy(bursts)
    o = sc.orbit
    sc.orbit = Orbit.from_arrays(o.t0, o.spacing, o.position, o.velocity, o.reference_epoch,
                                 OrbitInterpMethod.LEGENDRE)
    ref = _plain(sc, "ff")
    outs = _outputs(sc)
    batch = GeocodeBatch(_requests(sc, outs), "ff", BatchTuning(tiles_per_pop=2, use_graph=True))
    batch.run()
    _same(ref, outs)
    valid = sum(int((m == 1).sum()) for _, m in outs)
    assert valid > 0.2 * sum(m.numel() for _, m in outs)
    batch.close()


@pytest.mark.parametrize("graph,per_request", [(True, False), (False, False), (True, True)])
def test_batch_request_flags(bursts, graph, per_request):
    """Per-request completion words: every request's word is 1 once the
    batch has run, cleared words are set again by a replay, and the outputs
    are those of the plain calls."""
    ref = _plain(bursts, "fp64")
    outs = _outputs(bursts)
    n = len(bursts.bursts)
    flags = HostFlags(n + 3)
    batch = GeocodeBatch(_requests(bursts, outs), "fp64",
                         BatchTuning(tiles_per_pop=1, use_graph=graph, per_request=per_request), done_flags=flags)
    for _ in range(2):
        flags.clear()
        batch.run()
        assert flags.array[:n].tolist() == [1] * n
        assert flags.array[n:].tolist() == [0, 0, 0]      # words past the batch untouched
        _same(ref, outs)
    batch.close()
    with pytest.raises(ValueError):
        GeocodeBatch(_requests(bursts, outs), "fp64", done_flags=HostFlags(n - 1))
    flags.close()


def test_batch_rejects_host_arrays(bursts):
    b = bursts.bursts[0]
    w = b.window
    geo = np.zeros((w.length, w.width), np.complex64)
    req = GeocodeRequest(geo, b.slc, bursts.dem, b.radar_grid, w, bursts.orbit, bursts.native_doppler,
                         bursts.image_grid_doppler, bursts.ellipsoid, 1e-8, 25)
    with pytest.raises(ValueError):
        GeocodeBatch([req])


def test_ff_batch_with_a_doppler_request_runs_fp64(bursts):
    """The float-float Newton covers zero image-grid Doppler only.  A
    float-float batch holding one request with a non-zero image-grid Doppler
    runs every request in FP64, so each output equals its plain FP64 call."""
    from isce3_gb300.core import LUT2d
    b0 = bursts.bursts[0]
    rr = np.linspace(b0.radar_grid.starting_range - 5e4, b0.radar_grid.starting_range + 2e5, 8)
    tt = np.linspace(bursts.orbit.t0, bursts.orbit.t0 + bursts.orbit.spacing * (bursts.orbit.size - 1), 8)
    dop = LUT2d(rr, tt, np.full((8, 8), 12.0), "bilinear", False)
    img = [dop] + [bursts.image_grid_doppler] * (len(bursts.bursts) - 1)
    ref = _outputs(bursts)
    for b, (g, m), d in zip(bursts.bursts, ref, img):
        geocode_slc(g, b.slc, bursts.dem, b.radar_grid, b.window, bursts.orbit, bursts.native_doppler, d,
                    bursts.ellipsoid, bursts.threshold, bursts.maxiter, mask_block=m, az_carrier=b.az_carrier,
                    rg_carrier=b.rg_carrier, geo2rdr_precision="fp64")
    outs = _outputs(bursts)
    reqs = [GeocodeRequest(o[0], b.slc, bursts.dem, b.radar_grid, b.window, bursts.orbit, bursts.native_doppler, d,
                           bursts.ellipsoid, bursts.threshold, bursts.maxiter,
                           dict(mask_block=o[1], az_carrier=b.az_carrier, rg_carrier=b.rg_carrier))
            for b, o, d in zip(bursts.bursts, outs, img)]
    batch = GeocodeBatch(reqs, "ff", BatchTuning(tiles_per_pop=2))
    batch.run()
    _same(ref, outs)
    batch.close()


@pytest.mark.parametrize("precision", ["fp64", "ff"])
def test_cband_tops_bursts_match_oracle(oracle_mod, precision):
    """C-band TOPS bursts (0.0555 m, 2.33 m range spacing, quadratic azimuth
    steering carrier) on a 10 m UTM grid, geocoded in one persistent batch,
    against the oracle run on the same bursts: masks exact, values within the
    parity tolerance, splits and flips bounded."""
    from oracle.compare import assert_parity, compare
    sc = synth.scene_bursts(seed=6, n_az=2, n_sw=2, grid_px=4000, spacing=10.0, lines=(300, 380),
                            samples=(2200, 2600), device="cuda")
    bursts = sc.bursts[:3]
    outs, reqs = [], []
    for b in bursts:
        w = b.window
        shape = (w.length, w.width)
        o = dict(geo=torch.empty(shape, dtype=torch.complex64, device="cuda"),
                 mask=torch.empty(shape, dtype=torch.uint8, device="cuda"),
                 az=torch.empty(shape, dtype=torch.float64, device="cuda"),
                 rg=torch.empty(shape, dtype=torch.float64, device="cuda"))
        outs.append(o)
        reqs.append(GeocodeRequest(o["geo"], b.slc, sc.dem, b.radar_grid, w, sc.orbit, sc.native_doppler,
                                   sc.image_grid_doppler, sc.ellipsoid, sc.threshold, sc.maxiter,
                                   dict(mask_block=o["mask"], az_index_block=o["az"], rg_index_block=o["rg"],
                                        az_carrier=b.az_carrier, rg_carrier=b.rg_carrier)))
    batch = GeocodeBatch(reqs, precision, BatchTuning(tiles_per_pop=2, use_graph=True))
    batch.launch()
    batch.wait()
    n_valid = 0
    for b, o in zip(bursts, outs):
        w = b.window
        shape = (w.length, w.width)
        ora = dict(geo=np.zeros(shape, np.complex64), mask=np.zeros(shape, np.uint8), az=np.zeros(shape),
                   rg=np.zeros(shape))
        oracle_mod.geocode_slc(ora["geo"], b.slc.cpu().numpy(), sc.dem, b.radar_grid, w, sc.orbit,
                               sc.native_doppler, sc.image_grid_doppler, sc.ellipsoid, sc.threshold, sc.maxiter,
                               mask_block=ora["mask"], az_index_block=ora["az"], rg_index_block=ora["rg"],
                               az_carrier=b.az_carrier, rg_carrier=b.rg_carrier)
        g = {k: v.cpu().numpy() for k, v in o.items()}
        r = compare(g["geo"], ora["geo"], g["az"], ora["az"], g["rg"], ora["rg"], g["mask"], ora["mask"])
        print(r)
        assert_parity(r, max_flip_fraction=1e-3)
        n_valid += r["n_valid"]
    batch.close()
    assert n_valid > 100000
