"""Serving loop on the GPU: requests arriving while earlier batches run are
admitted into later batches on other streams, and every result equals the
same request geocoded alone."""
import pytest

torch = pytest.importorskip("torch")

from isce3_gb300 import synth  # noqa: E402
from isce3_gb300.core import Ellipsoid, LUT2d  # noqa: E402
from isce3_gb300.serve import GeocodeServer, ResidentStore, ServeRequest, serve_plain  # noqa: E402

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)


@pytest.fixture(scope="module")
def served():
    sc = synth.scene_serving(seed=8, n_slc=3, lines=(1024, 2048), samples=(1024, 2048), device="cuda")
    store = ResidentStore(sc.dem)
    for s in sc.slcs:
        store.add(s.key, s.slc, s.radar_grid, s.orbit, native_doppler=s.native_doppler, az_carrier=s.az_carrier,
                  rg_carrier=s.rg_carrier)
    trace = synth.serving_trace(sc, n_requests=24, rate_hz=2000.0, side=(64, 512), spacing=(10.0, 30.0), seed=9)
    return sc, store, trace


@pytest.mark.parametrize("precision,signaled,queue", [("fp64", True, False), ("ff", True, False),
                                                      ("fp64", False, False), ("fp64", True, True),
                                                      ("ff", True, True)])
def test_served_results_equal_alone(served, precision, signaled, queue):
    """Each request's outputs equal its plain call, served in the mix with
    the default batch forms (per-request kernels for two or more requests,
    the persistent queue for one) or with the persistent queue throughout."""
    from isce3_gb300.batch import BatchTuning
    sc, store, trace = served
    mixed = [ServeRequest(k, g, t) for k, g, t in trace]
    server = GeocodeServer(store, budget_bytes=2 * 10 ** 9, max_in_flight=3, max_batch=6,
                           geo2rdr_precision=precision, per_request_completion=signaled,
                           tuning=BatchTuning(use_graph=False) if queue else None)
    stats = server.serve(mixed, keep_outputs=True)
    server.close()
    assert stats["completed"] == len(trace) and stats["batches"] >= 2
    assert stats["per_request_completion"] is signaled
    assert all(r.t_admit <= r.t_done for r in mixed)
    alone = [ServeRequest(k, g, 0.0) for k, g, _ in trace]
    serve_plain(store, alone, geo2rdr_precision=precision, keep_outputs=True)
    for a, b in zip(sorted(mixed, key=lambda r: r.arrival), alone):
        assert torch.equal(a.mask, b.mask)
        assert torch.equal(torch.view_as_real(a.geo).view(torch.int32), torch.view_as_real(b.geo).view(torch.int32))
    assert stats["p99_ms"] >= stats["p50_ms"] > 0


def test_budget_limits_concurrency(served):
    sc, store, trace = served
    reqs = [ServeRequest(k, g, 0.0) for k, g, _ in trace[:8]]
    biggest = max(r.footprint for r in reqs)
    # the resident store counts against the budget: room for one request at a time
    server = GeocodeServer(store, budget_bytes=store.nbytes + biggest, max_in_flight=3, max_batch=8)
    stats = server.serve(reqs)
    assert stats["completed"] == 8
    assert stats["max_concurrent_batches"] >= 1


def test_served_requests_match_oracle(oracle_mod):
    """Requests on 30 m UTM grids, served by continuous batching over
    resident SLCs deramped once at load, against the oracle geocoding the
    original SLC with its carriers: masks exact, values within tolerance."""
    import numpy as np
    from oracle.compare import assert_parity, compare
    sc = synth.scene_serving(seed=12, n_slc=2, lines=(1536, 2048), samples=(1536, 2048), device="cuda")
    store = ResidentStore(sc.dem)
    for s in sc.slcs:
        store.add(s.key, s.slc, s.radar_grid, s.orbit, native_doppler=s.native_doppler, az_carrier=s.az_carrier,
                  rg_carrier=s.rg_carrier)
    trace = synth.serving_trace(sc, n_requests=6, rate_hz=5000.0, side=(128, 384), spacing=(30.0, 30.0), seed=13)
    reqs = []
    for key, g, t in trace:
        shape = (g.length, g.width)
        reqs.append(ServeRequest(key, g, t, dict(az_index_block=torch.empty(shape, dtype=torch.float64, device="cuda"),
                                                 rg_index_block=torch.empty(shape, dtype=torch.float64, device="cuda"))))
    server = GeocodeServer(store, budget_bytes=2 * 10 ** 9, max_in_flight=2, max_batch=4)
    stats = server.serve(reqs, keep_outputs=True)
    server.close()
    assert stats["completed"] == len(reqs)
    n_valid = 0
    for r in reqs:
        s = sc.slcs[r.slc_key]
        g = r.geogrid
        shape = (g.length, g.width)
        ora = dict(geo=np.zeros(shape, np.complex64), mask=np.zeros(shape, np.uint8), az=np.zeros(shape),
                   rg=np.zeros(shape))
        oracle_mod.geocode_slc(ora["geo"], s.slc.cpu().numpy(), sc.dem, s.radar_grid, g, s.orbit,
                               s.native_doppler, LUT2d(), Ellipsoid(), r.threshold_geo2rdr, r.num_iter_geo2rdr,
                               mask_block=ora["mask"], az_index_block=ora["az"], rg_index_block=ora["rg"],
                               az_carrier=s.az_carrier, rg_carrier=s.rg_carrier)
        gg, gm = r.geo.cpu().numpy(), r.mask.cpu().numpy()
        ga, gr = r.kwargs["az_index_block"].cpu().numpy(), r.kwargs["rg_index_block"].cpu().numpy()
        rep = compare(gg, ora["geo"], ga, ora["az"], gr, ora["rg"], gm, ora["mask"])
        print(g.spacing_x, shape, rep)
        assert g.spacing_x == 30.0
        assert_parity(rep, max_flip_fraction=1e-3)
        n_valid += rep["n_valid"]
    assert n_valid > 50000
