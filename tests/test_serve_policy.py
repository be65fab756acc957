"""Host logic of the serving loop: admission by HBM budget and batch slots,
first-in first-out, and latency statistics.  No GPU."""
import collections
from types import SimpleNamespace

import pytest

torch = pytest.importorskip("torch")

from isce3_gb300.serve import BYTES_PER_PX, REQUEST_OVERHEAD, AdmissionPolicy, ServeRequest, summarize  # noqa: E402


def _req(side, arrival=0.0):
    return ServeRequest(0, SimpleNamespace(length=side, width=side), arrival)


def test_admission_respects_budget_and_order():
    reqs = [_req(100), _req(200), _req(50), _req(300)]
    fp = [r.footprint for r in reqs]
    assert fp[0] == 100 * 100 * BYTES_PER_PX + REQUEST_OVERHEAD
    pol = AdmissionPolicy(budget_bytes=fp[0] + fp[1] + 10, max_in_flight=2, max_batch=8)
    q = collections.deque(reqs)
    adm, rej = pol.select(q, used_bytes=0, in_flight=0)
    assert adm == reqs[:2] and not rej and list(q) == reqs[2:]
    # the head does not fit: nothing behind it jumps the queue
    adm, rej = pol.select(q, used_bytes=fp[0] + fp[1], in_flight=1)
    assert adm == [] and list(q) == reqs[2:]
    # slots full
    adm, _ = pol.select(q, used_bytes=0, in_flight=2)
    assert adm == []
    adm, _ = pol.select(q, used_bytes=fp[0] + fp[1] - fp[2], in_flight=1)
    assert adm == [reqs[2]]


def test_admission_rejects_oversized_and_caps_batch():
    big = _req(10000)
    small = [_req(10) for _ in range(5)]
    pol = AdmissionPolicy(budget_bytes=10 ** 6, max_in_flight=4, max_batch=3)
    q = collections.deque([big] + small)
    adm, rej = pol.select(q, 0, 0)
    assert rej == [big] and big.error and adm == small[:3] and list(q) == small[3:]
    with pytest.raises(ValueError):
        AdmissionPolicy(0)


def test_summary_percentiles():
    reqs = []
    for k in range(100):
        r = _req(10, arrival=k * 0.01)
        r.t_done = r.arrival + (k + 1) * 1e-3
        reqs.append(r)
    s = summarize(reqs, batches=10, batch_sizes=[10] * 10)
    assert s["completed"] == 100 and s["output_px"] == 100 * 100
    assert abs(s["p50_ms"] - 50.5) < 1e-6 and abs(s["p99_ms"] - 99.01) < 1e-6
    assert s["mean_batch_requests"] == 10


def test_resident_store_counts_against_budget():
    """The resident store's bytes are held against the budget: a request that
    fits the budget alone but not beside the store is rejected, and the room
    left for admission shrinks by the store's size."""
    reqs = [_req(100), _req(100)]
    fp = reqs[0].footprint
    pol = AdmissionPolicy(budget_bytes=3 * fp, max_in_flight=2, max_batch=8)
    q = collections.deque(reqs)
    adm, rej = pol.select(q, used_bytes=0, in_flight=0, resident_bytes=2 * fp)
    assert adm == [reqs[0]] and not rej and list(q) == [reqs[1]]
    adm, rej = pol.select(q, used_bytes=0, in_flight=0, resident_bytes=3 * fp - 1)
    assert adm == [] and rej == [reqs[1]] and "resident" in reqs[1].error


def test_request_geo2rdr_arguments_default_to_reference_values():
    r = _req(10)
    assert r.threshold_geo2rdr == 1e-8 and r.num_iter_geo2rdr == 25
    r = ServeRequest(0, SimpleNamespace(length=4, width=4), 0.0, {}, 1e-9, 40)
    assert r.threshold_geo2rdr == 1e-9 and r.num_iter_geo2rdr == 40
