"""The request server (cbq_server_*): continuous batching over resident DAGs.

Each result must be the same alone (cbq_intersect_host on that request only)
and in the mix (submitted together with many others, batched into shared
launches, overlapping on the device)."""
import threading

import numpy as np
import pytest

import cubiquity_gb300 as cbq
import oracle
from cubiquity_gb300 import workloads as W

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

FIELDS = ("hit", "distance", "material", "position", "normal", "voxel", "status")


@pytest.fixture(scope="module")
def served():
    torch.cuda.set_device(0)
    scenes = [W.terrain_scaled(k, 500 + i) for i, k in enumerate((6, 7, 8, 7))]
    dags, pools = [], []
    for i, s in enumerate(scenes):
        nodes, root = s.build()
        dags.append(cbq.Dag(nodes, root))
        pools.append(W.serve_ray_pools(s, 40000, 128, 1000 + i))
    return dags, pools


def _query(collision):
    return cbq.Query(True, cbq.MAX_FOOTPRINT_DISABLED, use_tmax=collision)


def _same(a, b):
    for k in FIELDS:
        assert oracle.same_bits_nan_equal(a[k], b[k]), k


def test_each_result_is_the_same_alone_and_in_the_mix(served):
    dags, pools = served
    reqs = W.serve_requests(60, (40000, 128 * 128), seed=7, rays=(1, 20000), volumes=len(dags))
    server = cbq.Server(device_memory_budget=64 << 20, max_inflight_launches=3, max_batch_requests=16,
                        max_batch_rays=50000)
    tickets = []
    for r in reqs:
        (co, cd), (vo, vd) = pools[r.volume]
        o, d = (co, cd) if r.collision else (vo, vd)
        sl = slice(r.start, r.start + r.count)
        t, out = server.submit(dags[r.volume], o[sl], d[sl], _query(r.collision))
        tickets.append((t, out, r))
    for t, out, r in tickets:
        assert server.wait(t) == 0
        (co, cd), (vo, vd) = pools[r.volume]
        o, d = (co, cd) if r.collision else (vo, vd)
        sl = slice(r.start, r.start + r.count)
        alone = cbq.intersect_volume_host(dags[r.volume], o[sl], d[sl], use_tmax=r.collision)
        _same(out, alone)
    st = server.stats()
    assert st["completed"] == len(reqs) and st["rays_completed"] == sum(r.count for r in reqs)
    assert 0 < st["launches"] <= len(reqs)
    assert st["latency_p50_us"] > 0 and st["latency_p99_us"] >= st["latency_p50_us"]
    server.close()


def test_queued_requests_share_launches(served):
    """A request that finds a launch slot free is launched at once by the
    submitting thread; requests that arrive while every slot is busy queue and
    leave together in one launch."""
    dags, pools = served
    (co, cd), _ = pools[2]
    # 4 M rays in page-locked buffers (submit returns at once) occupy the only slot; the small
    # requests' buffers are pageable (their hits are copied back by the completion thread).
    big_o, big_d = _pinned(np.tile(co, (100, 1))), _pinned(np.tile(cd, (100, 1)))
    big_out = {k: _pinned(v) for k, v in cbq.alloc_host_hits(big_o.shape[0]).items()}
    server = cbq.Server(device_memory_budget=1 << 30, max_inflight_launches=1, max_batch_requests=64)
    t0, big = server.submit(dags[2], big_o, big_d, _query(True), out=big_out)
    small = [server.submit(dags[k % len(dags)], pools[k % len(dags)][0][0][k * 500:(k + 1) * 500],
                           pools[k % len(dags)][0][1][k * 500:(k + 1) * 500], _query(True)) for k in range(20)]
    assert server.wait(t0) == 0
    for t, _ in small:
        assert server.wait(t) == 0
    st = server.stats()
    assert st["completed"] == 21 and st["launches"] < 21
    for k, (t, out) in enumerate(small):
        (co_k, cd_k), _ = pools[k % len(dags)]
        _same(out, cbq.intersect_volume_host(dags[k % len(dags)], co_k[k * 500:(k + 1) * 500],
                                             cd_k[k * 500:(k + 1) * 500], use_tmax=True))
    server.close()


def test_collision_rays_match_the_oracle(served, orc):
    dags, pools = served
    (co, cd), _ = pools[1]
    nodes, root = W.terrain_scaled(7, 501).build()
    server = cbq.Server(device_memory_budget=32 << 20)
    t, out = server.submit(dags[1], co[:5000], cd[:5000], _query(True))
    server.wait(t)
    want = orc.intersect(nodes, orc.find_subdags(nodes, root), co[:5000], cd[:5000], use_tmax=True)
    for k in FIELDS:
        w = want[k]
        assert oracle.same_bits_nan_equal(out[k].astype(w.dtype) if k == "material" else out[k], w), k
    server.close()


def test_submissions_from_several_threads(served):
    dags, pools = served
    server = cbq.Server(device_memory_budget=64 << 20, max_inflight_launches=4)
    results = {}
    errors = []

    def worker(w):
        try:
            for k in range(10):
                (co, cd), _ = pools[(w + k) % len(dags)]
                sl = slice(1000 * k, 1000 * k + 777 + 100 * w)
                t, out = server.submit(dags[(w + k) % len(dags)], co[sl], cd[sl], _query(True))
                server.wait(t)
                results[(w, k)] = (out, (w + k) % len(dags), sl)
        except Exception as e:  # noqa: BLE001
            errors.append(e)

    th = [threading.Thread(target=worker, args=(w,)) for w in range(4)]
    for x in th:
        x.start()
    for x in th:
        x.join()
    assert not errors
    for (w, k), (out, v, sl) in results.items():
        (co, cd), _ = pools[v]
        _same(out, cbq.intersect_volume_host(dags[v], co[sl], cd[sl], use_tmax=True))
    server.close()


def test_cancel_queued_request(served):
    dags, pools = served
    (co, cd), _ = pools[0]
    # One launch slot and room for one request at a time: later requests queue.
    server = cbq.Server(device_memory_budget=1 << 20, max_inflight_launches=1)
    tickets = [server.submit(dags[0], co[:9000], cd[:9000])[0] for _ in range(6)]
    st = server.cancel(tickets[-1])
    assert st in (0, 7)  # cancelled while queued, or (if the GPU raced ahead) already launched
    for t in tickets[:-1]:
        assert server.wait(t) == 0
    if st == 0:
        with pytest.raises(cbq.CbqError) as e:
            server.wait(tickets[-1])
        assert e.value.status == 9  # CBQ_ERR_CANCELLED
    else:
        assert server.wait(tickets[-1]) == 0
    assert server.cancel(tickets[0]) == 8  # finished and collected: unknown
    server.close()


def test_admission_capacity_timeout_and_shutdown(served):
    dags, pools = served
    (co, cd), _ = pools[0]
    server = cbq.Server(device_memory_budget=1 << 20)  # about 13k rays of buffers
    with pytest.raises(cbq.CbqError) as e:
        server.submit(dags[0], co[:20000], cd[:20000])
    assert e.value.status == 10  # CBQ_ERR_CAPACITY: could never be admitted
    # Requests that together exceed the budget are admitted one after another.
    tickets = [server.submit(dags[0], co[i * 9000:(i + 1) * 9000], cd[i * 9000:(i + 1) * 9000])[0]
               for i in range(4)]
    for t in tickets:
        assert server.wait(t) == 0
    with pytest.raises(cbq.CbqError) as e:
        server.wait(123456789)
    assert e.value.status == 8  # unknown ticket
    t0, _ = server.submit(dags[0], co[:0], cd[:0])  # empty request completes at once
    assert server.wait(t0, 0) == 0
    # Destroy with work queued: everything finishes first.
    pending = [server.submit(dags[1], co[:5000], cd[:5000])[1] for _ in range(5)]
    server.close()
    want = cbq.intersect_volume_host(dags[1], co[:5000], cd[:5000])
    for out in pending:
        _same(out, want)


def _pinned(a):
    return torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()


def test_page_locked_requests_are_served_in_place(served):
    """With in_place, requests whose buffers are all page-locked host memory are
    traversed in host memory (no copies, no budget); the hits equal the staged
    path's."""
    dags, pools = served
    (co, cd), (vo, vd) = pools[2]
    cases = [(co[:7000], cd[:7000], True), (vo[100:5100], vd[100:5100], False), (co[9001:9002], cd[9001:9002], True)]
    direct = cbq.Server(device_memory_budget=1 << 20, in_place=True)  # too small for these if staged
    staged = cbq.Server(device_memory_budget=64 << 20)
    for o, d, coll in cases:
        po, pd = _pinned(o), _pinned(d)
        out = {k: _pinned(v) for k, v in cbq.alloc_host_hits(o.shape[0]).items()}
        t, got = direct.submit(dags[2], po, pd, _query(coll), out=out)
        assert direct.wait(t) == 0
        t2, want = staged.submit(dags[2], po, pd, _query(coll))
        assert staged.wait(t2) == 0
        _same(got, want)
        _same(got, cbq.intersect_volume_host(dags[2], o, d, use_tmax=coll))
    assert direct.stats()["direct_requests"] == len(cases)
    assert staged.stats()["direct_requests"] == 0
    # Pageable outputs: the request is staged (and still correct).
    t, got = direct.submit(dags[2], _pinned(co[:2000]), _pinned(cd[:2000]), _query(True))
    assert direct.wait(t) == 0
    _same(got, cbq.intersect_volume_host(dags[2], co[:2000], cd[:2000], use_tmax=True))
    assert direct.stats()["direct_requests"] == len(cases)
    direct.close()
    staged.close()


def test_native_replay_of_a_request_trace(served):
    """cbq_server_replay submits a trace at its arrival times from native
    threads; with a buffer ring smaller than the trace, a request reuses the
    buffers of the one `ring` places earlier only after it has completed, so
    every request's hits can be checked as they land (here each ring slot is
    checked after the replay against the last request that used it)."""
    dags, pools = served
    reqs = W.serve_requests(120, (40000, 128 * 128), seed=11, rays=(1, 9000), volumes=len(dags))
    ring = 16
    outs = [cbq.alloc_host_hits(9000) for _ in range(ring)]
    trace = np.zeros(len(reqs), cbq.REQUEST_DTYPE)
    keep = []
    for k, r in enumerate(reqs):
        (co, cd), (vo, vd) = pools[r.volume]
        o, d = (co, cd) if r.collision else (vo, vd)
        o, d = np.ascontiguousarray(o[r.start:r.start + r.count]), np.ascontiguousarray(d[r.start:r.start + r.count])
        keep.append((o, d))
        trace[k]["dag"] = dags[r.volume].handle.value
        trace[k]["origin_tmax"] = o.ctypes.data
        trace[k]["direction"] = d.ctypes.data
        trace[k]["ray_count"] = r.count
        trace[k]["compute_surface"] = 1
        trace[k]["max_footprint"] = cbq.MAX_FOOTPRINT_DISABLED
        trace[k]["flags"] = cbq.QUERY_TMAX if r.collision else 0
        for f in cbq.HIT_FIELDS:
            trace[k][f] = outs[k % ring][f].ctypes.data
    arrivals = np.cumsum(np.full(len(reqs), 2e-4))  # 5k requests/s
    server = cbq.Server(device_memory_budget=64 << 20, max_inflight_launches=3, max_batch_requests=16)
    res = server.replay(trace, arrivals, ring)
    assert res["submitted"] == len(reqs) and res["failed"] == 0
    assert res["wall_seconds"] >= arrivals[-1]
    assert res["lateness_us"].shape == (len(reqs),) and (res["lateness_us"] >= 0).all()
    st = server.stats()
    assert st["completed"] == len(reqs) and st["latency_p99_us"] > 0
    for slot in range(ring):
        k = max(k for k in range(len(reqs)) if k % ring == slot)
        r = reqs[k]
        o, d = keep[k]
        want = cbq.intersect_volume_host(dags[r.volume], o, d, use_tmax=r.collision)
        _same({f: v[: r.count] for f, v in outs[slot].items()}, want)
    # Arrival times must not decrease.
    with pytest.raises(cbq.CbqError):
        server.replay(trace[:2], np.array([1e-3, 0.0]), ring)
    server.close()
