"""Full-size parity of the batched, served and pathtracer forms.

The smaller tests (test_gpu_batch, test_gpu_server, test_gpu_pathtrace) check
the same code on volumes of edge 2^5..2^9.  These run the benchmark workloads
themselves and compare every ray's hit record with the oracle (the C
restatement of the reference's intersectVolume, raytracing.cpp:397-478, pinned
to the reference by tests/golden): bit for bit on hit, distance, material,
position, normal, voxel and status, NaN payloads aside.

  * batch-64: the 64 volumes of edge 2^7..2^11 (730 MB of node stores) and
    their 10.9 M rays, through one autotuned persistent launch replayed from a
    CUDA graph;
  * serve-8: the 8 resident terrain volumes (edges 1024..4096) and the first
    requests of the serving stream (70% tmax-bounded collision rays, 30% view
    rays), all submitted at once to a server so that they are grouped,
    overlapped and admitted by memory as in the benchmark;
  * city-8192: every extension and shadow wave of a reduced frame of the
    pathtracer (480x270, 2 samples per pixel, 4 bounces, LOD 0.0035) on the
    8192^3 city.
"""
import numpy as np
import pytest

import cubiquity_gb300 as cbq
import oracle
from cubiquity_gb300 import workloads as W

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

FIELDS = ("hit", "distance", "material", "position", "normal", "voxel", "status")


def _mismatched_rays(got: dict, want: dict, fields=FIELDS) -> np.ndarray:
    """Indices of rays whose record differs in any field (NaN equals NaN)."""
    n = want["hit"].shape[0]
    bad = np.zeros(n, bool)
    for k in fields:
        if k not in got:
            continue
        g = np.ascontiguousarray(got[k])
        w = np.ascontiguousarray(want[k])
        if k == "material":
            g = g.astype(np.uint32)
            w = w.astype(np.uint32)
        g = g.reshape(n, -1)
        w = w.reshape(n, -1)
        if g.dtype.kind == "f":
            diff = (g.view(np.uint32) != w.view(np.uint32)) & ~(np.isnan(g) & np.isnan(w))
        else:
            diff = g != w
        bad |= diff.any(axis=1)
    return np.nonzero(bad)[0]


def test_batch64_every_job_matches_the_oracle(orc):
    torch.cuda.set_device(0)
    vols = W.batch_volumes()
    jobs = []
    for v in vols:
        nodes, root = v.scene.build()
        o, d = v.make_rays()
        jobs.append((nodes, root, o, d))
    assert len(jobs) == 64 and sum(j[2].shape[0] for j in jobs) == 10_900_063
    dags = [cbq.Dag(n, r) for n, r, _, _ in jobs]
    dev = [(torch.from_numpy(o).cuda(), torch.from_numpy(d).cuda()) for _, _, o, d in jobs]
    batch = cbq.Batch([(g, o, d) for g, (o, d) in zip(dags, dev)])
    batch.autotune(1)
    for out in batch.outputs:
        for t in out.values():
            t.fill_(0xAB)
    batch.launch()
    torch.cuda.synchronize()
    total = mismatched = 0
    first_bad = []
    for j, ((nodes, root, o, d), out) in enumerate(zip(jobs, batch.outputs)):
        want = orc.intersect(nodes, orc.find_subdags(nodes, root), o, d)
        got = {k: v.cpu().numpy() for k, v in out.items()}
        bad = _mismatched_rays(got, want)
        total += o.shape[0]
        mismatched += bad.size
        if bad.size and len(first_bad) < 5:
            first_bad.append((j, bad[:5].tolist()))
    batch.destroy()
    for g in dags:
        g.destroy()
    assert total == 10_900_063
    assert mismatched == 0, f"{mismatched} of {total} rays differ from the oracle (job, rays): {first_bad}"


def test_serve8_requests_in_the_mix_match_the_oracle(orc):
    torch.cuda.set_device(0)
    scenes = W.serve_volumes()
    vols = []
    for i, s in enumerate(scenes):
        nodes, root = s.build()
        pools = W.serve_ray_pools(s, 1 << 19, 724, 7000 + i)
        vols.append((nodes, root, cbq.Dag(nodes, root), pools))
    assert sorted({1 << s.edge_log2 for s in scenes}) == [1024, 2048, 4096]
    # The oracle over each whole pool: a ray's record does not depend on the
    # request that carries it.
    want = []
    for nodes, root, _, ((co, cd), (vo, vd)) in vols:
        sd = orc.find_subdags(nodes, root)
        want.append((orc.intersect(nodes, sd, co, cd, use_tmax=True), orc.intersect(nodes, sd, vo, vd)))
    reqs = W.serve_requests(300, (1 << 19, 724 * 724), seed=1234)
    server = cbq.Server(device_memory_budget=2 << 30, max_inflight_launches=8, max_batch_requests=128,
                        max_batch_rays=4 << 20)
    queries = {True: cbq.Query(True, cbq.MAX_FOOTPRINT_DISABLED, True), False: cbq.Query()}
    tickets = []
    for r in reqs:
        _, _, dag, ((co, cd), (vo, vd)) = vols[r.volume]
        o, d = (co, cd) if r.collision else (vo, vd)
        sl = slice(r.start, r.start + r.count)
        t, out = server.submit(dag, o[sl], d[sl], queries[r.collision])
        tickets.append((t, out, r))
    rays = mismatched = 0
    first_bad = []
    for t, out, r in tickets:
        assert server.wait(t) == 0
        w = want[r.volume][0 if r.collision else 1]
        sl = slice(r.start, r.start + r.count)
        bad = _mismatched_rays(out, {k: v[sl] for k, v in w.items()})
        rays += r.count
        mismatched += bad.size
        if bad.size and len(first_bad) < 5:
            first_bad.append((r, bad[:5].tolist()))
    st = server.stats()
    server.close()
    for _, _, dag, _ in vols:
        dag.destroy()
    assert st["completed"] == len(reqs) and st["rays_completed"] == rays
    assert st["launches"] < len(reqs), "requests submitted together should share launches"
    assert sum(r.collision for r in reqs) > 0 and sum(not r.collision for r in reqs) > 0
    assert mismatched == 0, f"{mismatched} of {rays} rays differ from the oracle: {first_bad}"


def test_city8192_every_wave_matches_the_oracle(orc):
    torch.cuda.set_device(0)
    nodes, root = W.CITY_8192.build()
    dag = cbq.Dag(nodes, root)
    eye, target = W.city_camera(13)
    rec = cbq.WaveRecorder()
    _, stats = cbq.pathtrace(dag, 480, 270, 2, 4, eye, target, W.city_materials(), max_footprint=0.0035, seed=1,
                             on_wave=rec)
    sd = orc.find_subdags(nodes, root)
    checked = mismatched = 0
    first_bad = []
    for kind, depth, sample, o, d, hits, (cs, mf) in rec.waves:
        want = orc.intersect(nodes, sd, o, d, cs, mf)
        bad = _mismatched_rays(hits, want)
        checked += o.shape[0]
        mismatched += bad.size
        if bad.size and len(first_bad) < 5:
            first_bad.append((kind, depth, sample, bad[:5].tolist()))
    dag.destroy()
    assert {w[0] for w in rec.waves} == {0, 1} and max(w[1] for w in rec.waves) >= 3
    assert checked == stats["extension_rays"] + stats["shadow_rays"] and checked > 480 * 270 * 2
    assert mismatched == 0, f"{mismatched} of {checked} traversals differ from the oracle: {first_bad}"
