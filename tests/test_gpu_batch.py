"""The batched form (cbq_batch_*): many volumes in one persistent launch, from
a CUDA graph.  Every job's results must equal the single-volume path's and the
oracle's, bit for bit."""
import numpy as np
import pytest

import cubiquity_gb300 as cbq
import oracle
from cubiquity_gb300 import workloads as W

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

FIELDS = ("hit", "distance", "material", "position", "normal", "voxel", "status")


@pytest.fixture(scope="module")
def small_batch():
    torch.cuda.set_device(0)
    vols = W.batch_volumes(count=10, seed=77, edge_log2=(5, 7), rays=(500, 20000))
    jobs = []
    for v in vols:
        nodes, root = v.scene.build()
        o, d = v.make_rays()
        jobs.append((nodes, root, o, d))
    # A volume far from the origin (integer positions: launched beside the batch kernel) and an empty batch.
    from conftest import relocate
    n2, r2 = relocate(jobs[0][0], jobs[0][1], vols[0].scene.edge_log2, (1 << 30, 0, 0))
    o2 = jobs[0][2].copy()
    o2[:, 0] += np.float32(1 << 30)
    jobs.append((n2, r2, o2, jobs[0][3].copy()))
    jobs.append((jobs[1][0], jobs[1][1], np.zeros((0, 4), np.float32), np.zeros((0, 4), np.float32)))
    dags = [cbq.Dag(n, r) for n, r, _, _ in jobs]
    dev = [(torch.from_numpy(np.ascontiguousarray(o)).cuda(), torch.from_numpy(np.ascontiguousarray(d)).cuda())
           for _, _, o, d in jobs]
    return jobs, dags, dev


def _eq(a, b):
    return oracle.same_bits_nan_equal(a.cpu().numpy(), b.cpu().numpy())


def test_batch_graph_and_direct_equal_single_volume_path(small_batch, orc):
    jobs, dags, dev = small_batch
    single = [cbq.intersect_volume(g, o, d) for g, (o, d) in zip(dags, dev)]
    batch = cbq.Batch([(g, o, d) for g, (o, d) in zip(dags, dev)])
    # The far volume's rays (job 10) run beside the batch kernel, not in its ray count.
    assert batch.total_rays == sum(o.shape[0] for o, _ in dev) - dev[10][0].shape[0]
    batch.launch()
    torch.cuda.synchronize()
    for j, (a, b) in enumerate(zip(batch.outputs, single)):
        for k in FIELDS:
            assert _eq(a[k], b[k]), f"job {j} {k} (graph)"
    for out in batch.outputs:
        for v in out.values():
            v.fill_(0)
    batch.launch_direct()
    batch.launch()  # replay the graph a second time
    torch.cuda.synchronize()
    for j, (a, b) in enumerate(zip(batch.outputs, single)):
        for k in FIELDS:
            assert _eq(a[k], b[k]), f"job {j} {k} (replay)"
    # and against the oracle, job by job
    for j, ((n, r, o, d), out) in enumerate(zip(jobs, batch.outputs)):
        if o.shape[0] == 0:
            continue
        want = orc.intersect(n, orc.find_subdags(n, r), o, d)
        for k in FIELDS:
            w = want[k].astype(np.int32) if k == "material" else want[k]
            assert oracle.same_bits_nan_equal(out[k].cpu().numpy(), w), f"job {j} {k} vs oracle"
    batch.destroy()


@pytest.mark.parametrize("block,refill", [(32, 1), (64, 8), (256, 32)])
def test_batch_launch_shapes_do_not_change_results(small_batch, block, refill):
    jobs, dags, dev = small_batch
    ref = [cbq.intersect_volume(g, o, d) for g, (o, d) in zip(dags, dev)]
    batch = cbq.Batch([(g, o, d) for g, (o, d) in zip(dags, dev)])
    batch.set_config(block, refill)
    assert batch.config()["block"] == block and batch.config()["refill_min"] == refill
    batch.launch()
    torch.cuda.synchronize()
    for a, b in zip(batch.outputs, ref):
        for k in FIELDS:
            assert _eq(a[k], b[k]), k
    batch.destroy()


@pytest.mark.parametrize("registers,stack,form", [(0, cbq.STACK_LOCAL, cbq.FORM_SORTED),
                                                  (56, cbq.STACK_LOCAL, cbq.FORM_SORTED),
                                                  (0, cbq.STACK_SHARED, cbq.FORM_PERSISTENT),
                                                  (0, cbq.STACK_SHARED, cbq.FORM_SORTED)])
@pytest.mark.parametrize("block,steps", [(64, 4), (256, 16)])
def test_batch_stack_and_octant_order_do_not_change_results(small_batch, registers, stack, form, block, steps):
    """The autotuner's other axes: the descent stack in shared memory, and each
    job's rays grouped by octant before the launch (inside the graph)."""
    jobs, dags, dev = small_batch
    ref = [cbq.intersect_volume(g, o, d) for g, (o, d) in zip(dags, dev)]
    batch = cbq.Batch([(g, o, d) for g, (o, d) in zip(dags, dev)])
    batch.set_launch_config(block=block, refill_min=8, steps=steps, registers=registers, stack=stack, form=form)
    cfg = batch.config()
    assert (cfg["stack"], cfg["form"], cfg["registers"], cfg["steps"]) == (stack, form, registers, steps)
    for rep in range(2):  # graph capture, then replay
        for out in batch.outputs:
            for v in out.values():
                v.fill_(0x5A)
        batch.launch()
        torch.cuda.synchronize()
        for j, (a, b) in enumerate(zip(batch.outputs, ref)):
            for k in FIELDS:
                assert _eq(a[k], b[k]), f"job {j} {k} (launch {rep})"
    batch.destroy()


def test_batch_rejects_bad_launch_config(small_batch):
    jobs, dags, dev = small_batch
    batch = cbq.Batch([(g, o, d) for g, (o, d) in zip(dags, dev)])
    for kw in ({"block": 48}, {"refill_min": 0}, {"steps": 33}, {"registers": 48}, {"stack": 7}, {"form": 0}):
        with pytest.raises(cbq.CbqError) as e:
            batch.set_launch_config(**kw)
        assert e.value.status == 1
    batch.destroy()


def test_batch_autotune_keeps_results(small_batch):
    jobs, dags, dev = small_batch
    ref = [cbq.intersect_volume(g, o, d) for g, (o, d) in zip(dags, dev)]
    batch = cbq.Batch([(g, o, d) for g, (o, d) in zip(dags, dev)])
    cfg = batch.autotune(1)
    assert cfg["block"] in (64, 128, 256) and cfg["refill_min"] in (4, 8, 12, 16)
    assert cfg["steps"] in (4, 8, 16) and cfg["stack"] in (cbq.STACK_LOCAL, cbq.STACK_SHARED)
    assert cfg["form"] in (cbq.FORM_PERSISTENT, cbq.FORM_SORTED)
    batch.launch()
    torch.cuda.synchronize()
    for a, b in zip(batch.outputs, ref):
        for k in FIELDS:
            assert _eq(a[k], b[k]), k
    batch.destroy()


def test_one_shot_intersect_batch(small_batch):
    import ctypes
    jobs, dags, dev = small_batch
    outs = [cbq.alloc_hits(o.shape[0]) for o, _ in dev]
    arr = (cbq._Job * len(dags))()
    for i, (g, (o, d)) in enumerate(zip(dags, dev)):
        arr[i].dag = g.handle
        arr[i].rays = cbq._Rays(o.data_ptr(), d.data_ptr())
        arr[i].ray_count = o.shape[0]
        arr[i].hits = cbq._hits_struct(outs[i])
    q = cbq.Query().c()
    st = cbq.lib().cbq_intersect_batch(arr, len(dags), ctypes.byref(q), torch.cuda.current_stream().cuda_stream)
    assert st == 0
    for g, (o, d), out in zip(dags, dev, outs):
        ref = cbq.intersect_volume(g, o, d)
        for k in FIELDS:
            assert _eq(out[k], ref[k]), k


def test_batch_rejects_bad_jobs(small_batch):
    import ctypes
    jobs, dags, dev = small_batch
    o, d = dev[0]
    arr = (cbq._Job * 1)()
    arr[0].dag = dags[0].handle
    arr[0].rays = cbq._Rays(o.data_ptr() + 4, d.data_ptr())  # misaligned
    arr[0].ray_count = 4
    h = ctypes.c_void_p()
    assert cbq.lib().cbq_batch_create(arr, 1, None, ctypes.byref(h)) == 1
    arr[0].dag = None
    assert cbq.lib().cbq_batch_create(arr, 1, None, ctypes.byref(h)) == 1


@pytest.mark.parametrize("stack,form", [(cbq.STACK_LOCAL, cbq.FORM_PERSISTENT), (cbq.STACK_SHARED, cbq.FORM_SORTED)])
def test_batch_lod_and_tmax_query(small_batch, stack, form):
    """The batch's query applies to every job: with a LOD footprint the walk
    stops above the leaves (findNearestMaterial picks the material) and with
    tmax the far hits become misses, exactly as on the single-volume path."""
    jobs, dags, dev = small_batch
    kw = dict(compute_surface_properties=True, max_footprint=0.02, use_tmax=True)
    tmaxed = []
    for o, d in dev:
        o2 = o.clone()
        o2[:, 3] = 40.0
        tmaxed.append((o2, d))
    ref = [cbq.intersect_volume(g, o, d, **kw) for g, (o, d) in zip(dags, tmaxed)]
    batch = cbq.Batch([(g, o, d) for g, (o, d) in zip(dags, tmaxed)], **kw)
    batch.set_launch_config(block=128, refill_min=8, steps=8, registers=0, stack=stack, form=form)
    batch.launch()
    torch.cuda.synchronize()
    for j, (a, b) in enumerate(zip(batch.outputs, ref)):
        for k in FIELDS:
            assert _eq(a[k], b[k]), f"job {j} {k}"
    assert any(int(r["hit"].sum()) > 0 for r in ref)
    batch.destroy()


def test_batch_l2_window_on_the_graph_keeps_results(small_batch):
    """A persisting L2 window over one job's node store, set on the graph's
    kernel nodes, changes caching only: the results stay the same bits, and
    removing it leaves the next launches unchanged too."""
    jobs, dags, dev = small_batch
    ref = [cbq.intersect_volume(g, o, d) for g, (o, d) in zip(dags, dev)]
    batch = cbq.Batch([(g, o, d) for g, (o, d) in zip(dags, dev)])
    big = max(range(len(dags) - 2), key=lambda i: dags[i].device_bytes)
    for fraction in (1.0, 0.0):
        batch.set_l2_persistence(dags[big] if fraction else None, fraction)
        for out in batch.outputs:
            for v in out.values():
                v.fill_(0x3C)
        batch.launch()
        torch.cuda.synchronize()
        for j, (a, b) in enumerate(zip(batch.outputs, ref)):
            for k in FIELDS:
                assert _eq(a[k], b[k]), f"job {j} {k} (window fraction {fraction})"
    with pytest.raises(cbq.CbqError):
        batch.set_l2_persistence(dags[0], 1.5)
    batch.destroy()
