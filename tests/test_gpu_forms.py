"""Launch forms and the autotuner: every form (plain, persistent, octant-sorted
persistent) x stack placement x block size gives the same bits as the plain
drop-in; the autotuner picks one of them and its cache re-applies it."""
import numpy as np
import pytest

import cubiquity_gb300 as cbq
import oracle
from cubiquity_gb300 import workloads as W

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

FIELDS = ("hit", "distance", "material", "position", "normal", "voxel", "status")


@pytest.fixture(scope="module")
def scene():
    torch.cuda.set_device(0)
    spec = W.terrain_scaled(10, 424242)
    nodes, root = spec.build()
    dag = cbq.Dag(nodes, root)
    o, d = W.camera_scaled(10, 384, 256).rays()
    prim = cbq.intersect_volume(dag, torch.from_numpy(o).cuda(), torch.from_numpy(d).cuda())
    bo, bd = W.bounce_from_hits({k: v.cpu().numpy() for k, v in prim.items()}, o.shape[0])
    rays = {"primary": (torch.from_numpy(o).cuda(), torch.from_numpy(d).cuda()),
            "bounce": (torch.from_numpy(bo).cuda(), torch.from_numpy(bd).cuda())}
    return dag, rays


def _same(a, b):
    for k in FIELDS:
        assert oracle.same_bits_nan_equal(a[k].cpu().numpy(), b[k].cpu().numpy()), k


@pytest.mark.parametrize("form", [cbq.FORM_PLAIN, cbq.FORM_PERSISTENT, cbq.FORM_SORTED])
@pytest.mark.parametrize("stack", [cbq.STACK_SHARED, cbq.STACK_LOCAL])
@pytest.mark.parametrize("block,steps", [(64, 1), (256, 3), (128, 8)])
def test_every_form_equals_the_drop_in(scene, form, stack, block, steps):
    dag, rays = scene
    scratch = cbq.scratch_for(max(o.shape[0] for o, _ in rays.values()))
    for label, (o, d) in rays.items():
        dag.set_launch_config(cbq.KERNEL_NESTED)
        want = cbq.intersect_volume(dag, o, d)  # the reference's loop structure as written
        dag.set_launch_config(cbq.KERNEL_FLAT, block, 0, 4, stack, form, steps)
        got = cbq.intersect_auto(dag, o, d, scratch)
        _same(got, want)
    dag.set_launch_config()


def test_autotune_and_cache(scene, tmp_path, monkeypatch):
    from cubiquity_gb300 import autotune
    monkeypatch.setattr(autotune, "CACHE_PATH", tmp_path / "tune.json")
    dag, rays = scene
    o, d = rays["bounce"]
    scratch = cbq.scratch_for(o.shape[0])
    out = cbq.alloc_hits(o.shape[0])
    first = autotune.tune(dag, o, d, scratch, out, repetitions=1)
    assert not first["cached"] and first["form"] in (0, 1, 2) and first["stack"] in (0, 1)
    assert first["block"] in (64, 128, 256) and first["ms"] > 0
    dag.set_launch_config()
    second = autotune.tune(dag, o, d, scratch, out)
    assert second["cached"] and second["key"] == first["key"]
    cfg = dag.launch_config()
    assert (cfg["form"], cfg["block"], cfg["stack"]) == (first["form"], first["block"], first["stack"])
    got = cbq.intersect_auto(dag, o, d, scratch)
    dag.set_launch_config(cbq.KERNEL_FLAT, 64, 0, 0, cbq.STACK_SHARED, cbq.FORM_PLAIN)
    _same(got, cbq.intersect_volume(dag, o, d))
    dag.set_launch_config()
    assert autotune.ray_mix(rays["primary"][1]) == "coherent"
    assert autotune.ray_mix(o.new_tensor(np.random.default_rng(0).normal(size=(5000, 4)).astype(np.float32))) == \
        "incoherent"


def test_scratch_checks(scene):
    dag, rays = scene
    o, d = rays["primary"]
    small = cbq.scratch_for(10)
    with pytest.raises(cbq.CbqError):
        cbq.intersect_auto(dag, o, d, small)


def test_l2_persistence_window_keeps_results(scene):
    """cbq_dag_set_l2_persistence marks the node store persisting in L2 for a
    stream (a per-context setting): results are unchanged, and 0 clears it."""
    dag, rays = scene
    o, d = rays["bounce"]
    want = cbq.intersect_volume(dag, o, d)
    stream = torch.cuda.Stream()
    dag.set_l2_persistence(1.0, stream=stream)
    with torch.cuda.stream(stream):
        got = cbq.intersect_volume(dag, o, d, stream=stream)
    stream.synchronize()
    _same(got, want)
    dag.set_l2_persistence(0.0, stream=stream)
    with pytest.raises(cbq.CbqError):
        dag.set_l2_persistence(1.5)


def test_l2_probes():
    """cbq_measure_l2: the streaming and random-sector L2 read rates used as the
    traversal's L2 roofline are finite and ordered (random 32 B sectors move
    fewer bytes per second than streaming reads)."""
    torch.cuda.set_device(0)
    stream_gbs, sectors_gsps = cbq.measure_l2(32 << 20, 5)
    assert 1000.0 < stream_gbs < 100000.0
    assert 1.0 < sectors_gsps and sectors_gsps * 32.0 < stream_gbs
    with pytest.raises(cbq.CbqError):
        cbq.measure_l2(32 << 20, 0)


@pytest.mark.parametrize("form", [cbq.FORM_PLAIN, cbq.FORM_PERSISTENT, cbq.FORM_SORTED])
@pytest.mark.parametrize("width", [384, 96, 12, 4, 12288, 383, 392])
def test_image_order_gives_the_same_bits(scene, form, width):
    """Rays dealt to warps in 4x8 tiles of an image (query image_width): the same
    bits as rays in order, every ray written once (outputs start as a sentinel).
    384 is the camera's own width; 96, 12, 4 and 12288 (one band) also tile the
    98,304 rays; 383 (not a multiple of 4) and 392 (not whole 8-row bands) are
    ignored by the launch; the sorted form keeps its octant order."""
    dag, rays = scene
    dag.set_launch_config(cbq.KERNEL_FLAT, 128, 0, 8, cbq.STACK_SHARED, form, 8)
    try:
        for label in ("primary", "bounce"):
            o, d = rays[label]
            scratch = cbq.scratch_for(o.shape[0])
            want = cbq.intersect_auto(dag, o, d, scratch)
            out = cbq.alloc_hits(o.shape[0])
            for v in out.values():
                v.view(torch.uint8).fill_(0xA5)
            got = cbq.intersect_auto(dag, o, d, scratch, out=out, image_width=width)
            _same(got, want)
            got2 = cbq.intersect_volume(dag, o, d, image_width=width)
            _same(got2, want)
    finally:
        dag.set_launch_config()


def test_image_order_through_the_host_entry_point(scene):
    """cbq_intersect_host with an image width: its chunks take the image order
    where they are whole bands; the bits equal the device call's."""
    dag, rays = scene
    o, d = rays["primary"]
    want = cbq.intersect_volume(dag, o, d)
    got = cbq.intersect_volume_host(dag, o.cpu().numpy(), d.cpu().numpy(), image_width=384)
    for k in FIELDS:
        assert oracle.same_bits_nan_equal(got[k], want[k].cpu().numpy()), k


def test_drop_in_on_concurrent_streams_and_in_a_graph(scene):
    """cbq_intersect's persistent form keeps one work counter per stream: launches
    on several streams at once, and one captured into a CUDA graph (the plain
    form there), give the plain form's bits."""
    dag, rays = scene
    o, d = rays["bounce"]
    dag.set_launch_config(cbq.KERNEL_FLAT, 64, 0, 0, cbq.STACK_LOCAL, cbq.FORM_PLAIN)
    parts = [(o[i::4].contiguous(), d[i::4].contiguous()) for i in range(4)]
    want = [cbq.intersect_volume(dag, po, pd) for po, pd in parts]
    dag.set_launch_config()
    streams = [torch.cuda.Stream() for _ in parts]
    outs = []
    for _ in range(3):  # the same streams again: their counters are reused in stream order
        outs = []
        for s_, (po, pd) in zip(streams, parts):
            with torch.cuda.stream(s_):
                outs.append(cbq.intersect_volume(dag, po, pd, stream=s_))
        torch.cuda.synchronize()
        for got, w in zip(outs, want):
            _same(got, w)
    s_ = torch.cuda.Stream()
    po, pd = parts[0]
    out = cbq.alloc_hits(po.shape[0])
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s_):
        cbq.intersect_volume(dag, po, pd, out=out, stream=s_)
    g.replay()
    torch.cuda.synchronize()
    _same(out, want[0])


@pytest.mark.parametrize("form", [cbq.FORM_PERSISTENT, cbq.FORM_SORTED])
@pytest.mark.parametrize("block,steps", [(64, 8), (128, 16), (256, 4)])
def test_register_capped_kernel_equals_the_drop_in(scene, form, block, steps):
    """The persistent local-stack kernel held to 56 registers (launch config
    registers = 56) gives the same bits; other register values are refused."""
    dag, rays = scene
    scratch = cbq.scratch_for(max(o.shape[0] for o, _ in rays.values()))
    for label, (o, d) in rays.items():
        dag.set_launch_config(cbq.KERNEL_FLAT, 64, 0, 0, cbq.STACK_LOCAL, cbq.FORM_PLAIN)
        want = cbq.intersect_volume(dag, o, d)
        dag.set_launch_config(cbq.KERNEL_FLAT, block, 0, 8, cbq.STACK_LOCAL, form, steps, registers=56)
        assert dag.launch_config()["registers"] == 56
        _same(cbq.intersect_auto(dag, o, d, scratch), want)
    with pytest.raises(cbq.CbqError):
        dag.set_launch_config(registers=48)
    dag.set_launch_config()
