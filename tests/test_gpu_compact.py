"""The compact node store on the device (LAYOUT_COMPACT): the same traversal
decisions, so the same bits as the reference layout and the oracle, in every
launch form, query, batch and the server; fewer node loads."""
import numpy as np
import pytest

import cubiquity_gb300 as cbq
import oracle
from cubiquity_gb300 import workloads as W

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

FIELDS = ("hit", "distance", "material", "position", "normal", "voxel", "status")


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _same(a, b, what=""):
    for k in FIELDS:
        x, y = a[k], b[k]
        x = x.cpu().numpy() if hasattr(x, "cpu") else x
        y = y.cpu().numpy() if hasattr(y, "cpu") else y
        if k == "material":
            x, y = x.astype(np.uint32), y.astype(np.uint32)
        assert oracle.same_bits_nan_equal(x, y), f"{what}: {k}"


@pytest.fixture(scope="module")
def terrain():
    torch.cuda.set_device(0)
    nodes, root = W.terrain_scaled(10, 424242).build()
    ref = cbq.Dag(nodes, root)
    cmp = cbq.Dag(nodes, root, cbq.LAYOUT_COMPACT)
    assert ref.layout == cbq.LAYOUT_REFERENCE and cmp.layout == cbq.LAYOUT_COMPACT
    assert cmp.device_bytes < ref.device_bytes
    o, d = W.camera_scaled(10, 320, 240).rays()
    prim = cbq.intersect_volume(ref, _dev(o), _dev(d))
    bo, bd = W.bounce_from_hits({k: v.cpu().numpy() for k, v in prim.items()}, o.shape[0])
    rays = {"primary": (_dev(o), _dev(d)), "bounce": (_dev(bo), _dev(bd))}
    return nodes, root, ref, cmp, rays


@pytest.mark.parametrize("form", [cbq.FORM_PLAIN, cbq.FORM_PERSISTENT, cbq.FORM_SORTED])
@pytest.mark.parametrize("stack", [cbq.STACK_SHARED, cbq.STACK_LOCAL])
@pytest.mark.parametrize("block,steps", [(64, 1), (256, 8)])
def test_every_form_equals_the_reference_layout(terrain, form, stack, block, steps):
    nodes, root, ref, cmp, rays = terrain
    scratch = cbq.scratch_for(max(o.shape[0] for o, _ in rays.values()))
    for label, (o, d) in rays.items():
        want = cbq.intersect_volume(ref, o, d)
        cmp.set_launch_config(cbq.KERNEL_FLAT, block, 0, 4, stack, form, steps)
        _same(cbq.intersect_auto(cmp, o, d, scratch), want, f"{label} form {form} stack {stack}")
    cmp.set_launch_config()


@pytest.mark.parametrize("cs,mf,tmax", [(False, -1.0, False), (True, 0.01, False), (True, 0.002, False),
                                        (True, -1.0, True)])
def test_queries_equal_the_oracle(terrain, orc, cs, mf, tmax):
    nodes, root, ref, cmp, rays = terrain
    o, d = rays["bounce"]
    o, d = o[:20000].clone(), d[:20000].clone()
    if tmax:
        o[:, 3] = 40.0
    got = cbq.intersect_volume(cmp, o, d, cs, mf, use_tmax=tmax)
    want = orc.intersect(nodes, orc.find_subdags(nodes, root), o.cpu().numpy(), d.cpu().numpy(), cs, mf,
                         use_tmax=tmax)
    _same(got, want, f"cs={cs} mf={mf} tmax={tmax}")


def test_golden_fixtures(golden):
    name, fx = golden
    dag = cbq.Dag(fx["nodes"], int(fx["root"]), cbq.LAYOUT_COMPACT)
    assert dag.layout == cbq.LAYOUT_COMPACT
    for query, (cs, mf) in {"surface": (True, -1.0), "nosurface": (False, -1.0), "lod": (True, 0.05)}.items():
        out = cbq.intersect_volume(dag, _dev(fx["origin_tmax"]), _dev(fx["direction"]), cs, mf)
        for k in ("hit", "distance", "material", "position", "normal", "voxel"):
            g = out[k].cpu().numpy()
            w = fx[f"{query}_{k}"]
            if k == "material":
                g, w = g.astype(np.uint32), w.astype(np.uint32)
            if k == "distance":
                w = w.astype(np.float32)
            assert oracle.same_bits_nan_equal(g, w), f"{name}/{query}: {k}"


def test_fewer_node_loads(terrain):
    nodes, root, ref, cmp, rays = terrain
    o, d = rays["bounce"]
    probes = cbq.count_fetches(ref, o, d).long()
    loads = cbq.count_fetches(cmp, o, d).long()
    assert (loads <= probes).all()
    assert loads.sum().item() < 0.9 * probes.sum().item()


def test_malformed_dag_iteration_cap(orc):
    nodes, root = W.SceneSpec(cbq.SCENE_SPHERES, 6, 11, 16).build()
    nodes = nodes.copy()
    empty_node = nodes.size // 8
    nodes = np.concatenate([nodes, np.zeros(8, np.uint32)])
    sd = cbq.find_subdags(nodes, root)[7]
    nodes[8 * sd.node_index: 8 * sd.node_index + 8] = empty_node
    o, d = W.CameraSpec((-40.0, -40.0, 90.0), (32.0, 32.0, 32.0), 4, 4).rays()
    want = orc.intersect(nodes, orc.find_subdags(nodes, root), o, d, True, 0.5)
    dag = cbq.Dag(nodes, root, cbq.LAYOUT_COMPACT)
    assert dag.layout == cbq.LAYOUT_COMPACT
    got = cbq.intersect_volume(dag, _dev(o), _dev(d), True, 0.5)
    assert (want["status"] == cbq.RAY_ITER_LIMIT).any()
    _same(got, want, "iteration cap")


def test_far_volume_falls_back_to_the_reference_layout():
    from conftest import relocate
    nodes, root = W.SceneSpec(cbq.SCENE_SPHERES, 6, 21, 10).build()
    n2, r2 = relocate(nodes, root, 6, (1 << 30, 0, 0))
    dag = cbq.Dag(n2, r2, cbq.LAYOUT_COMPACT)
    assert dag.layout == cbq.LAYOUT_REFERENCE
    with pytest.raises(cbq.CbqError):
        cbq.Dag(nodes, root, 7)


def test_mixed_layout_batch_and_server(terrain):
    nodes, root, ref, cmp, rays = terrain
    vols = W.batch_volumes(count=6, seed=91, edge_log2=(5, 8), rays=(500, 8000))
    dags, dev = [], []
    for i, v in enumerate(vols):
        n, r = v.scene.build()
        dags.append(cbq.Dag(n, r, cbq.LAYOUT_COMPACT if i % 2 else cbq.LAYOUT_REFERENCE))
        o, d = v.make_rays()
        dev.append((_dev(o), _dev(d)))
    assert {g.layout for g in dags} == {cbq.LAYOUT_REFERENCE, cbq.LAYOUT_COMPACT}
    single = [cbq.intersect_volume(g, o, d) for g, (o, d) in zip(dags, dev)]
    batch = cbq.Batch([(g, o, d) for g, (o, d) in zip(dags, dev)])
    batch.launch()
    torch.cuda.synchronize()
    for i, (out, want) in enumerate(zip(batch.outputs, single)):
        _same(out, want, f"batch job {i}")
    server = cbq.Server(device_memory_budget=64 << 20, max_inflight_launches=2)
    tickets = []
    for g, (o, d) in zip(dags, dev):
        tickets.append(server.submit(g, o.cpu().numpy(), d.cpu().numpy()))
    for (t, out), want in zip(tickets, single):
        assert server.wait(t) == 0
        _same(out, want, "server")
    server.close()


def test_pathtracer_on_the_compact_layout(orc):
    """Every wave of a frame on the compact layout equals the oracle (waves are
    compacted with atomics, so their ray order differs from run to run), and the
    frame equals the reference layout's to float-atomic rounding."""
    spec = W.SceneSpec(cbq.SCENE_CITY, 9, 31337)
    nodes, root = spec.build()
    eye, target = W.city_camera(9)
    rec = cbq.WaveRecorder()
    img_c, stats = cbq.pathtrace(cbq.Dag(nodes, root, cbq.LAYOUT_COMPACT), 48, 32, 2, 3, eye, target,
                                 W.city_materials(), seed=3, on_wave=rec)
    sd = orc.find_subdags(nodes, root)
    checked = 0
    for kind, depth, sample, o, d, hits, (cs, mf) in rec.waves:
        want = orc.intersect(nodes, sd, o, d, cs, mf)
        for k, v in hits.items():
            w = want[k]
            assert oracle.same_bits_nan_equal(v.astype(w.dtype) if k == "material" else v, w), k
        checked += o.shape[0]
    assert checked == stats["extension_rays"] + stats["shadow_rays"]
    img_r, _ = cbq.pathtrace(cbq.Dag(nodes, root), 48, 32, 2, 3, eye, target, W.city_materials(), seed=3)
    assert torch.allclose(img_c, img_r, rtol=1e-5, atol=1e-6)
