"""Parity of the CUDA path (through the C ABI) with the reference and the oracle.

Bar: hit, material, voxel and status bit-exact; distance, position and normal
are also required bit-exact here (the kernel performs the reference's FP32
operations in the reference's order), which is stricter than the 1e-5
relative tolerance the path is specified with.
"""
import hashlib

import numpy as np
import pytest

import cubiquity_gb300 as cbq
import oracle
from cubiquity_gb300 import workloads as W
from conftest import subdags_of

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

FIELDS = ("hit", "distance", "material", "position", "normal", "voxel")
QUERIES = {"surface": (True, -1.0), "nosurface": (False, -1.0), "lod": (True, 0.05)}


@pytest.fixture(scope="module", autouse=True)
def _device():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    torch.cuda.set_device(0)


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _host(out):
    return {k: v.cpu().numpy() for k, v in out.items()}


def _bits_equal(a, b):
    # Bit-exact, with every NaN equal to every NaN (payloads are platform-specific).
    return oracle.same_bits_nan_equal(a, b)


def _assert_same(got, want, fields=FIELDS, what=""):
    for k in fields:
        g = got[k]
        w = want[k]
        if k == "material":
            g, w = g.astype(np.uint32), w.astype(np.uint32)
        if k == "distance":
            w = w.astype(np.float32)
        if not _bits_equal(g, w):
            bad = np.nonzero((g != w).reshape(g.shape[0], -1).any(axis=1))[0]
            raise AssertionError(f"{what} {k}: {bad.size} rays differ, first {bad[:10].tolist()}")


def _spread(a, n):
    """n rays spread over the whole image (the top rows of the camera are sky)."""
    return np.ascontiguousarray(a[:: max(1, a.shape[0] // n)][:n])


def _digest(out):
    res = {}
    for k in FIELDS:
        a = out[k]
        if k == "material":
            a = a.astype(np.uint32)
        res[k] = hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()
    res["hits"] = int(out["hit"].sum())
    return res


KERNELS = {"flat": cbq.KERNEL_FLAT, "nested": cbq.KERNEL_NESTED}


@pytest.mark.parametrize("kernel", list(KERNELS))
@pytest.mark.parametrize("query", list(QUERIES))
def test_gpu_matches_reference_golden(golden, query, kernel):
    name, fx = golden
    cs, mf = QUERIES[query]
    dag = cbq.Dag(fx["nodes"], int(fx["root"]))
    dag.set_launch_config(KERNELS[kernel])
    assert dag.launch_config()["kernel"] == KERNELS[kernel]
    assert [s.as_tuple() for s in dag.subdags] == subdags_of(fx)
    out = _host(cbq.intersect_volume(dag, _dev(fx["origin_tmax"]), _dev(fx["direction"]), cs, mf))
    assert not out["status"].any()
    _assert_same(out, {k: fx[f"{query}_{k}"] for k in FIELDS}, what=f"{name}/{query}")


def test_gpu_full_spheres256_matches_reference_digest(digests, orc):
    dg = digests["spheres256"]
    nodes, root = W.SPHERES_256.build()
    assert cbq.canonical_hash(nodes, root) == dg["canonical_dag_sha256"]
    o, d = W.SPHERES_256_CAMERA.rays()
    dag = cbq.Dag(nodes, root)
    out = _host(cbq.intersect_volume(dag, _dev(o), _dev(d), True, -1.0))
    assert _digest(out) == dg["surface"]
    lod = _host(cbq.intersect_volume(dag, _dev(o), _dev(d), True, dg["lod_max_footprint"]))
    assert _digest(lod) == dg["lod"]
    # and ray by ray against the oracle
    _assert_same(out, orc.intersect(nodes, orc.find_subdags(nodes, root), o, d), what="spheres256")


@pytest.fixture(scope="module")
def terrain():
    nodes, root = W.TERRAIN_4096.build()
    dag = cbq.Dag(nodes, root)
    o, d = W.TERRAIN_4096_CAMERA.rays()
    yield nodes, root, dag, o, d
    dag.destroy()


def test_gpu_full_terrain4096_matches_reference_digest(terrain, digests, orc):
    nodes, root, dag, o, d = terrain
    dg = digests["terrain4096"]
    assert cbq.canonical_hash(nodes, root) == dg["canonical_dag_sha256"]
    prim = _host(cbq.intersect_volume(dag, _dev(o), _dev(d)))
    assert _digest(prim) == dg["primary"]
    bo, bd = W.bounce_from_hits(prim, o.shape[0])
    assert hashlib.sha256(bo.tobytes() + bd.tobytes()).hexdigest() == dg["bounce_rays_sha256"]
    boun = _host(cbq.intersect_volume(dag, _dev(bo), _dev(bd)))
    assert _digest(boun) == dg["bounce"]
    sd = orc.find_subdags(nodes, root)
    _assert_same(prim, orc.intersect(nodes, sd, o, d), what="terrain primary")
    _assert_same(boun, orc.intersect(nodes, sd, bo, bd), what="terrain bounce")


@pytest.mark.parametrize("kernel,chunk", [("flat", 0), ("flat", 1), ("flat", 32), ("nested", 0),
                                          ("nested", 96)])
def test_persistent_equals_plain(terrain, kernel, chunk):
    nodes, root, dag, o, d = terrain
    to, td = _dev(o), _dev(d)
    a = _host(cbq.intersect_volume(dag, to, td))
    dag.set_launch_config(KERNELS[kernel])
    try:
        ctr = torch.zeros(1, dtype=torch.int64, device="cuda")
        b = _host(cbq.intersect_volume_persistent(dag, to, td, ctr, chunk=chunk))
        c = _host(cbq.intersect_volume(dag, to, td))
    finally:
        dag.set_launch_config()
    _assert_same(b, a, FIELDS + ("status",), what=f"persistent {kernel} chunk={chunk}")
    _assert_same(c, a, FIELDS + ("status",), what=f"plain {kernel}")


@pytest.mark.parametrize("origin,flat", [((1 << 30, -(1 << 26), 3 << 20), False),
                                         ((3 << 20, 1 << 23, -(1 << 22)), False),
                                         (((1 << 21) - 64, -(1 << 21), 5 << 18), True),
                                         ((1 << 21, 0, 0), False)])
def test_relocated_volume(orc, origin, flat):
    """A volume away from the origin: the float-position kernel applies while
    every SubDAG lies within +-2^21 (flat=True: its box touches 2^21 and -2^21);
    beyond, the flat kernel keeps integer positions instead.  The nested
    kernel, asked for, also agrees with the oracle."""
    from conftest import relocate
    nodes, root = W.SceneSpec(cbq.SCENE_SPHERES, 6, 11, 16).build()
    n2, r2 = relocate(nodes, root, 6, origin)
    cam = W.CameraSpec(tuple(np.add((-40.0, -40.0, 90.0), origin)), tuple(np.add((32.0, 32.0, 32.0), origin)), 48, 48)
    o, d = cam.rays()
    # The compact layout needs the float-position form: which layout the DAG
    # gets shows which form applies.
    probe = cbq.Dag(n2, r2, cbq.LAYOUT_COMPACT)
    assert probe.layout == (cbq.LAYOUT_COMPACT if flat else cbq.LAYOUT_REFERENCE)
    probe.destroy()
    dag = cbq.Dag(n2, r2)
    assert dag.launch_config()["kernel"] == cbq.KERNEL_FLAT
    want = orc.intersect(n2, orc.find_subdags(n2, r2), o, d)
    for form in (cbq.FORM_PERSISTENT, cbq.FORM_PLAIN):
        for stack in (cbq.STACK_LOCAL, cbq.STACK_SHARED):
            dag.set_launch_config(cbq.KERNEL_FLAT, 64, 0, 8, stack, form, 8, 56)
            got = _host(cbq.intersect_volume(dag, _dev(o), _dev(d)))
            _assert_same(got, want, FIELDS + ("status",), what=f"relocated {origin} form {form} stack {stack}")
    dag.set_launch_config(cbq.KERNEL_NESTED)
    got2 = _host(cbq.intersect_volume(dag, _dev(o), _dev(d)))
    _assert_same(got2, want, FIELDS + ("status",), what=f"relocated {origin} nested")
    lod = orc.intersect(n2, orc.find_subdags(n2, r2), o, d, True, 0.05)
    dag.set_launch_config()
    got3 = _host(cbq.intersect_volume(dag, _dev(o), _dev(d), True, 0.05))
    _assert_same(got3, lod, FIELDS + ("status",), what=f"relocated {origin} LOD")


def test_host_api_equals_device_api(terrain):
    nodes, root, dag, o, d = terrain
    n = 300_001  # not a multiple of any block size
    a = _host(cbq.intersect_volume(dag, _dev(_spread(o, n)), _dev(_spread(d, n))))
    b = cbq.intersect_volume_host(dag, _spread(o, n), _spread(d, n))
    _assert_same(b, a, FIELDS + ("status",), what="host api")
    c = cbq.intersect_volume_host(dag, _spread(o, n)[:1000], _spread(d, n)[:1000])  # reuses staging buffers
    _assert_same(c, {k: v[:1000] for k, v in a.items()}, FIELDS, what="host api reuse")


@pytest.mark.parametrize("n", [4095, (1 << 18) - 1, 3 * (1 << 18) + 17, 8 << 18, (8 << 18) + 4095, 2_500_003])
def test_host_api_chunks(terrain, n):
    """Large host calls are split into chunks whose copies overlap the traversal
    (one chunk per 2^18 rays, at most 8), each chunk taking every k-th block of
    4096 rays: every chunk count, block boundary and partial last block gives
    the device path's bits, with all or some hit fields requested, from
    pageable or page-locked buffers."""
    nodes, root, dag, o, d = terrain
    so, sd = _spread(o, n), _spread(d, n)
    want = _host(cbq.intersect_volume(dag, _dev(so), _dev(sd), True, -1.0, use_tmax=True))
    got = cbq.intersect_volume_host(dag, so, sd, use_tmax=True)
    _assert_same(got, want, FIELDS + ("status",), what=f"host chunks {n}")
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()  # noqa: E731
    part = {k: pin(v) for k, v in cbq.alloc_host_hits(n).items() if k in ("hit", "voxel", "status")}
    got = cbq.intersect_volume_host(dag, pin(so), pin(sd), use_tmax=True, out=part)
    _assert_same(got, want, ("hit", "voxel", "status"), what=f"host chunks {n}, pinned, some fields")


def test_host_api_from_several_threads(terrain):
    """Host calls from four threads on one DAG handle (serialised by its staging
    lock, each on the handle's own streams) give every thread its own bits."""
    import threading
    nodes, root, dag, o, d = terrain
    n = 600_000
    parts = [(_spread(o, 4 * n)[k::4], _spread(d, 4 * n)[k::4]) for k in range(4)]
    want = [_host(cbq.intersect_volume(dag, _dev(po), _dev(pd))) for po, pd in parts]
    got = [None] * 4
    errors = []

    def worker(k):
        try:
            for _ in range(3):
                got[k] = cbq.intersect_volume_host(dag, *parts[k])
        except Exception as e:  # noqa: BLE001  (reported below)
            errors.append(e)

    th = [threading.Thread(target=worker, args=(k,)) for k in range(4)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert not errors, errors
    for k in range(4):
        _assert_same(got[k], want[k], FIELDS + ("status",), what=f"thread {k}")


def test_fetch_counts_match_oracle(terrain, orc):
    nodes, root, dag, o, d = terrain
    n = 200_000
    f = cbq.count_fetches(dag, _dev(_spread(o, n)), _dev(_spread(d, n))).cpu().numpy().astype(np.uint32)
    want = orc.count_fetches(nodes, orc.find_subdags(nodes, root), _spread(o, n), _spread(d, n))
    assert np.array_equal(f, want)


def test_tmax_post_filter(terrain, orc):
    nodes, root, dag, o, d = terrain
    n = 100_000
    sl = slice(o.shape[0] // 2, o.shape[0] // 2 + n)  # mid-image rows: mostly terrain
    o2 = o[sl].copy()
    o2[:, 3] = np.random.default_rng(1).uniform(0, 6000, n).astype(np.float32)
    out = _host(cbq.intersect_volume(dag, _dev(o2), _dev(d[sl]), use_tmax=True))
    want = orc.intersect(nodes, orc.find_subdags(nodes, root), o2, d[sl], use_tmax=True)
    _assert_same(out, want, what="tmax")
    full = _host(cbq.intersect_volume(dag, _dev(o2), _dev(d[sl])))
    assert 0 < out["hit"].sum() < full["hit"].sum()


def test_null_fields_and_empty_batch(terrain):
    nodes, root, dag, o, d = terrain
    n = 5000
    full = _host(cbq.intersect_volume(dag, _dev(_spread(o, n)), _dev(_spread(d, n))))
    part = cbq.alloc_hits(n, fields=("voxel", "material"))
    cbq.intersect_volume(dag, _dev(_spread(o, n)), _dev(_spread(d, n)), out=part)
    assert np.array_equal(part["voxel"].cpu().numpy(), full["voxel"])
    assert np.array_equal(part["material"].cpu().numpy(), full["material"])
    empty = torch.empty((0, 4), dtype=torch.float32, device="cuda")
    cbq.intersect_volume(dag, empty, empty)
    torch.cuda.synchronize()


def test_misaligned_rays_rejected(terrain):
    nodes, root, dag, o, d = terrain
    buf = _dev(np.zeros(4 * 65, np.float32))
    rays = cbq._Rays(buf.data_ptr() + 4, buf.data_ptr())
    q = cbq.Query().c()
    hits = cbq._Hits()
    st = cbq.lib().cbq_intersect(dag.handle, rays, 64, q, hits, None)
    assert st == 1


def degenerate_rays(n=2000, seed=5):
    """Zero direction components with origins on, beside and between voxel
    faces.  Where an origin lies exactly on an axis plane with a zero direction
    component, 0/0 makes the octant distances NaN and the reference's octant
    loop (raytracing.cpp:441-475) never advances: those rays end with
    CBQ_RAY_STUCK on both sides here."""
    rng = np.random.default_rng(seed)
    o = np.zeros((n, 4), np.float32)
    d = np.zeros((n, 4), np.float32)
    o[:, :3] = np.floor(rng.uniform(0, 64, (n, 3))) + rng.choice([0.5, 0.25, 0.0, -0.5], (n, 3))
    o[:, 3] = np.inf
    v = rng.normal(size=(n, 3))
    v[rng.random((n, 3)) < 0.4] = 0
    v[(v == 0).all(1), 0] = 1
    d[:, :3] = v / np.linalg.norm(v, axis=1, keepdims=True)
    return o, d


def test_degenerate_rays_and_stuck_status(orc):
    nodes, root = W.SceneSpec(cbq.SCENE_SPHERES, 6, 11, 16).build()
    o, d = degenerate_rays()
    want = orc.intersect(nodes, orc.find_subdags(nodes, root), o, d)
    assert (want["status"] == cbq.RAY_STUCK).sum() > 0
    dag = cbq.Dag(nodes, root)
    got = _host(cbq.intersect_volume(dag, _dev(o), _dev(d)))
    _assert_same(got, want, FIELDS + ("status",), what="degenerate")


def test_iteration_cap_on_malformed_dag(orc):
    """An internal node whose children are all empty never occurs in a baked
    DAG; findNearestMaterial would spin on it.  The fetch cap ends the ray with
    CBQ_RAY_ITER_LIMIT (bounded: at most 2^17 fetches)."""
    nodes, root = W.SceneSpec(cbq.SCENE_SPHERES, 6, 11, 16).build()
    nodes = nodes.copy()
    empty_node = nodes.size // 8
    nodes = np.concatenate([nodes, np.zeros(8, np.uint32)])
    # Route every child of the sub-DAG root to the all-empty node.
    sd = cbq.find_subdags(nodes, root)[7]
    nodes[8 * sd.node_index: 8 * sd.node_index + 8] = empty_node
    o, d = W.CameraSpec((-40.0, -40.0, 90.0), (32.0, 32.0, 32.0), 4, 4).rays()
    want = orc.intersect(nodes, orc.find_subdags(nodes, root), o, d, True, 0.5)
    dag = cbq.Dag(nodes, root)
    got = _host(cbq.intersect_volume(dag, _dev(o), _dev(d), True, 0.5))
    assert (want["status"] == cbq.RAY_ITER_LIMIT).any()
    _assert_same(got, want, FIELDS + ("status",), what="iteration cap")


def dotted_line_dag(height=20):
    """Voxels at odd x on the line y = z = 0 of a 2^height volume at the
    origin: one leaf node, then one node per level with two children."""
    nodes = [np.repeat(np.arange(256, dtype=np.uint32), 8).reshape(256, 8)]
    leaf = np.zeros(8, np.uint32)
    leaf[1] = 1  # child (x=1, y=0, z=0): material 1
    rows = [leaf]
    for _ in range(height - 1):
        r = np.zeros(8, np.uint32)
        r[0] = r[1] = 256 + len(rows) - 1
        rows.append(r)
    for _ in range(31 - height):  # single-child chain up to height 31
        r = np.zeros(8, np.uint32)
        r[0] = 256 + len(rows) - 1
        rows.append(r)
    root = np.zeros(8, np.uint32)
    root[7] = 256 + len(rows) - 1  # the octant x, y, z >= 0
    rows.append(root)
    nodes.append(np.stack(rows))
    return np.concatenate(nodes).reshape(-1), 256 + len(rows) - 1


def test_iteration_cap_inside_the_walk(orc):
    """A ray grazing the line (in the voxel row y = 1) visits every leaf node along it
    without a hit: more than 2^17 steps, so the walk itself reaches the fetch
    cap and the ray ends with CBQ_RAY_ITER_LIMIT, in every kernel and layout."""
    nodes, root = dotted_line_dag()
    # Voxel v spans [v - 0.5, v + 0.5): rows y = 1 graze, y = 0 hits x = 1.
    o = np.array([[-1.0, 1.0, 0.0, 0.0], [-1.0, 0.0, 0.0, 0.0], [-3.0, 1.25, -0.25, 0.0],
                  [1000.0, 1.0, 0.0, 0.0]], np.float32)
    d = np.array([[1.0, 1e-7, 1e-7, 0.0], [1.0, 1e-7, 1e-7, 0.0], [1.0, 2e-7, -1e-7, 0.0],
                  [1.0, 1e-7, 1e-7, 0.0]], np.float32)
    want = orc.intersect(nodes, orc.find_subdags(nodes, root), o, d)
    assert want["status"].tolist() == [cbq.RAY_ITER_LIMIT, cbq.RAY_OK, cbq.RAY_ITER_LIMIT, cbq.RAY_ITER_LIMIT]
    assert want["hit"].tolist() == [0, 1, 0, 0]
    for layout in (cbq.LAYOUT_REFERENCE, cbq.LAYOUT_COMPACT):
        dag = cbq.Dag(nodes, root, layout)
        assert dag.layout == layout
        for kernel in (cbq.KERNEL_FLAT, cbq.KERNEL_NESTED) if layout == cbq.LAYOUT_REFERENCE else (cbq.KERNEL_FLAT,):
            for steps in (1, 3, 16):
                dag.set_launch_config(kernel, 64, 0, 0, cbq.STACK_LOCAL, cbq.FORM_PERSISTENT, steps)
                scratch = cbq.scratch_for(o.shape[0])
                got = _host(cbq.intersect_auto(dag, _dev(o), _dev(d), scratch))
                _assert_same(got, want, FIELDS + ("status",), what=f"layout {layout} kernel {kernel} steps {steps}")


def slab_boundary_rays(n=8192, seed=9):
    """Rays on both sides of the condition under which the step takes min/max
    with fminf/fmaxf (every |dir| component at least FLT_MIN, the reflected
    origin finite): normal rays, components exactly FLT_MIN, subnormal and zero
    components, huge, infinite and NaN origins, NaN directions.  Runs of 32
    rays share a kind (so whole warps take either form) and single odd rays
    sit among normal ones (so warps switch to the reference's form)."""
    rng = np.random.default_rng(seed)
    tiny = np.float32(np.finfo(np.float32).tiny)
    o = np.zeros((n, 4), np.float32)
    d = np.zeros((n, 4), np.float32)
    o[:, :3] = rng.uniform(-20, 84, (n, 3))
    o[:, 3] = np.inf
    v = rng.normal(size=(n, 3))
    d[:, :3] = v / np.linalg.norm(v, axis=1, keepdims=True)
    kinds = rng.integers(0, 8, n // 32)
    for r, k in enumerate(kinds):
        sl = slice(32 * r, 32 * r + 32)
        ax = rng.integers(0, 3)
        if k == 1:
            d[sl, ax] = np.copysign(tiny, d[sl, ax])               # exactly FLT_MIN: still the fast form
        elif k == 2:
            d[sl, ax] = np.copysign(tiny / 4, d[sl, ax])           # subnormal: 1/|d| overflows
        elif k == 3:
            d[sl, ax] = 0.0
        elif k == 4:
            o[sl, ax] = np.float32(3e38) * rng.choice([-1, 1])
        elif k == 5:
            o[sl, ax] = np.inf * rng.choice([-1, 1])
        elif k == 6:
            o[sl, ax] = np.nan
    odd = rng.choice(n, n // 64, replace=False)                    # single odd lanes in normal warps
    d[odd, 0] = rng.choice(np.array([0.0, tiny / 2, np.nan], np.float32), odd.size)
    return o, d


@pytest.mark.parametrize("form", [cbq.FORM_PLAIN, cbq.FORM_PERSISTENT])
def test_slab_min_max_forms_at_their_boundary(orc, form):
    nodes, root = W.SceneSpec(cbq.SCENE_SPHERES, 6, 11, 16).build()
    o, d = slab_boundary_rays()
    want = orc.intersect(nodes, orc.find_subdags(nodes, root), o, d)
    assert want["hit"].sum() > 0
    dag = cbq.Dag(nodes, root)
    dag.set_launch_config(cbq.KERNEL_FLAT, 64, 0, 8, cbq.STACK_LOCAL, form, 8, 0)
    scratch = cbq.scratch_for(o.shape[0])
    got = _host(cbq.intersect_auto(dag, _dev(o), _dev(d), scratch))
    _assert_same(got, want, FIELDS + ("status",), what="slab boundary")
    dag.destroy()
