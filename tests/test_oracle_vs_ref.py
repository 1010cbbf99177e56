"""The oracle restatement and the bulk builder against the reference itself,
run side by side (CPU).  Skipped where the reference checkout is absent."""
import numpy as np
import pytest

import cubiquity_gb300 as cbq
import oracle
from cubiquity_gb300 import workloads as W

FIELDS = ("hit", "material", "position", "normal", "voxel")

SCENES = [
    W.SceneSpec(cbq.SCENE_SPHERES, 6, 1001, 24),
    W.SceneSpec(cbq.SCENE_SPHERES, 7, 1002, 40),
    W.terrain_scaled(6, 1003),
    W.terrain_scaled(7, 1004),
    W.SceneSpec(cbq.SCENE_CITY, 7, 1005),
]


def ref_volume(ref, spec):
    e = 1 << spec.edge_log2
    vox = spec.voxels((0, 0, 0), (e, e, e))
    zz, yy, xx = np.nonzero(vox)
    vol = ref.new_volume()
    vol.set_voxels(np.stack([xx, yy, zz], 1), vox[zz, yy, xx])
    vol.bake()
    return vol


def random_rays(edge, n, seed):
    rng = np.random.default_rng(seed)
    o = np.zeros((n, 4), np.float32)
    d = np.zeros((n, 4), np.float32)
    o[:, :3] = rng.uniform(-edge * 0.5, edge * 1.5, (n, 3))
    o[:, 3] = np.inf
    inside = rng.random(n) < 0.5
    o[inside, :3] = rng.uniform(0, edge, (inside.sum(), 3))
    tgt = rng.uniform(0, edge, (n, 3))
    v = tgt - o[:, :3]
    d[:, :3] = v / np.linalg.norm(v, axis=1, keepdims=True)
    return o, d


def _eq(a, b, k):
    if k == "distance":
        a = a.astype(np.float32)
        b = b.astype(np.float32)
    return np.array_equal(np.ascontiguousarray(a).view(np.uint8), np.ascontiguousarray(b).view(np.uint8))


@pytest.mark.reference
@pytest.mark.parametrize("spec", SCENES, ids=lambda s: f"k{s.kind}e{s.edge_log2}s{s.seed}")
def test_builder_equals_setvoxel_bake(ref, spec):
    vol = ref_volume(ref, spec)
    nodes, root = spec.build()
    assert cbq.canonical_hash(nodes, root) == cbq.canonical_hash(vol.nodes(), vol.root)


@pytest.mark.reference
@pytest.mark.parametrize("spec", SCENES, ids=lambda s: f"k{s.kind}e{s.edge_log2}s{s.seed}")
@pytest.mark.parametrize("query", [(True, -1.0), (False, -1.0), (True, 0.03)])
def test_oracle_equals_reference_random_rays(ref, orc, spec, query):
    vol = ref_volume(ref, spec)
    nodes = vol.nodes()
    sd = vol.find_subdags()
    o, d = random_rays(1 << spec.edge_log2, 20000, spec.seed)
    a = vol.intersect(sd, o, d, *query)
    b = orc.intersect(nodes, sd, o, d, *query)
    assert not b["status"].any()
    for k in FIELDS + ("distance",):
        assert _eq(a[k], b[k], k), k


@pytest.mark.reference
def test_oracle_equals_reference_on_degenerate_rays_that_terminate(ref, orc):
    """Zero direction components and on-face origins.  The reference is only
    run on rays the oracle finished with status OK: the oracle follows the
    reference's steps exactly up to the point where it stops a ray the
    reference would loop on, so OK rays are rays the reference finishes."""
    spec = W.SceneSpec(cbq.SCENE_SPHERES, 6, 11, 16)
    vol = ref_volume(ref, spec)
    nodes = vol.nodes()
    sd = vol.find_subdags()
    rng = np.random.default_rng(9)
    n = 4000
    o = np.zeros((n, 4), np.float32)
    d = np.zeros((n, 4), np.float32)
    o[:, :3] = np.floor(rng.uniform(-8, 72, (n, 3))) + rng.choice([0.5, 0.25, 0.0, -0.5], (n, 3))
    o[:, 3] = np.inf
    v = rng.normal(size=(n, 3))
    v[rng.random((n, 3)) < 0.4] = 0
    v[(v == 0).all(1), 0] = 1
    d[:, :3] = v / np.linalg.norm(v, axis=1, keepdims=True)
    b = orc.intersect(nodes, sd, o, d)
    ok = b["status"] == 0
    assert (~ok).sum() > 0 and ok.sum() > 0.9 * n
    # Rays that read never-written stack slots have no defined reference result.
    undefined = oracle.undefined_stack_rays(orc, nodes, sd, o, d)
    print(f"{undefined.size} rays read uninitialised stack slots: {undefined.tolist()}")
    assert undefined.size <= 0.002 * n
    ok[undefined] = False
    a = vol.intersect(sd, o[ok], d[ok])
    for k in FIELDS + ("distance",):
        want = a[k].astype(np.float32) if k == "distance" else a[k]
        assert oracle.same_bits_nan_equal(want, b[k][ok]), k


@pytest.mark.reference
def test_reference_reads_dag_files_we_write(ref, tmp_path):
    nodes, root = W.terrain_scaled(7, 5).build()
    p = tmp_path / "t.dag"
    cbq.save_dag(p, nodes, root)
    vol = ref.load(p)
    assert vol.root == root and np.array_equal(vol.nodes(), nodes)
    rng = np.random.default_rng(2)
    for x, y, z in rng.integers(0, 128, (500, 3)):
        assert vol.voxel(int(x), int(y), int(z)) == cbq.dag_voxel(nodes, root, int(x), int(y), int(z))


@pytest.mark.reference
def test_we_read_dag_files_the_reference_writes(ref, tmp_path):
    spec = W.SceneSpec(cbq.SCENE_SPHERES, 6, 77, 9)
    vol = ref_volume(ref, spec)
    p = tmp_path / "r.dag"
    vol.save(p)
    nodes, root = cbq.load_dag(p)
    assert root == vol.root and np.array_equal(nodes, vol.nodes())


@pytest.mark.reference
@pytest.mark.parametrize("seed", range(8))
def test_random_dags_oracle_equals_reference(ref, orc, seed):
    """Random voxel sets at random places (tests/dagbuild.py): the reference's
    setVoxel + bake gives the graph the test builder gives, and the oracle
    gives the reference's results on random rays (those the oracle finishes
    with status OK and that read no never-written stack slot)."""
    from dagbuild import build_dag, random_voxels, random_rays as rays_for
    rng = np.random.default_rng(5000 + seed)
    edge = 1 << int(rng.integers(2, 6))
    vox = random_voxels(rng, edge)
    origin = tuple(int(x) * edge for x in rng.integers(-(1 << 12) // edge, (1 << 12) // edge, 3))
    nodes, root = build_dag(vox, origin)
    vol = ref.new_volume()
    zz, yy, xx = np.nonzero(vox)
    if zz.size:
        vol.set_voxels(np.stack([xx + origin[0], yy + origin[1], zz + origin[2]], 1), vox[zz, yy, xx])
    vol.bake()
    assert cbq.canonical_hash(nodes, root) == cbq.canonical_hash(vol.nodes(), vol.root)
    sd = vol.find_subdags()
    assert sd == orc.find_subdags(vol.nodes(), vol.root)
    assert [s[:2] for s in sd] == [s[:2] for s in orc.find_subdags(nodes, root)]  # node numbering differs
    o, d = rays_for(rng, origin, edge, 3000)
    o[:, 3] = np.inf
    for query in [(True, -1.0), (False, -1.0), (True, 0.05)]:
        b = orc.intersect(vol.nodes(), sd, o, d, *query)
        ok = b["status"] == 0
        undefined = oracle.undefined_stack_rays(orc, vol.nodes(), sd, o, d, compute_surface=query[0],
                                                max_footprint=query[1])
        ok[undefined] = False
        assert ok.sum() > 0.9 * o.shape[0]
        a = vol.intersect(sd, o[ok], d[ok], *query)
        for k in FIELDS + ("distance",):
            want = a[k].astype(np.float32) if k == "distance" else a[k]
            assert oracle.same_bits_nan_equal(want, b[k][ok]), (query, k)
