"""Host-side logic and the C ABI surface (no GPU calls)."""
import os
import re
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

import cubiquity_gb300 as cbq
from cubiquity_gb300 import workloads as W
from conftest import ROOT, subdags_of


def header_functions():
    text = (ROOT / "include" / "cubiquity_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(cbq_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_function():
    names = header_functions()
    assert len(names) >= 20
    lib = cbq.lib()
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", str(cbq.LIB_PATH)], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (cbq_\w+)", out))
    assert set(names) <= exported


def test_status_strings_and_version():
    assert cbq.lib().cbq_abi_version() == 1
    for s in range(12):
        assert cbq.lib().cbq_status_string(s).decode() == cbq._STATUS[s]


def test_import_fails_loudly_without_library(tmp_path):
    pkg = tmp_path / "cubiquity_gb300"
    pkg.mkdir()
    (pkg / "__init__.py").write_text((ROOT / "cubiquity_gb300" / "__init__.py").read_text())
    r = subprocess.run([sys.executable, "-c", "import cubiquity_gb300"], cwd=tmp_path, capture_output=True,
                       text=True)
    assert r.returncode != 0 and "no CPU fallback" in r.stderr


def _small_dag():
    return W.SceneSpec(cbq.SCENE_SPHERES, 5, 3, 6).build()


def test_validate_rejects_malformed():
    nodes, root = _small_dag()
    cbq.validate(nodes, root)
    bad = nodes.copy()
    bad[-1] = nodes.size // 8  # child index out of range
    with pytest.raises(cbq.CbqError) as e:
        cbq.validate(bad, root)
    assert e.value.status == 2
    bad = nodes.copy()
    bad[8 * 5 + 3] = 6  # material slot 5 no longer self-referencing
    with pytest.raises(cbq.CbqError):
        cbq.validate(bad, root)
    with pytest.raises(cbq.CbqError):
        cbq.validate(nodes, nodes.size // 8)
    with pytest.raises(cbq.CbqError):
        cbq.validate(nodes[: 8 * 100], 0)
    # A cycle (a node that is its own child) would let a traversal descend
    # below the leaves; it is rejected before any upload.
    sd = cbq.find_subdags(nodes, root)[7]
    bad = nodes.copy()
    bad[8 * sd.node_index + 3] = sd.node_index
    with pytest.raises(cbq.CbqError) as e:
        cbq.validate(bad, root)
    assert e.value.status == 2


def test_find_subdags_matches_golden(golden):
    name, fx = golden
    got = [s.as_tuple() for s in cbq.find_subdags(fx["nodes"], int(fx["root"]))]
    assert got == subdags_of(fx)


def test_builder_matches_reference_bake(golden):
    """The bulk builder gives the graph the reference's setVoxel + bake gave."""
    name, fx = golden
    kind, edge_log2, seed, param = (int(v) for v in fx["scene"])
    nodes, root = cbq.build_scene(kind, edge_log2, seed, param)
    assert cbq.canonical_hash(nodes, root) == cbq.canonical_hash(fx["nodes"], int(fx["root"]))


def test_builder_is_deterministic_across_thread_counts():
    for spec in (W.SceneSpec(cbq.SCENE_SPHERES, 7, 5, 20), W.terrain_scaled(8, 9),
                 W.SceneSpec(cbq.SCENE_CITY, 9, 4)):
        a, ra = spec.build(threads=1)
        b, rb = spec.build(threads=7)
        assert ra == rb and np.array_equal(a, b)


@pytest.mark.parametrize("spec", [W.SceneSpec(cbq.SCENE_SPHERES, 6, 21, 10), W.terrain_scaled(6, 31),
                                  W.SceneSpec(cbq.SCENE_CITY, 7, 41)])
def test_dag_voxels_equal_scene_voxels(spec):
    nodes, root = spec.build()
    e = 1 << spec.edge_log2
    vox = spec.voxels((0, 0, 0), (e, e, e))
    rng = np.random.default_rng(0)
    for x, y, z in rng.integers(0, e, (2000, 3)):
        assert cbq.dag_voxel(nodes, root, int(x), int(y), int(z)) == vox[z, y, x]
    assert cbq.dag_voxel(nodes, root, -1, 0, 0) == 0
    assert cbq.dag_voxel(nodes, root, e, e, e) == 0


def test_dag_file_roundtrip(tmp_path):
    nodes, root = _small_dag()
    p = tmp_path / "small.dag"
    cbq.save_dag(p, nodes, root)
    assert p.stat().st_size == 8 + (nodes.size // 8 - 256) * 32
    n2, r2 = cbq.load_dag(p)
    assert r2 == root and np.array_equal(n2, nodes)
    (tmp_path / "trunc.dag").write_bytes(p.read_bytes()[:40])
    with pytest.raises(cbq.CbqError):
        cbq.load_dag(tmp_path / "trunc.dag")
    with pytest.raises(cbq.CbqError):
        cbq.load_dag(tmp_path / "missing.dag")


def test_reorder_bfs_keeps_the_graph(orc):
    nodes, root = W.terrain_scaled(7, 3).build()
    n2, r2 = cbq.reorder_bfs(nodes, root)
    assert cbq.canonical_hash(n2, r2) == cbq.canonical_hash(nodes, root)
    o, d = W.camera_scaled(7, 64, 64).rays()
    a = orc.intersect(nodes, orc.find_subdags(nodes, root), o, d)
    b = orc.intersect(n2, orc.find_subdags(n2, r2), o, d)
    for k in ("hit", "distance", "material", "position", "normal", "voxel"):
        assert np.array_equal(a[k], b[k])


def test_relocated_scene_voxels_and_subdags():
    from conftest import relocate
    nodes, root = W.SceneSpec(cbq.SCENE_SPHERES, 6, 21, 10).build()
    origin = (1 << 30, -(1 << 26), 3 << 20)
    n2, r2 = relocate(nodes, root, 6, origin)
    cbq.validate(n2, r2)
    rng = np.random.default_rng(3)
    for x, y, z in rng.integers(0, 64, (300, 3)):
        a = cbq.dag_voxel(nodes, root, int(x), int(y), int(z))
        b = cbq.dag_voxel(n2, r2, int(x) + origin[0], int(y) + origin[1], int(z) + origin[2])
        assert a == b
    sd = [s for s in cbq.find_subdags(n2, r2) if s.node_index]
    assert len(sd) == 1 and tuple(sd[0].lower_bound) == origin


def test_log_handler_receives_library_messages():
    got = []
    cbq.set_log_handler(lambda level, msg: got.append((level, msg)))
    try:
        W.SceneSpec(cbq.SCENE_SPHERES, 5, 3, 6).build()
    finally:
        cbq.set_log_handler(None)
    assert any(level == cbq.LOG_INFO and "built scene" in msg for level, msg in got)
    n = len(got)
    W.SceneSpec(cbq.SCENE_SPHERES, 5, 3, 6).build()
    assert len(got) == n  # disabled


def test_bounce_rays_are_unit_and_in_hemisphere():
    pos = np.array([[1.0, 2.0, 3.0], [5.0, 5.0, 5.0]], np.float32)
    nrm = np.array([[0.0, 0.0, 1.0], [-1.0, 0.0, 0.0]], np.float32)
    o, d = cbq.bounce_rays(pos, nrm, 4000, 99)
    assert np.allclose(np.linalg.norm(d[:, :3], axis=1), 1.0, atol=1e-5)
    cos = np.einsum("ij,ij->i", d[:, :3], nrm[np.arange(4000) % 2])
    assert (cos >= -1e-6).all() and abs(cos.mean() - 2 / 3) < 0.03  # cosine-weighted: E[cos] = 2/3
    assert np.allclose(o[0, :3], pos[0] + nrm[0] * np.float32(0.01))
    o2, d2 = cbq.bounce_rays(pos, nrm, 4000, 99)
    assert np.array_equal(d, d2)
