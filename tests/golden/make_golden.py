"""Generates the golden fixtures in this directory from the REFERENCE itself.

Run where the reference checkout is available (oracle/Makefile compiles its
src/library sources into oracle/_ref/libcbq_ref.so):

    python tests/golden/make_golden.py

Fixtures
  spheres64.npz, terrain64.npz
      Small seeded scenes built through the reference's Volume::setVoxel + bake
      (storage.cpp:396-437, 387), its node array and SubDAGs (findSubDAGs,
      raytracing.cpp:89), a few thousand rays (camera, random segments inside
      the bounds as in test_rendering.cpp:23-82, and edge cases), and the
      reference's intersectVolume outputs for three query settings plus
      traceRayRef's.
  digests.json
      Full-size pins: the canonical hash of the spheres-256 DAG the reference
      builds, and SHA-256 digests of the reference's intersectVolume outputs on
      the full spheres-256 camera (1,048,576 rays) and on the terrain-4096
      primary (4,194,304) and bounce (4,194,304) rays, traced by the reference
      on the byte-identical node array produced by libcbq's builder.
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

import cubiquity_gb300 as cbq  # noqa: E402
import oracle  # noqa: E402
from cubiquity_gb300 import workloads as W  # noqa: E402

QUERIES = {
    "surface": dict(compute_surface=True, max_footprint=-1.0),
    "nosurface": dict(compute_surface=False, max_footprint=-1.0),
    # Large enough that the small scenes' camera distances stop above the leaves
    # and exercise findNearestMaterial (raytracing.cpp:134-162).
    "lod": dict(compute_surface=True, max_footprint=0.05),
}
LOD_256 = 0.02
FIELDS = ("hit", "distance", "material", "position", "normal", "voxel")


canonical_hash = cbq.canonical_hash


def output_digest(out: dict) -> dict:
    """Per-field SHA-256 of the raw output bytes (distance as float32)."""
    res = {}
    for k in FIELDS:
        a = out[k]
        if k == "distance":
            a = np.asarray(a)
            if a.dtype == np.float64:
                f = a.astype(np.float32)
                assert np.array_equal(f.astype(np.float64), a), "reference distance is not a widened float"
                a = f
        res[k] = hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()
    res["hits"] = int(np.asarray(out["hit"]).sum())
    return res


def reference_volume(ref, spec: W.SceneSpec):
    e = 1 << spec.edge_log2
    vox = spec.voxels((0, 0, 0), (e, e, e))
    zz, yy, xx = np.nonzero(vox)
    vol = ref.new_volume()
    vol.set_voxels(np.stack([xx, yy, zz], 1), vox[zz, yy, xx])
    vol.bake()
    return vol


def edge_case_rays(edge: int, rng: np.random.Generator):
    """Axis-aligned, diagonal, inside-solid, signed-zero and outward rays.

    Zero direction components only ever come with origins whose coordinate on
    that axis is not a voxel face (x + 0.5 not an integer): a zero component
    with the origin on a face gives 0 * inf = NaN slabs, on which the
    reference's loop does not terminate."""
    o, d = [], []
    mid = edge / 2
    for axis in range(3):
        for sgn in (1.0, -1.0):
            for k in range(24):
                p = rng.uniform(0, edge, 3)
                p = np.floor(p) + 0.25
                p[axis] = -3.75 if sgn > 0 else edge + 3.75
                dd = np.zeros(3)
                dd[axis] = sgn
                if k % 3 == 1:
                    dd = np.where(dd == 0, -0.0, dd)
                o.append(p)
                d.append(dd)
    for k in range(64):
        p = rng.uniform(-edge * 0.5, edge * 1.5, 3)
        dd = np.array([1.0, 1.0, 1.0]) * np.sign(mid - p)
        dd = dd / np.linalg.norm(dd)
        o.append(p)
        d.append(dd)
    for k in range(64):  # rays starting inside the volume, some inside solids
        p = rng.uniform(0, edge, 3)
        v = rng.normal(size=3)
        o.append(p)
        d.append(v / np.linalg.norm(v))
    for k in range(32):  # pointing away from the volume
        p = np.array([edge * 2.0, edge * 2.0, edge * 2.0]) + rng.uniform(0, 10, 3)
        v = np.abs(rng.normal(size=3)) + 0.1
        o.append(p)
        d.append(v / np.linalg.norm(v))
    o = np.array(o, dtype=np.float32)
    d = np.array(d, dtype=np.float32)
    return _pack(o, d)


def _pack(o3, d3):
    n = o3.shape[0]
    o = np.zeros((n, 4), np.float32)
    d = np.zeros((n, 4), np.float32)
    o[:, :3] = o3
    o[:, 3] = np.inf
    d[:, :3] = d3
    return o, d


def segment_rays(edge: int, n: int, rng: np.random.Generator):
    """Random segments inside the bounds (test_rendering.cpp:29-49)."""
    a = rng.uniform(0, edge, (n, 3)).astype(np.float32)
    b = rng.uniform(0, edge, (n, 3)).astype(np.float32)
    d = (b - a).astype(np.float64)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return _pack(a, d.astype(np.float32))


def small_fixture(ref, name: str, spec: W.SceneSpec, cam: W.CameraSpec, seed: int):
    vol = reference_volume(ref, spec)
    nodes, root = vol.nodes(), vol.root
    sd = vol.find_subdags()
    rng = np.random.default_rng(seed)
    edge = 1 << spec.edge_log2
    parts = [cam.rays(), segment_rays(edge, 1024, rng), edge_case_rays(edge, rng)]
    o = np.concatenate([p[0] for p in parts])
    d = np.concatenate([p[1] for p in parts])
    data = {"nodes": nodes, "root": np.uint32(root),
            "subdags": np.array([[*lb, h, node] for (lb, h, node) in sd], dtype=np.int64),
            "origin_tmax": o, "direction": d,
            "scene": np.array([spec.kind, spec.edge_log2, spec.seed, spec.param], dtype=np.int64)}
    for q, kw in QUERIES.items():
        out = vol.intersect(sd, o, d, kw["compute_surface"], kw["max_footprint"])
        for k in FIELDS:
            v = out[k]
            if k == "distance":
                v = v.astype(np.float32)
                assert np.array_equal(v.astype(np.float64), out[k])
            data[f"{q}_{k}"] = v
    tr = vol.trace_ray_ref(o, d)
    for k in ("hit", "distance", "material"):
        data[f"traceref_{k}"] = tr[k]
    np.savez_compressed(HERE / f"{name}.npz", **data)
    print(name, "nodes", nodes.size // 8, "rays", o.shape[0], "hits", int(data["surface_hit"].sum()))


def main() -> None:
    oracle.build(reference=True)
    ref = oracle.Reference()
    small_fixture(ref, "spheres64", W.SceneSpec(cbq.SCENE_SPHERES, 6, 11, 16),
                  W.CameraSpec((-40.0, -40.0, 90.0), (32.0, 32.0, 32.0), 32, 32), 101)
    small_fixture(ref, "terrain64", W.terrain_scaled(6, 77), W.camera_scaled(6, 32, 32), 202)

    digests = {}
    # spheres-256: DAG built by the reference itself, traced by the reference.
    vol = reference_volume(ref, W.SPHERES_256)
    o, d = W.SPHERES_256_CAMERA.rays()
    sd = vol.find_subdags()
    digests["spheres256"] = {
        "scene": list(map(int, (W.SPHERES_256.kind, W.SPHERES_256.edge_log2, W.SPHERES_256.seed, W.SPHERES_256.param))),
        "canonical_dag_sha256": canonical_hash(vol.nodes(), vol.root),
        "node_count": int(vol.nodes().size // 8),
        "rays": int(o.shape[0]),
        "surface": output_digest(vol.intersect(sd, o, d, True, -1.0)),
        "lod_max_footprint": LOD_256,
        "lod": output_digest(vol.intersect(sd, o, d, True, LOD_256)),
    }
    # terrain-4096: libcbq's builder output handed to the reference via .dag.
    nodes, root = W.TERRAIN_4096.build()
    tvol = ref.volume_from_nodes(nodes, root)
    tsd = tvol.find_subdags()
    po, pd = W.TERRAIN_4096_CAMERA.rays()
    prim = tvol.intersect(tsd, po, pd, True, -1.0)
    bo, bd = W.bounce_from_hits(prim, po.shape[0])
    boun = tvol.intersect(tsd, bo, bd, True, -1.0)
    digests["terrain4096"] = {
        "scene": list(map(int, (W.TERRAIN_4096.kind, W.TERRAIN_4096.edge_log2, W.TERRAIN_4096.seed, W.TERRAIN_4096.param))),
        "canonical_dag_sha256": canonical_hash(nodes, root),
        "node_count": int(nodes.size // 8),
        "primary_rays": int(po.shape[0]),
        "primary": output_digest(prim),
        "bounce_rays_sha256": hashlib.sha256(bo.tobytes() + bd.tobytes()).hexdigest(),
        "bounce": output_digest(boun),
    }
    (HERE / "digests.json").write_text(json.dumps(digests, indent=1) + "\n")
    print(json.dumps(digests, indent=1))


if __name__ == "__main__":
    main()
