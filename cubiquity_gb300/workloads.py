"""Seeded synthetic workloads for the traversal (scenes + rays).

The reference publishes no dataset for this path (its sample .dag files are a
download), so these seeded scenes stand in, with the shapes and sizes of the
benchmark configurations:

  spheres-256   256^3, 64 spheres (centres in [32,224]^3, radii 8..40,
                material 1 + i mod 7, first sphere wins) over a ground slab z<32
                of material 8; 1024x1024 pinhole at (-128,-128,300) looking at
                (128,128,128), 60 degree vertical fov: 1,048,576 primary rays.
  terrain-4096  4096^3 fBm value-noise terrain (6 octaves, base period 1024,
                gain 0.5, heights in [512,2048]) with caves where 3D value noise
                (period 128) > 0.35 and 16 materials banded by height;
                2048x2048 primary rays plus 4,194,304 cosine-weighted bounce
                rays from the primary hits (origin offset 0.01 along the normal).

Everything is generated by libcbq (C++), so the same inputs come out on every
machine: ray generation uses only + - * / sqrt in double precision.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

import cubiquity_gb300 as cbq

TAN_30 = 0.57735026918962576451  # tan(60 degrees / 2)


@dataclass(frozen=True)
class SceneSpec:
    kind: int
    edge_log2: int
    seed: int
    param: int = 0

    def build(self, threads: int = 0):
        return cbq.build_scene(self.kind, self.edge_log2, self.seed, self.param, threads)

    def voxels(self, lo, size):
        return cbq.scene_voxels(self.kind, self.edge_log2, self.seed, self.param, lo, size)


@dataclass(frozen=True)
class CameraSpec:
    eye: tuple
    target: tuple
    width: int
    height: int
    tan_half_fov: float = TAN_30

    def rays(self):
        return cbq.pinhole_rays(self.eye, self.target, self.tan_half_fov, self.width, self.height)


SPHERES_256 = SceneSpec(cbq.SCENE_SPHERES, 8, 20240607, 64)
SPHERES_256_CAMERA = CameraSpec((-128.0, -128.0, 300.0), (128.0, 128.0, 128.0), 1024, 1024)

TERRAIN_4096 = SceneSpec(cbq.SCENE_TERRAIN, 12, 4096001)
TERRAIN_4096_CAMERA = CameraSpec((-1024.0, -1024.0, 3072.0), (2048.0, 2048.0, 1024.0), 2048, 2048)
TERRAIN_BOUNCE_SEED = 0xB0B0C0DE


def terrain_scaled(edge_log2: int, seed: int = 4096001) -> SceneSpec:
    return SceneSpec(cbq.SCENE_TERRAIN, edge_log2, seed)


def camera_scaled(edge_log2: int, width: int, height: int) -> CameraSpec:
    """The terrain camera of TERRAIN_4096_CAMERA scaled to an edge of 2^edge_log2."""
    s = (1 << edge_log2) / 4096.0
    return CameraSpec(tuple(v * s for v in TERRAIN_4096_CAMERA.eye), tuple(v * s for v in TERRAIN_4096_CAMERA.target),
                      width, height)


@dataclass(frozen=True)
class BatchVolume:
    """One volume of the batching workload and its ray batch: `pinhole` camera
    rays at the volume plus `interior` rays from uniform interior points in
    uniform directions."""
    scene: SceneSpec
    camera: CameraSpec
    interior: int
    ray_seed: int

    @property
    def rays(self) -> int:
        return self.camera.width * self.camera.height + self.interior

    def make_rays(self):
        o1, d1 = self.camera.rays()
        e = float(1 << self.scene.edge_log2)
        o2, d2 = cbq.sphere_rays((0.0, 0.0, 0.0), (e, e, e), self.interior, self.ray_seed)
        return np.concatenate([o1, o2]), np.concatenate([d1, d2])


def batch_volumes(count: int = 64, seed: int = 20240610, edge_log2=(7, 11), rays=(16384, 1 << 20)):
    """The batching workload: `count` volumes of edge 2^k, k uniform in
    edge_log2, each a seeded sphere or terrain scene, each with a ray batch of
    log-uniform size in `rays`, half pinhole rays at the volume and half rays
    from uniform interior points in uniform directions.  Deterministic on every
    machine (Python's Mersenne Twister; scenes and rays come from libcbq)."""
    import math
    import random

    rng = random.Random(seed)
    out = []
    for i in range(count):
        k = rng.randint(edge_log2[0], edge_log2[1])
        kind = cbq.SCENE_SPHERES if rng.random() < 0.5 else cbq.SCENE_TERRAIN
        scene = SceneSpec(kind, k, seed * 1000 + i, 64 if kind == cbq.SCENE_SPHERES else 0)
        n = int(round(math.exp(rng.uniform(math.log(rays[0]), math.log(rays[1])))))
        w = max(1, int(math.isqrt(n // 2)))
        h = max(1, (n // 2) // w)
        e = float(1 << k)
        theta = rng.uniform(0.0, 2.0 * math.pi)
        phi = rng.uniform(0.15, 1.2)  # elevation above the horizon
        c = (e / 2, e / 2, e / 4)
        r = 1.6 * e
        eye = (c[0] + r * math.cos(phi) * math.cos(theta), c[1] + r * math.cos(phi) * math.sin(theta),
               c[2] + r * math.sin(phi))
        out.append(BatchVolume(scene, CameraSpec(eye, c, w, h), n - w * h, seed * 7919 + i))
    return out


CITY_8192 = SceneSpec(cbq.SCENE_CITY, 13, 8192001)
CITY_EMISSIVE = (7, 23)  # the two emissive building materials


def city_camera(edge_log2: int = 13):
    """Eye and target of the city pathtracer view (z up), scaled to the edge."""
    e = float(1 << edge_log2)
    return (-0.15 * e, -0.2 * e, 0.45 * e), (0.55 * e, 0.5 * e, 0.0)


def city_materials(seed: int = 77) -> np.ndarray:
    """(256, 2, 3) albedo/emission: ground (1) grey, 32 building materials
    (2..33) with seeded albedo in [0.2, 0.9], two of them emissive."""
    import random

    rng = random.Random(seed)
    m = np.zeros((256, 2, 3), np.float32)
    m[:, 0] = 0.5
    m[1, 0] = (0.45, 0.45, 0.42)
    for k in range(2, 34):
        m[k, 0] = [rng.uniform(0.2, 0.9) for _ in range(3)]
    for k in CITY_EMISSIVE:
        m[k, 1] = (4.0, 3.4, 2.6)
    return m


SERVE_EDGES_LOG2 = (10, 11, 12, 10, 11, 12, 11, 10)


def serve_volumes(seed: int = 4242):
    """The serving workload's 8 resident DAGs: seeded terrain scenes with edges
    1024..4096."""
    return [terrain_scaled(k, seed + i) for i, k in enumerate(SERVE_EDGES_LOG2)]


def serve_ray_pools(scene: SceneSpec, collision: int, view_side: int, seed: int):
    """Ray pools from which serving requests take contiguous slices:
    collision rays from uniform points of the lower half of the volume (where
    the terrain is) in uniform directions, with tmax uniform in [8, 64]
    voxels; and unbounded view rays of a view_side^2 pinhole camera."""
    import random

    e = float(1 << scene.edge_log2)
    co, cd = cbq.sphere_rays((0.0, 0.0, 0.0), (e, e, e / 2), collision, seed)
    rng = random.Random(seed)
    co[:, 3] = np.array([rng.uniform(8.0, 64.0) for _ in range(collision)], dtype=np.float32)
    vo, vd = camera_scaled(scene.edge_log2, view_side, view_side).rays()
    return (co, cd), (vo, vd)


@dataclass(frozen=True)
class ServeRequest:
    volume: int          # index into serve_volumes()
    collision: bool      # True: tmax-bounded collision rays; False: unbounded view rays
    start: int           # slice start in the pool
    count: int


def serve_requests(count: int, pool_sizes: tuple, seed: int = 99, rays=(1024, 262144), collision_share=0.7,
                   volumes: int = len(SERVE_EDGES_LOG2)):
    """Request stream: sizes log-uniform in `rays`, 70% collision and 30% view
    rays, volumes uniform.  pool_sizes = (collision pool size, view pool size)."""
    import math
    import random

    rng = random.Random(seed)
    out = []
    for _ in range(count):
        n = int(round(math.exp(rng.uniform(math.log(rays[0]), math.log(rays[1])))))
        coll = rng.random() < collision_share
        size = pool_sizes[0] if coll else pool_sizes[1]
        n = min(n, size)
        out.append(ServeRequest(rng.randrange(volumes), coll, rng.randrange(0, size - n + 1), n))
    return out


def bounce_from_hits(hits: dict, n: int, seed: int = TERRAIN_BOUNCE_SEED):
    """Bounce rays from the hits of a primary pass (host arrays or tensors)."""
    hit = _np(hits["hit"]).astype(bool)
    pos = _np(hits["position"])[hit]
    nrm = _np(hits["normal"])[hit]
    if pos.shape[0] == 0:
        raise ValueError("no primary hits to bounce from")
    return cbq.bounce_rays(pos, nrm, n, seed)


def _np(a):
    if isinstance(a, np.ndarray):
        return a
    return a.detach().cpu().numpy()
