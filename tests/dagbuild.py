"""Builds reference-format DAGs from small dense voxel arrays (test helper).

The node store follows storage.h:51-116: slots 0..255 are the self-referencing
material nodes, a child value below 256 is a uniform subtree of that material
(0 = empty), and an internal node whose eight children are one material value
collapses to that value (storage.cpp:261-263).  Identical nodes are shared.
The root sits at height 32 and spans [-2^31, 2^31) on each axis; a box of
edge 2^k placed at `origin` is reached through a chain of single-child nodes
(child ids from the unsigned coordinates' bits, storage.cpp:481-499)."""
import numpy as np


def build_dag(voxels: np.ndarray, origin=(0, 0, 0)):
    """voxels: uint8 array [z][y][x] of edge 2^k (k >= 1); origin: a multiple of
    2^k per axis.  Returns (nodes uint32[count * 8], root)."""
    edge = voxels.shape[0]
    k = edge.bit_length() - 1
    assert voxels.shape == (edge, edge, edge) and (1 << k) == edge and k >= 1
    assert all(int(o) % edge == 0 for o in origin)
    rows = [[m] * 8 for m in range(256)]
    index = {}

    def intern(children):
        if all(c == children[0] for c in children) and children[0] < 256:
            return children[0]
        key = tuple(children)
        if key not in index:
            index[key] = len(rows)
            rows.append(list(key))
        return index[key]

    def node(x, y, z, size):
        if size == 1:
            return int(voxels[z, y, x])
        h = size // 2
        return intern([node(x + (c & 1) * h, y + ((c >> 1) & 1) * h, z + ((c >> 2) & 1) * h, h)
                       for c in range(8)])

    top = node(0, 0, 0, edge)
    u = [(int(o) + (1 << 31)) & 0xFFFFFFFF for o in origin]
    cur = top
    for height in range(k + 1, 33):
        b = height - 1
        cid = ((u[0] >> b) & 1) | (((u[1] >> b) & 1) << 1) | (((u[2] >> b) & 1) << 2)
        children = [0] * 8
        children[cid] = cur
        if cur == 0:
            cur = 0  # nothing below: stays empty
            continue
        cur = len(rows)
        rows.append(children)
    if cur < 256:  # an empty (or uniform) volume still needs an internal root
        children = [0] * 8
        rows.append(children)
        cur = len(rows) - 1
    return np.array(rows, dtype=np.uint32).reshape(-1), cur


def random_voxels(rng, edge: int) -> np.ndarray:
    """Spheres, boxes, solid octants, noise and empty regions, 1-6 materials."""
    v = np.zeros((edge, edge, edge), np.uint8)
    mats = rng.integers(1, 256, size=rng.integers(1, 7))
    zz, yy, xx = np.meshgrid(np.arange(edge), np.arange(edge), np.arange(edge), indexing="ij")
    for _ in range(rng.integers(0, 4)):  # spheres
        c = rng.uniform(0, edge, 3)
        r = rng.uniform(1, edge / 3)
        v[(xx - c[0]) ** 2 + (yy - c[1]) ** 2 + (zz - c[2]) ** 2 <= r * r] = rng.choice(mats)
    for _ in range(rng.integers(0, 4)):  # boxes
        lo = rng.integers(0, edge, 3)
        hi = np.minimum(lo + rng.integers(1, edge, 3), edge)
        v[lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]] = rng.choice(mats)
    if rng.random() < 0.5:  # a solid aligned octant (a uniform subtree)
        h = edge // 2
        o = rng.integers(0, 2, 3) * h
        v[o[2]:o[2] + h, o[1]:o[1] + h, o[0]:o[0] + h] = rng.choice(mats)
    if rng.random() < 0.5:  # sparse noise
        mask = rng.random(v.shape) < rng.uniform(0.001, 0.05)
        v[mask] = rng.choice(mats, size=int(mask.sum()))
    if rng.random() < 0.3:  # carve an empty aligned octant
        h = edge // 2
        o = rng.integers(0, 2, 3) * h
        v[o[2]:o[2] + h, o[1]:o[1] + h, o[0]:o[0] + h] = 0
    return v


def random_rays(rng, origin, edge: int, n: int):
    """Rays from outside and inside the box in random, axis-aligned and
    diagonal directions; origin_tmax[:, 3] is a random tmax."""
    lo = np.array(origin, np.float64)
    o = np.empty((n, 4), np.float32)
    d = np.zeros((n, 4), np.float32)
    kind = rng.integers(0, 4, n)
    inside = lo + rng.uniform(-0.5, edge - 0.5, (n, 3))
    outside = lo + edge / 2 + rng.normal(size=(n, 3)) * edge * 1.5
    o[:, :3] = np.where((kind % 2 == 0)[:, None], inside, outside)
    target = lo + rng.uniform(0, edge, (n, 3))
    dirs = target - o[:, :3]
    axis = rng.integers(0, 3, n)
    aligned = np.zeros((n, 3))
    aligned[np.arange(n), axis] = rng.choice([-1.0, 1.0], n)
    diag = rng.choice([-1.0, 1.0], (n, 3))
    dirs = np.where((kind == 1)[:, None], aligned, dirs)
    dirs = np.where((kind == 3)[:, None] & (rng.random(n) < 0.3)[:, None], diag, dirs)
    dirs /= np.maximum(np.linalg.norm(dirs, axis=1, keepdims=True), 1e-30)
    d[:, :3] = dirs
    o[:, 3] = rng.uniform(0.0, 2.0 * edge, n)
    # Grid-aligned origins (voxel faces and centres) for the tie-breaking paths.
    snap = rng.random(n) < 0.15
    o[snap, :3] = np.round(o[snap, :3] * 2.0) / 2.0
    return o, d
