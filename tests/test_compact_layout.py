"""The compact node store (LAYOUT_COMPACT), decoded on the host: every node
reachable from a SubDAG root has the same children as in the reference's
array, and an empty child is visible from the reference to its parent alone."""
from collections import deque

import numpy as np
import pytest

import cubiquity_gb300 as cbq
from cubiquity_gb300 import workloads as W


def child(store, ref, slot):
    mask = ref & 0xFF
    if not (mask >> slot) & 1:
        return 0
    return int(store[(ref >> 8) * 2 + bin(mask & ((1 << slot) - 1)).count("1")])


def check_equivalent(nodes, root):
    store, refs = cbq.compact_store(nodes, root)
    sds = cbq.find_subdags(nodes, root)
    seen = {}
    todo = deque()
    for sd, ref in zip(sds, refs):
        n = sd.node_index
        if n == 0:
            assert ref == 0
        elif n < 256:  # uniform octant: eight children of material n
            assert ref & 0xFF == 0xFF and all(child(store, ref, s) == n for s in range(8))
        else:
            todo.append((n, ref))
    while todo:
        n, ref = todo.popleft()
        if n in seen:
            assert seen[n] == ref  # one reference per node: the graph stays a DAG
            continue
        seen[n] = ref
        assert ref >= 256
        for s in range(8):
            c = int(nodes[8 * n + s])
            got = child(store, ref, s)
            if c < 256:
                assert got == c
            else:
                assert got >= 256
                todo.append((c, got))
    return store, seen


@pytest.mark.parametrize("spec", [W.SceneSpec(cbq.SCENE_SPHERES, 6, 21, 10), W.terrain_scaled(7, 31),
                                  W.SceneSpec(cbq.SCENE_CITY, 8, 41)])
def test_compact_store_has_the_same_children(spec):
    nodes, root = spec.build()
    store, seen = check_equivalent(nodes, root)
    assert store.nbytes < nodes.nbytes  # empty children take no room
    assert store[:2].tolist() == [0, 0]  # unit 0 is never a node


def test_compact_store_of_golden_dags(golden):
    name, fx = golden
    check_equivalent(fx["nodes"], int(fx["root"]))


def test_compact_store_edge_cases():
    nodes, root = W.SceneSpec(cbq.SCENE_SPHERES, 5, 3, 6).build()
    # An internal node whose eight children are empty is kept (as a reference
    # with an empty mask): a traversal must still see a non-zero child there.
    sd = [s for s in cbq.find_subdags(nodes, root) if s.node_index >= 256][0]
    bad = nodes.copy()
    empty = bad.size // 8
    bad = np.concatenate([bad, np.zeros(8, np.uint32)])
    k = next(s for s in range(8) if bad[8 * sd.node_index + s] >= 256)
    bad[8 * sd.node_index + k] = empty
    store, seen = check_equivalent(bad, root)
    assert seen[empty] & 0xFF == 0
    # A volume that is one material everywhere: SubDAGs rooted at materials.
    solid = np.repeat(np.arange(256, dtype=np.uint32), 8)
    solid = np.concatenate([solid, np.full(8, 7, np.uint32)])
    store, refs = cbq.compact_store(solid, 256)
    assert all(child(store, r, s) == 7 for r in refs for s in range(8))
