"""cbq_intersect_host_noalloc: host-buffer traversal without device allocation.

It exists for callers that must not call cudaMalloc (a frame-deadline render or
physics thread, where cudaMalloc can synchronise the device; a host application
whose allocator owns all device memory).  Its staging lives in a fixed array
compiled into the library, materialised when a DAG is created, so it must give
exactly what cbq_intersect_host gives, call after call, without the device's
free memory moving: not on the first call on a fresh DAG, and not on the first
call in a process either (this file runs alone as well as after the other
tests; run alone, its first call is the process's first).

This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

import cubiquity_gb300 as cbq  # noqa: E402
import oracle  # noqa: E402
from cubiquity_gb300 import workloads as W  # noqa: E402

FIELDS = ("hit", "distance", "material", "position", "normal", "voxel", "status")
MAX_RAYS = 65536  # CBQ_NOALLOC_MAX_RAYS


def _bind():
    fn = cbq.lib().cbq_intersect_host_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64,
                   ctypes.POINTER(cbq._Query), ctypes.POINTER(cbq._Hits)]
    fn.restype = ctypes.c_int
    return fn


def _call(fn, dag, o, d, query, fields=FIELDS):
    """One call; returns (status, hits, change of free device memory across it)."""
    full = cbq.alloc_host_hits(o.shape[0])
    out = {k: full[k] for k in fields}
    hits = cbq._Hits(*[out[k].ctypes.data if k in out else None for k in cbq.HIT_FIELDS])
    free_before = torch.cuda.mem_get_info()[0]
    st = fn(dag.handle, o.ctypes.data, d.ctypes.data, o.shape[0], ctypes.byref(query), ctypes.byref(hits))
    free_after = torch.cuda.mem_get_info()[0]
    return st, out, free_after - free_before


def _same(a, b, fields=FIELDS):
    for k in fields:
        assert oracle.same_bits_nan_equal(a[k], b[k]), k


def test_no_alloc_equals_host_entry_point_on_consecutive_calls():
    assert torch.cuda.is_available()
    torch.cuda.set_device(0)
    fn = _bind()
    nodes, root = W.terrain_scaled(8, 5).build()
    dag = cbq.Dag(nodes, root)
    q = cbq.Query().c()

    # Call 1: camera rays.  Call 2: a different, larger batch of bounce rays,
    # so stale contents from call 1 would show up as differences.
    o1, d1 = W.camera_scaled(8, 128, 96).rays()
    st, first, moved = _call(fn, dag, o1, d1, q)
    assert st == 0
    assert moved == 0, "the first no-allocation call changed free device memory"
    want1 = cbq.intersect_volume_host(dag, o1, d1)
    _same(first, want1)

    o2, d2 = W.bounce_from_hits(want1, MAX_RAYS)
    st, second, moved = _call(fn, dag, o2, d2, q)
    assert st == 0
    assert moved == 0, "the no-allocation entry point changed free device memory"
    _same(second, cbq.intersect_volume_host(dag, o2, d2))

    # Beyond the stated maximum: refused with CBQ_ERR_CAPACITY (10).
    o3 = np.zeros((MAX_RAYS + 1, 4), np.float32)
    d3 = np.zeros((MAX_RAYS + 1, 4), np.float32)
    d3[:, 0] = 1.0
    st, _, _ = _call(fn, dag, o3, d3, q)
    assert st == 10
    dag.destroy()


def test_no_alloc_first_call_on_a_fresh_dag_and_partial_outputs():
    """A DAG created after the others: its first call allocates nothing either.
    Only the hit flag and distance are asked for, with surface properties off
    (the skipped fields are neither written nor copied), and the results equal
    cbq_intersect_host's for the same fields and query."""
    torch.cuda.set_device(0)
    fn = _bind()
    nodes, root = W.SPHERES_256.build()
    dag = cbq.Dag(nodes, root)
    q = cbq.Query(compute_surface_properties=False)
    o, d = W.CameraSpec((-128.0, -128.0, 300.0), (128.0, 128.0, 128.0), 256, 200).rays()
    for _ in range(2):
        st, got, moved = _call(fn, dag, o, d, q.c(), fields=("hit", "distance"))
        assert st == 0
        assert moved == 0, "a call on a fresh DAG changed free device memory"
        want = cbq.intersect_volume_host(dag, o, d, compute_surface_properties=False,
                                         out={k: v for k, v in cbq.alloc_host_hits(o.shape[0]).items()
                                              if k in ("hit", "distance")})
        _same(got, want, fields=("hit", "distance"))
        assert int(got["hit"].sum()) > 0
    dag.destroy()
