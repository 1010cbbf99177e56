"""cbq_intersect_host_noalloc: host-buffer traversal without device allocation.

It exists for callers that must not call cudaMalloc (a frame-deadline render or
physics thread, where cudaMalloc can synchronise the device; a host application
whose allocator owns all device memory).  Its staging lives in a fixed array
compiled into the library, so it must give exactly what cbq_intersect_host
gives, call after call, without the device's free memory moving.

This file is collected last on purpose, and runs alone as well as after the
other tests.
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


def _bind():
    fn = cbq.lib().cbq_intersect_host_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64,
                   ctypes.POINTER(cbq._Query), ctypes.POINTER(cbq._Hits)]
    fn.restype = ctypes.c_int
    return fn


def _call(fn, dag, o, d, query):
    out = cbq.alloc_host_hits(o.shape[0])
    hits = cbq._Hits(*[out[k].ctypes.data for k in cbq.HIT_FIELDS])
    st = fn(dag.handle, o.ctypes.data, d.ctypes.data, o.shape[0], ctypes.byref(query), ctypes.byref(hits))
    return st, out


def _same(a, b):
    for k in FIELDS:
        assert oracle.same_bits_nan_equal(a[k], b[k]), k


def test_no_alloc_equals_host_entry_point_on_consecutive_calls():
    assert torch.cuda.is_available()
    torch.cuda.set_device(0)
    fn = _bind()
    nodes, root = W.terrain_scaled(8, 5).build()
    dag = cbq.Dag(nodes, root)
    q = cbq.Query().c()
    max_rays = 65536  # CBQ_NOALLOC_MAX_RAYS

    # Call 1: camera rays.  Call 2: a different, larger batch of bounce rays,
    # so stale contents from call 1 would show up as differences.
    o1, d1 = W.camera_scaled(8, 128, 96).rays()
    st, first = _call(fn, dag, o1, d1, q)
    assert st == 0
    want1 = cbq.intersect_volume_host(dag, o1, d1)
    _same(first, want1)

    o2, d2 = W.bounce_from_hits(want1, max_rays)
    free_before = torch.cuda.mem_get_info()[0]
    st, second = _call(fn, dag, o2, d2, q)
    free_after = torch.cuda.mem_get_info()[0]
    assert st == 0
    assert free_after == free_before, "the no-allocation entry point changed free device memory"
    _same(second, cbq.intersect_volume_host(dag, o2, d2))

    # Beyond the stated maximum: refused with CBQ_ERR_CAPACITY (10).
    o3 = np.zeros((max_rays + 1, 4), np.float32)
    d3 = np.zeros((max_rays + 1, 4), np.float32)
    d3[:, 0] = 1.0
    st, _ = _call(fn, dag, o3, d3, q)
    assert st == 10
    dag.destroy()
