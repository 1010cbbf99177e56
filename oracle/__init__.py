"""Test-only checkers for the ray traversal.  TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may import
this package, and only to check or time against it.  The product (cubiquity_gb300)
never imports it.

Two checkers:
  * ``Oracle``     - liboracle.so, the plain-C restatement in esvo_oracle.c.
                     Builds anywhere with gcc.
  * ``Reference``  - _ref/libcbq_ref.so, the reference's own library sources
                     compiled in place plus ref_driver.cpp.  Available only where
                     the reference checkout is (REF in the Makefile).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

ORACLE_DIR = Path(__file__).resolve().parent
ORACLE_LIB = ORACLE_DIR / "_build" / "liboracle.so"
REF_LIB = ORACLE_DIR / "_ref" / "libcbq_ref.so"

_P = ctypes.c_void_p
_U64 = ctypes.c_uint64
_U32 = ctypes.c_uint32


class OrcSubdag(ctypes.Structure):
    _fields_ = [("lower", ctypes.c_int32 * 3), ("height", ctypes.c_int32), ("pad0", ctypes.c_uint32),
                ("node", ctypes.c_uint32), ("pad1", ctypes.c_uint32), ("pad2", ctypes.c_uint32)]


class OrcHits(ctypes.Structure):
    _fields_ = [("hit", _P), ("distance", _P), ("material", _P), ("position", _P), ("normal", _P),
                ("voxel", _P), ("status", _P)]


def build(reference: bool | None = None) -> None:
    """Builds liboracle.so, and _ref/libcbq_ref.so when the reference checkout
    exists.  Where the checkout is, is the Makefile's business (its REF, which
    CBQ_REFERENCE_ROOT in the environment overrides)."""
    make = ["make", "-s", "-C", str(ORACLE_DIR)]
    subprocess.run(make + ["all"], check=True)
    if reference is None:
        reference = subprocess.run(make + ["ref-check"], stdout=subprocess.DEVNULL,
                                   stderr=subprocess.DEVNULL).returncode == 0
    if reference:
        subprocess.run(make + ["ref"], check=True)


def reference_available() -> bool:
    return REF_LIB.exists()


def _ptr(a):
    return None if a is None else a.ctypes.data


def _subdag_array(subdags) -> "ctypes.Array":
    arr = (OrcSubdag * 8)()
    for i, s in enumerate(subdags):
        if hasattr(s, "lower_bound"):
            arr[i].lower[:] = list(s.lower_bound)
            arr[i].height = s.node_height
            arr[i].node = s.node_index
        elif hasattr(s, "lower"):
            arr[i].lower[:] = list(s.lower)
            arr[i].height = s.height
            arr[i].node = s.node
        else:  # (lower tuple, height, node)
            arr[i].lower[:] = list(s[0])
            arr[i].height = s[1]
            arr[i].node = s[2]
    return arr


def undefined_stack_rays(orc: "Oracle", nodes, subdags, origin_tmax, direction, **kw) -> np.ndarray:
    """Indices of rays whose result depends on never-written descent-stack slots
    (uninitialised in the reference, so its result there is undefined)."""
    a = orc.intersect(nodes, subdags, origin_tmax, direction, **kw)
    b = orc.intersect(nodes, subdags, origin_tmax, direction, unwritten_slot_is_start_node=True, **kw)
    diff = np.zeros(a["hit"].shape[0], bool)
    for k in ("hit", "material", "status", "voxel", "normal"):
        diff |= (a[k] != b[k]).reshape(diff.size, -1).any(axis=1)
    return np.nonzero(diff)[0]


def same_bits_nan_equal(a, b) -> bool:
    """Bit equality, except that every NaN equals every NaN: NaN payloads differ
    between x86, Arm and the GPU even for the reference itself."""
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    if a.shape != b.shape:
        return False
    if a.dtype.kind == "f" and b.dtype.kind == "f":
        if a.dtype != b.dtype:
            return False
        na, nb = np.isnan(a), np.isnan(b)
        if not np.array_equal(na, nb):
            return False
        a = np.where(na, 0, a)
        b = np.where(nb, 0, b)
    return np.array_equal(a.view(np.uint8), b.view(np.uint8))


def _alloc(n: int) -> dict:
    return {"hit": np.zeros(n, np.uint8), "distance": np.zeros(n, np.float32), "material": np.zeros(n, np.uint32),
            "position": np.zeros((n, 3), np.float32), "normal": np.zeros((n, 3), np.float32),
            "voxel": np.zeros((n, 3), np.int32), "status": np.zeros(n, np.uint8)}


class Oracle:
    """ctypes wrapper of liboracle.so (esvo_oracle.c)."""

    def __init__(self):
        if not ORACLE_LIB.exists():
            build(reference=False)
        lib = ctypes.CDLL(str(ORACLE_LIB))
        lib.orc_find_subdags.argtypes = [_P, _U64, _U32, ctypes.POINTER(OrcSubdag)]
        lib.orc_intersect_batch.argtypes = [_P, _U64, ctypes.POINTER(OrcSubdag), _P, _P, _U64, ctypes.c_int,
                                            ctypes.c_float, ctypes.c_int, ctypes.POINTER(OrcHits), ctypes.c_int]
        lib.orc_intersect_batch_ex.argtypes = lib.orc_intersect_batch.argtypes + [ctypes.c_int]
        lib.orc_count_fetches.argtypes = [_P, _U64, ctypes.POINTER(OrcSubdag), _P, _P, _U64, ctypes.c_int,
                                          ctypes.c_float, _P, ctypes.c_int]
        lib.orc_trace_fp64_batch.argtypes = [_P, _U64, ctypes.POINTER(OrcSubdag), _P, _P, _U64, _P, _P, _P,
                                             ctypes.c_int]
        self.lib = lib

    def find_subdags(self, nodes: np.ndarray, root: int):
        nodes = np.ascontiguousarray(nodes, dtype=np.uint32)
        out = (OrcSubdag * 8)()
        rc = self.lib.orc_find_subdags(_ptr(nodes), nodes.size // 8, root, out)
        if rc:
            raise RuntimeError(f"orc_find_subdags failed ({rc})")
        return [(tuple(s.lower), s.height, s.node) for s in out]

    def intersect(self, nodes, subdags, origin_tmax, direction, compute_surface=True, max_footprint=-1.0,
                  use_tmax=False, threads=0, unwritten_slot_is_start_node=False) -> dict:
        nodes = np.ascontiguousarray(nodes, dtype=np.uint32)
        o = np.ascontiguousarray(origin_tmax, dtype=np.float32).reshape(-1, 4)
        d = np.ascontiguousarray(direction, dtype=np.float32).reshape(-1, 4)
        n = o.shape[0]
        out = _alloc(n)
        hits = OrcHits(*[_ptr(out[k]) for k in ("hit", "distance", "material", "position", "normal", "voxel",
                                                "status")])
        rc = self.lib.orc_intersect_batch_ex(_ptr(nodes), nodes.size // 8, _subdag_array(subdags), _ptr(o), _ptr(d),
                                             n, 1 if compute_surface else 0, max_footprint, 1 if use_tmax else 0,
                                             ctypes.byref(hits), threads, 1 if unwritten_slot_is_start_node else 0)
        if rc:
            raise RuntimeError(f"orc_intersect_batch failed ({rc})")
        return out

    def count_fetches(self, nodes, subdags, origin_tmax, direction, compute_surface=True, max_footprint=-1.0,
                      threads=0) -> np.ndarray:
        nodes = np.ascontiguousarray(nodes, dtype=np.uint32)
        o = np.ascontiguousarray(origin_tmax, dtype=np.float32).reshape(-1, 4)
        d = np.ascontiguousarray(direction, dtype=np.float32).reshape(-1, 4)
        f = np.zeros(o.shape[0], np.uint32)
        rc = self.lib.orc_count_fetches(_ptr(nodes), nodes.size // 8, _subdag_array(subdags), _ptr(o), _ptr(d),
                                        o.shape[0], 1 if compute_surface else 0, max_footprint, _ptr(f), threads)
        if rc:
            raise RuntimeError(f"orc_count_fetches failed ({rc})")
        return f

    def trace_fp64(self, nodes, subdags, origin_tmax, direction, threads=0):
        nodes = np.ascontiguousarray(nodes, dtype=np.uint32)
        o = np.ascontiguousarray(origin_tmax, dtype=np.float32).reshape(-1, 4)
        d = np.ascontiguousarray(direction, dtype=np.float32).reshape(-1, 4)
        n = o.shape[0]
        hit = np.zeros(n, np.uint8)
        dist = np.zeros(n, np.float64)
        mat = np.zeros(n, np.uint32)
        rc = self.lib.orc_trace_fp64_batch(_ptr(nodes), nodes.size // 8, _subdag_array(subdags), _ptr(o), _ptr(d),
                                           n, _ptr(hit), _ptr(dist), _ptr(mat), threads)
        if rc:
            raise RuntimeError(f"orc_trace_fp64_batch failed ({rc})")
        return {"hit": hit, "distance": dist, "material": mat}


class RefSubDAG(ctypes.Structure):
    _fields_ = [("lowerBound", ctypes.c_int32 * 3), ("nodeHeight", ctypes.c_int32), ("padding0", ctypes.c_uint32),
                ("nodeIndex", ctypes.c_uint32), ("padding1", ctypes.c_uint32), ("padding2", ctypes.c_uint32)]


class Reference:
    """ctypes wrapper of _ref/libcbq_ref.so: the reference library itself."""

    def __init__(self):
        if not REF_LIB.exists():
            build(reference=True)
        if not REF_LIB.exists():
            raise RuntimeError("reference library not available")
        lib = ctypes.CDLL(str(REF_LIB))
        lib.ref_volume_new.restype = _P
        lib.ref_volume_free.argtypes = [_P]
        lib.ref_volume_set_voxels.argtypes = [_P, _P, _P, _U64]
        lib.ref_volume_fill.argtypes = [_P, ctypes.c_uint8]
        lib.ref_volume_bake.argtypes = [_P]
        lib.ref_volume_root.argtypes = [_P]
        lib.ref_volume_root.restype = _U32
        lib.ref_volume_node_count.argtypes = [_P]
        lib.ref_volume_node_count.restype = _U64
        lib.ref_volume_copy_nodes.argtypes = [_P, _P, _U64]
        lib.ref_volume_voxel.argtypes = [_P, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]
        lib.ref_volume_voxel.restype = ctypes.c_uint8
        lib.ref_volume_load.argtypes = [ctypes.c_char_p, ctypes.POINTER(_P)]
        lib.ref_volume_save.argtypes = [_P, ctypes.c_char_p]
        lib.ref_volume_from_nodes.argtypes = [_P, _U64, _U32, ctypes.POINTER(_P)]
        lib.ref_find_subdags.argtypes = [_P, ctypes.POINTER(RefSubDAG)]
        lib.ref_intersect_batch.argtypes = [_P, ctypes.POINTER(RefSubDAG), _P, _P, _U64, ctypes.c_int,
                                            ctypes.c_float, _P, _P, _P, _P, _P, _P, ctypes.c_int]
        lib.ref_trace_ray_ref_batch.argtypes = [_P, _P, _P, _U64, _P, _P, _P, ctypes.c_int]
        self.lib = lib

    # Volume lifecycle -----------------------------------------------------
    def new_volume(self):
        return RefVolume(self, self.lib.ref_volume_new())

    def volume_from_nodes(self, nodes: np.ndarray, root: int):
        nodes = np.ascontiguousarray(nodes, dtype=np.uint32)
        h = _P()
        rc = self.lib.ref_volume_from_nodes(_ptr(nodes), nodes.size // 8, root, ctypes.byref(h))
        if rc:
            raise RuntimeError(f"ref_volume_from_nodes failed ({rc})")
        return RefVolume(self, h.value)

    def load(self, path):
        h = _P()
        if self.lib.ref_volume_load(os.fsencode(path), ctypes.byref(h)):
            raise RuntimeError(f"cannot load {path}")
        return RefVolume(self, h.value)


class RefVolume:
    def __init__(self, ref: Reference, handle):
        self.ref = ref
        self.h = handle

    def __del__(self):
        try:
            if self.h:
                self.ref.lib.ref_volume_free(self.h)
                self.h = None
        except Exception:
            pass

    def set_voxels(self, xyz: np.ndarray, mat: np.ndarray) -> None:
        xyz = np.ascontiguousarray(xyz, dtype=np.int32).reshape(-1, 3)
        mat = np.ascontiguousarray(mat, dtype=np.uint8).reshape(-1)
        self.ref.lib.ref_volume_set_voxels(self.h, _ptr(xyz), _ptr(mat), xyz.shape[0])

    def fill(self, m: int) -> None:
        self.ref.lib.ref_volume_fill(self.h, m)

    def bake(self) -> None:
        self.ref.lib.ref_volume_bake(self.h)

    def save(self, path) -> None:
        self.ref.lib.ref_volume_save(self.h, os.fsencode(path))

    @property
    def root(self) -> int:
        return self.ref.lib.ref_volume_root(self.h)

    def nodes(self) -> np.ndarray:
        n = self.ref.lib.ref_volume_node_count(self.h)
        out = np.empty(n * 8, np.uint32)
        if self.ref.lib.ref_volume_copy_nodes(self.h, _ptr(out), n):
            raise RuntimeError("copy failed")
        return out

    def voxel(self, x, y, z) -> int:
        return self.ref.lib.ref_volume_voxel(self.h, x, y, z)

    def find_subdags(self):
        out = (RefSubDAG * 8)()
        self.ref.lib.ref_find_subdags(self.h, out)
        return [(tuple(s.lowerBound), s.nodeHeight, s.nodeIndex) for s in out]

    def intersect(self, subdags, origin_tmax, direction, compute_surface=True, max_footprint=-1.0, threads=0):
        o = np.ascontiguousarray(origin_tmax, dtype=np.float32).reshape(-1, 4)
        d = np.ascontiguousarray(direction, dtype=np.float32).reshape(-1, 4)
        n = o.shape[0]
        sd = (RefSubDAG * 8)()
        for i, (lb, h, node) in enumerate(subdags):
            sd[i].lowerBound[:] = list(lb)
            sd[i].nodeHeight = h
            sd[i].nodeIndex = node
        out = {"hit": np.zeros(n, np.uint8), "distance": np.zeros(n, np.float64),
               "material": np.zeros(n, np.uint32), "position": np.zeros((n, 3), np.float32),
               "normal": np.zeros((n, 3), np.float32), "voxel": np.zeros((n, 3), np.int32)}
        self.ref.lib.ref_intersect_batch(self.h, sd, _ptr(o), _ptr(d), n, 1 if compute_surface else 0,
                                         max_footprint, _ptr(out["hit"]), _ptr(out["distance"]),
                                         _ptr(out["material"]), _ptr(out["position"]), _ptr(out["normal"]),
                                         _ptr(out["voxel"]), threads)
        return out

    def trace_ray_ref(self, origin_tmax, direction, threads=0):
        o = np.ascontiguousarray(origin_tmax, dtype=np.float32).reshape(-1, 4)
        d = np.ascontiguousarray(direction, dtype=np.float32).reshape(-1, 4)
        n = o.shape[0]
        out = {"hit": np.zeros(n, np.uint8), "distance": np.zeros(n, np.float64),
               "material": np.zeros(n, np.uint32)}
        self.ref.lib.ref_trace_ray_ref_batch(self.h, _ptr(o), _ptr(d), n, _ptr(out["hit"]), _ptr(out["distance"]),
                                             _ptr(out["material"]), threads)
        return out
