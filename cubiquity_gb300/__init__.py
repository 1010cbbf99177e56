"""cubiquity_gb300: GB300-native sparse-voxel-DAG ray traversal.

Python mirror of the C ABI in include/cubiquity_gb300.h (libcbq.so, loaded with
ctypes).  Names follow the reference's ray-cast interface
(src/library/raytracing.h): ``find_subdags`` ~ ``findSubDAGs``,
``intersect_volume`` ~ ``intersectVolume`` (batched), with the same argument
meaning (``compute_surface_properties``, ``max_footprint``) and the same result
fields (hit, distance, material, position, normal) plus the integer hit voxel.

There is no CPU fallback: importing this package fails if libcbq.so has not been
built, and every traversal call runs the CUDA kernels.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass
from pathlib import Path

import numpy as np

PKG_DIR = Path(__file__).resolve().parent
LIB_PATH = PKG_DIR / "libcbq.so"

MATERIAL_COUNT = 256
MAX_FOOTPRINT_DISABLED = -1.0
QUERY_TMAX = 0x1
RAY_OK, RAY_ITER_LIMIT, RAY_STUCK = 0, 1, 2
SCENE_SPHERES, SCENE_TERRAIN, SCENE_CITY = 0, 1, 2

_STATUS = {
    0: "ok", 1: "invalid argument", 2: "malformed DAG", 3: "out of memory", 4: "CUDA error", 5: "timeout",
    6: "I/O error", 7: "busy", 8: "not found", 9: "cancelled", 10: "request exceeds capacity", 11: "shut down",
}


class CbqError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        super().__init__(f"{what}: {_STATUS.get(status, 'unknown status')} ({status})")


class SubDag(ctypes.Structure):
    """cbq_subdag: the reference's SubDAG layout (raytracing.h:57-65)."""
    _fields_ = [("lower_bound", ctypes.c_int32 * 3), ("node_height", ctypes.c_int32),
                ("padding0", ctypes.c_uint32), ("node_index", ctypes.c_uint32),
                ("padding1", ctypes.c_uint32), ("padding2", ctypes.c_uint32)]

    def as_tuple(self):
        return (tuple(self.lower_bound), self.node_height, self.node_index)


class _Rays(ctypes.Structure):
    _fields_ = [("origin_tmax", ctypes.c_void_p), ("direction", ctypes.c_void_p)]


class _Hits(ctypes.Structure):
    _fields_ = [("hit", ctypes.c_void_p), ("distance", ctypes.c_void_p), ("material", ctypes.c_void_p),
                ("position", ctypes.c_void_p), ("normal", ctypes.c_void_p), ("voxel", ctypes.c_void_p),
                ("status", ctypes.c_void_p)]


class _Query(ctypes.Structure):
    _fields_ = [("compute_surface", ctypes.c_int32), ("max_footprint", ctypes.c_float),
                ("flags", ctypes.c_uint32), ("image_width", ctypes.c_uint32)]


KERNEL_AUTO, KERNEL_NESTED, KERNEL_FLAT = 0, 1, 2


STACK_SHARED, STACK_LOCAL = 0, 1
FORM_PLAIN, FORM_PERSISTENT, FORM_SORTED = 0, 1, 2


class LaunchConfig(ctypes.Structure):
    """cbq_launch_config."""
    _fields_ = [("kernel", ctypes.c_int32), ("block", ctypes.c_int32), ("chunk", ctypes.c_uint32),
                ("refill_min", ctypes.c_uint32), ("stack", ctypes.c_int32), ("form", ctypes.c_int32),
                ("steps", ctypes.c_int32), ("registers", ctypes.c_int32)]

    def as_dict(self):
        return {"kernel": self.kernel, "block": self.block, "chunk": self.chunk, "refill_min": self.refill_min,
                "stack": self.stack, "form": self.form, "steps": self.steps, "registers": self.registers}


class _DagInfo(ctypes.Structure):
    _fields_ = [("node_count", ctypes.c_uint64), ("bytes", ctypes.c_uint64), ("root", ctypes.c_uint32),
                ("max_subdag_height", ctypes.c_int32), ("subdags", SubDag * 8),
                ("device_nodes", ctypes.c_void_p), ("layout", ctypes.c_uint32), ("device_bytes", ctypes.c_uint64)]


def _load() -> ctypes.CDLL:
    if not LIB_PATH.exists():
        raise ImportError(
            f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
            "(there is no CPU fallback for the traversal)")
    return ctypes.CDLL(str(LIB_PATH))


_lib = _load()

_P = ctypes.c_void_p
_U64 = ctypes.c_uint64
_U32 = ctypes.c_uint32
_I32 = ctypes.c_int32


def _sig(name, argtypes, restype=ctypes.c_int):
    fn = getattr(_lib, name)
    fn.argtypes = argtypes
    fn.restype = restype
    return fn


_sig("cbq_status_string", [ctypes.c_int], ctypes.c_char_p)
_sig("cbq_abi_version", [], ctypes.c_int)
_sig("cbq_dag_validate", [_P, _U64, _U32])
_sig("cbq_find_subdags", [_P, _U64, _U32, ctypes.POINTER(SubDag)])
_sig("cbq_dag_create", [_P, _U64, _U32, ctypes.POINTER(_P)])
_sig("cbq_dag_create_ex", [_P, _U64, _U32, _U32, ctypes.POINTER(_P)])
_sig("cbq_compact_store", [_P, _U64, _U32, ctypes.POINTER(ctypes.POINTER(ctypes.c_uint32)), ctypes.POINTER(_U64),
                           ctypes.POINTER(_U32)])
_sig("cbq_dag_destroy", [_P])
_sig("cbq_dag_get_info", [_P, ctypes.POINTER(_DagInfo)])
_sig("cbq_dag_set_l2_persistence", [_P, _P, ctypes.c_float])
_sig("cbq_dag_set_launch_config", [_P, ctypes.POINTER(LaunchConfig)])
_sig("cbq_dag_get_launch_config", [_P, ctypes.POINTER(LaunchConfig)])
_sig("cbq_intersect", [_P, ctypes.POINTER(_Rays), _U64, ctypes.POINTER(_Query), ctypes.POINTER(_Hits), _P])
_sig("cbq_intersect_host", [_P, _P, _P, _U64, ctypes.POINTER(_Query), ctypes.POINTER(_Hits)])
_sig("cbq_intersect_persistent", [_P, ctypes.POINTER(_Rays), _U64, ctypes.POINTER(_Query), ctypes.POINTER(_Hits),
                                  _P, _U32, _P])
_sig("cbq_count_fetches", [_P, ctypes.POINTER(_Rays), _U64, ctypes.POINTER(_Query), _P, _P])
_sig("cbq_scratch_bytes", [_U64], _U64)
_sig("cbq_intersect_auto", [_P, ctypes.POINTER(_Rays), _U64, ctypes.POINTER(_Query), ctypes.POINTER(_Hits), _P, _U64,
                            _P])
_sig("cbq_autotune", [_P, ctypes.POINTER(_Rays), _U64, ctypes.POINTER(_Query), ctypes.POINTER(_Hits), _P, _U64,
                      ctypes.c_int32, ctypes.POINTER(LaunchConfig), ctypes.POINTER(ctypes.c_float), _P])
_sig("cbq_build_scene", [ctypes.c_int, ctypes.c_int, _U64, ctypes.c_int, ctypes.c_int,
                         ctypes.POINTER(ctypes.POINTER(ctypes.c_uint32)), ctypes.POINTER(_U64),
                         ctypes.POINTER(_U32)])
_sig("cbq_scene_voxels", [ctypes.c_int, ctypes.c_int, _U64, ctypes.c_int, _I32, _I32, _I32, _I32, _I32, _I32, _P])
_sig("cbq_free", [_P], None)
_sig("cbq_dag_voxel", [_P, _U64, _U32, _I32, _I32, _I32, ctypes.POINTER(ctypes.c_uint8)])
_sig("cbq_dag_save", [ctypes.c_char_p, _P, _U64, _U32])
_sig("cbq_dag_load", [ctypes.c_char_p, ctypes.POINTER(ctypes.POINTER(ctypes.c_uint32)), ctypes.POINTER(_U64),
                      ctypes.POINTER(_U32)])
_sig("cbq_dag_reorder_bfs", [_P, _U64, _U32, _P, ctypes.POINTER(_U64), ctypes.POINTER(_U32)])
_sig("cbq_gen_pinhole_rays", [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), ctypes.c_double,
                              _I32, _I32, _P, _P])
_sig("cbq_gen_bounce_rays", [_P, _P, _U64, _U64, _U64, _P, _P])
_sig("cbq_measure_l2", [_U64, ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)])
_sig("cbq_gen_sphere_rays", [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), _U64, _U64, _P, _P])


class _Job(ctypes.Structure):
    _fields_ = [("dag", ctypes.c_void_p), ("rays", _Rays), ("ray_count", ctypes.c_uint64), ("hits", _Hits)]


_sig("cbq_batch_create", [ctypes.POINTER(_Job), ctypes.c_int32, ctypes.POINTER(_Query), ctypes.POINTER(_P)])
_sig("cbq_batch_set_config", [_P, ctypes.c_int32, _U32])
_sig("cbq_batch_get_config", [_P, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(_U32), ctypes.POINTER(_U64)])
class _BatchConfig(ctypes.Structure):
    _fields_ = [("block", ctypes.c_int32), ("refill_min", ctypes.c_uint32), ("steps", ctypes.c_int32),
                ("registers", ctypes.c_int32), ("stack", ctypes.c_int32), ("form", ctypes.c_int32)]


_sig("cbq_batch_set_launch_config", [_P, ctypes.POINTER(_BatchConfig)])
_sig("cbq_batch_get_launch_config", [_P, ctypes.POINTER(_BatchConfig)])
_sig("cbq_batch_autotune", [_P, _P, ctypes.c_int32])
_sig("cbq_batch_launch", [_P, _P])
_sig("cbq_batch_set_l2_persistence", [_P, _P, ctypes.c_float])
_sig("cbq_batch_launch_direct", [_P, _P])
_sig("cbq_batch_destroy", [_P])
_sig("cbq_intersect_batch", [ctypes.POINTER(_Job), ctypes.c_int32, ctypes.POINTER(_Query), _P])


def sphere_rays(lo, hi, n: int, seed: int) -> tuple[np.ndarray, np.ndarray]:
    """Origins uniform in the box [lo, hi], directions uniform on the sphere."""
    o = np.empty((n, 4), dtype=np.float32)
    d = np.empty((n, 4), dtype=np.float32)
    _check(_lib.cbq_gen_sphere_rays((ctypes.c_double * 3)(*lo), (ctypes.c_double * 3)(*hi), n, seed, _np_ptr(o),
                                    _np_ptr(d)), "cbq_gen_sphere_rays")
    return o, d


LOG_DEBUG, LOG_INFO, LOG_WARNING = 0, 1, 2
LOG_FN = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_int32, ctypes.c_char_p)
_sig("cbq_set_log_handler", [LOG_FN, ctypes.c_void_p], None)
_log_keep = [None]


def set_log_handler(fn) -> None:
    """Routes the library's diagnostics to fn(level, message); None disables."""
    cb = LOG_FN(lambda user, level, msg: fn(level, msg.decode(errors="replace"))) if fn else LOG_FN()
    _log_keep[0] = cb
    _lib.cbq_set_log_handler(cb, None)


def _check(status: int, what: str) -> None:
    if status != 0:
        raise CbqError(status, what)


def lib() -> ctypes.CDLL:
    """The loaded libcbq.so (for callers that bind further entry points)."""
    return _lib


def _np_ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data


def _nodes_arg(nodes: np.ndarray) -> np.ndarray:
    nodes = np.ascontiguousarray(nodes, dtype=np.uint32).reshape(-1)
    if nodes.size % 8 != 0:
        raise ValueError("node array length must be a multiple of 8")
    return nodes


# ----------------------------------------------------------------- host helpers

def validate(nodes: np.ndarray, root: int) -> None:
    n = _nodes_arg(nodes)
    _check(_lib.cbq_dag_validate(_np_ptr(n), n.size // 8, root), "cbq_dag_validate")


def find_subdags(nodes: np.ndarray, root: int) -> list[SubDag]:
    """findSubDAGs (raytracing.cpp:89-97)."""
    n = _nodes_arg(nodes)
    out = (SubDag * 8)()
    _check(_lib.cbq_find_subdags(_np_ptr(n), n.size // 8, root, out), "cbq_find_subdags")
    return list(out)


def _take_malloced(ptr, count_words: int) -> np.ndarray:
    arr = np.ctypeslib.as_array(ptr, shape=(count_words,)).copy()
    _lib.cbq_free(ctypes.cast(ptr, ctypes.c_void_p))
    return arr


def compact_store(nodes: np.ndarray, root: int) -> tuple[np.ndarray, list[int]]:
    """The compact node store (LAYOUT_COMPACT) and the SubDAG root references in it."""
    n = _nodes_arg(nodes)
    p = ctypes.POINTER(ctypes.c_uint32)()
    words = _U64()
    refs = (_U32 * 8)()
    _check(_lib.cbq_compact_store(_np_ptr(n), n.size // 8, root, ctypes.byref(p), ctypes.byref(words), refs),
           "cbq_compact_store")
    return _take_malloced(p, words.value), list(refs)


def build_scene(kind: int, edge_log2: int, seed: int, param: int = 0, threads: int = 0) -> tuple[np.ndarray, int]:
    """Canonical DAG of a seeded scene; returns (nodes uint32[count*8], root)."""
    p = ctypes.POINTER(ctypes.c_uint32)()
    cnt = _U64()
    root = _U32()
    _check(_lib.cbq_build_scene(kind, edge_log2, seed, param, threads, ctypes.byref(p), ctypes.byref(cnt),
                                ctypes.byref(root)), "cbq_build_scene")
    return _take_malloced(p, cnt.value * 8), root.value


def scene_voxels(kind: int, edge_log2: int, seed: int, param: int, lo, size) -> np.ndarray:
    """Voxel materials of a scene over a box, shape (sz, sy, sx)."""
    sx, sy, sz = (int(v) for v in size)
    out = np.empty((sz, sy, sx), dtype=np.uint8)
    _check(_lib.cbq_scene_voxels(kind, edge_log2, seed, param, int(lo[0]), int(lo[1]), int(lo[2]), sx, sy, sz,
                                 _np_ptr(out)), "cbq_scene_voxels")
    return out


def dag_voxel(nodes: np.ndarray, root: int, x: int, y: int, z: int) -> int:
    """Volume::voxel (storage.cpp:481-499)."""
    n = _nodes_arg(nodes)
    m = ctypes.c_uint8()
    _check(_lib.cbq_dag_voxel(_np_ptr(n), n.size // 8, root, x, y, z, ctypes.byref(m)), "cbq_dag_voxel")
    return m.value


def save_dag(path: str | os.PathLike, nodes: np.ndarray, root: int) -> None:
    n = _nodes_arg(nodes)
    _check(_lib.cbq_dag_save(os.fsencode(path), _np_ptr(n), n.size // 8, root), "cbq_dag_save")


def load_dag(path: str | os.PathLike) -> tuple[np.ndarray, int]:
    p = ctypes.POINTER(ctypes.c_uint32)()
    cnt = _U64()
    root = _U32()
    _check(_lib.cbq_dag_load(os.fsencode(path), ctypes.byref(p), ctypes.byref(cnt), ctypes.byref(root)),
           "cbq_dag_load")
    return _take_malloced(p, cnt.value * 8), root.value


def reorder_bfs(nodes: np.ndarray, root: int) -> tuple[np.ndarray, int]:
    n = _nodes_arg(nodes)
    out = np.empty_like(n)
    cnt = _U64()
    r = _U32()
    _check(_lib.cbq_dag_reorder_bfs(_np_ptr(n), n.size // 8, root, _np_ptr(out), ctypes.byref(cnt), ctypes.byref(r)),
           "cbq_dag_reorder_bfs")
    return out[: cnt.value * 8].copy(), r.value


def canonical_hash(nodes: np.ndarray, root: int) -> str:
    """SHA-256 of the DAG renumbered breadth-first: equal iff the graphs are equal."""
    import hashlib
    canon, croot = reorder_bfs(nodes, root)
    h = hashlib.sha256()
    h.update(np.uint32(croot).tobytes())
    h.update(canon.tobytes())
    return h.hexdigest()


def pinhole_rays(eye, target, tan_half_fov: float, width: int, height: int) -> tuple[np.ndarray, np.ndarray]:
    """Scanline-order pinhole rays as (origin_tmax[n,4], direction[n,4]) float32."""
    n = width * height
    o = np.empty((n, 4), dtype=np.float32)
    d = np.empty((n, 4), dtype=np.float32)
    e = (ctypes.c_double * 3)(*eye)
    t = (ctypes.c_double * 3)(*target)
    _check(_lib.cbq_gen_pinhole_rays(e, t, tan_half_fov, width, height, _np_ptr(o), _np_ptr(d)),
           "cbq_gen_pinhole_rays")
    return o, d


def bounce_rays(hit_position: np.ndarray, hit_normal: np.ndarray, n: int, seed: int) -> tuple[np.ndarray, np.ndarray]:
    """Cosine-weighted bounce rays from hit points (pathtracing_demo.cpp:163-166)."""
    hp = np.ascontiguousarray(hit_position, dtype=np.float32).reshape(-1, 3)
    hn = np.ascontiguousarray(hit_normal, dtype=np.float32).reshape(-1, 3)
    o = np.empty((n, 4), dtype=np.float32)
    d = np.empty((n, 4), dtype=np.float32)
    _check(_lib.cbq_gen_bounce_rays(_np_ptr(hp), _np_ptr(hn), hp.shape[0], n, seed, _np_ptr(o), _np_ptr(d)),
           "cbq_gen_bounce_rays")
    return o, d


# --------------------------------------------------------------- device DAG

def measure_l2(working_set_bytes: int = 64 << 20, iterations: int = 20) -> tuple[float, float]:
    """(streaming L2 read GB/s, random 32-byte-sector reads in Gsectors/s) on the current device."""
    a = ctypes.c_double()
    b = ctypes.c_double()
    _check(_lib.cbq_measure_l2(working_set_bytes, iterations, ctypes.byref(a), ctypes.byref(b)), "cbq_measure_l2")
    return a.value, b.value


HIT_FIELDS = ("hit", "distance", "material", "position", "normal", "voxel", "status")


@dataclass
class Query:
    compute_surface_properties: bool = True
    max_footprint: float = MAX_FOOTPRINT_DISABLED
    use_tmax: bool = False
    image_width: int = 0  # rays are the pixels of a row-major image this wide (see cbq_query)

    def c(self) -> _Query:
        return _Query(1 if self.compute_surface_properties else 0, float(self.max_footprint),
                      QUERY_TMAX if self.use_tmax else 0, int(self.image_width))


class Dag:
    """A DAG resident on the current CUDA device (cbq_dag).  layout selects the
    device node store (LAYOUT_REFERENCE, or LAYOUT_COMPACT where possible;
    see .layout)."""

    def __init__(self, nodes: np.ndarray, root: int, layout: int = 0):
        n = _nodes_arg(nodes)
        h = _P()
        _check(_lib.cbq_dag_create_ex(_np_ptr(n), n.size // 8, root, layout, ctypes.byref(h)), "cbq_dag_create_ex")
        self._h = h
        info = _DagInfo()
        _check(_lib.cbq_dag_get_info(h, ctypes.byref(info)), "cbq_dag_get_info")
        self.node_count = info.node_count
        self.bytes = info.bytes
        self.root = info.root
        self.max_subdag_height = info.max_subdag_height
        self.subdags = list(info.subdags)
        self.device_nodes = info.device_nodes
        self.layout = info.layout
        self.device_bytes = info.device_bytes

    @property
    def handle(self):
        if self._h is None:
            raise RuntimeError("DAG destroyed")
        return self._h

    def destroy(self) -> None:
        if getattr(self, "_h", None) is not None:
            _lib.cbq_dag_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

    def set_launch_config(self, kernel: int = KERNEL_AUTO, block: int = 0, chunk: int = 0,
                          refill_min: int = 0, stack: int = STACK_SHARED, form: int = FORM_PERSISTENT,
                          steps: int = 16, registers: int = 0) -> None:
        cfg = LaunchConfig(kernel, block, chunk, refill_min, stack, form, steps, registers)
        _check(_lib.cbq_dag_set_launch_config(self.handle, ctypes.byref(cfg)), "cbq_dag_set_launch_config")

    def launch_config(self) -> dict:
        cfg = LaunchConfig()
        _check(_lib.cbq_dag_get_launch_config(self.handle, ctypes.byref(cfg)), "cbq_dag_get_launch_config")
        return cfg.as_dict()

    def set_l2_persistence(self, fraction: float, stream=None) -> None:
        _check(_lib.cbq_dag_set_l2_persistence(self.handle, _stream_ptr(stream), fraction),
               "cbq_dag_set_l2_persistence")


def _stream_ptr(stream):
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


def _torch_ptr(t):
    return None if t is None else t.data_ptr()


def alloc_hits(n: int, device="cuda", fields=HIT_FIELDS) -> dict:
    import torch
    shapes = {"hit": ((n,), torch.uint8), "distance": ((n,), torch.float32), "material": ((n,), torch.int32),
              "position": ((n, 3), torch.float32), "normal": ((n, 3), torch.float32),
              "voxel": ((n, 3), torch.int32), "status": ((n,), torch.uint8)}
    return {k: torch.empty(*shapes[k][0], dtype=shapes[k][1], device=device) for k in fields}


def _hits_struct(out: dict) -> _Hits:
    return _Hits(*[_torch_ptr(out.get(k)) for k in HIT_FIELDS])


def _check_rays_tensor(t, n=None):
    import torch
    if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float32 and t.dim() == 2
            and t.shape[1] == 4 and t.is_contiguous()):
        raise ValueError("rays must be contiguous float32 CUDA tensors of shape (n, 4)")
    if n is not None and t.shape[0] != n:
        raise ValueError("origin and direction arrays differ in length")


def intersect_volume(dag: Dag, origin_tmax, direction, compute_surface_properties: bool = True,
                     max_footprint: float = MAX_FOOTPRINT_DISABLED, use_tmax: bool = False, out: dict | None = None,
                     stream=None, image_width: int = 0) -> dict:
    """Batched intersectVolume (raytracing.cpp:397-478) on device tensors.

    origin_tmax, direction: float32 CUDA tensors (n, 4).  Returns a dict of
    device tensors (see HIT_FIELDS); pass ``out`` to reuse buffers.  When the
    rays are the pixels of a row-major image, ``image_width`` lets the kernel
    take them in 4x8 pixel tiles (same results; see cbq_query.image_width).
    """
    _check_rays_tensor(origin_tmax)
    n = origin_tmax.shape[0]
    _check_rays_tensor(direction, n)
    if out is None:
        out = alloc_hits(n, origin_tmax.device)
    rays = _Rays(origin_tmax.data_ptr(), direction.data_ptr())
    q = Query(compute_surface_properties, max_footprint, use_tmax, image_width).c()
    _check(_lib.cbq_intersect(dag.handle, ctypes.byref(rays), n, ctypes.byref(q), ctypes.byref(_hits_struct(out)),
                              _stream_ptr(stream)), "cbq_intersect")
    return out


def intersect_volume_persistent(dag: Dag, origin_tmax, direction, work_counter, compute_surface_properties=True,
                                max_footprint=MAX_FOOTPRINT_DISABLED, use_tmax=False, chunk: int = 0,
                                out: dict | None = None, stream=None, image_width: int = 0) -> dict:
    """The persistent-warp form; ``work_counter`` is an int64 CUDA tensor (>= 1 element)."""
    _check_rays_tensor(origin_tmax)
    n = origin_tmax.shape[0]
    _check_rays_tensor(direction, n)
    if out is None:
        out = alloc_hits(n, origin_tmax.device)
    rays = _Rays(origin_tmax.data_ptr(), direction.data_ptr())
    q = Query(compute_surface_properties, max_footprint, use_tmax, image_width).c()
    _check(_lib.cbq_intersect_persistent(dag.handle, ctypes.byref(rays), n, ctypes.byref(q),
                                         ctypes.byref(_hits_struct(out)), work_counter.data_ptr(), chunk,
                                         _stream_ptr(stream)), "cbq_intersect_persistent")
    return out


def scratch_for(n: int, device="cuda"):
    """Device scratch for intersect_auto / autotune over n rays (uint8 tensor)."""
    import torch
    return torch.empty(int(_lib.cbq_scratch_bytes(n)), dtype=torch.uint8, device=device)


def intersect_auto(dag: Dag, origin_tmax, direction, scratch, compute_surface_properties=True,
                   max_footprint=MAX_FOOTPRINT_DISABLED, use_tmax=False, out: dict | None = None, stream=None,
                   image_width: int = 0) -> dict:
    """Traverses with the form and launch shape in the DAG's launch config
    (plain, persistent or octant-sorted persistent), e.g. as set by autotune()."""
    _check_rays_tensor(origin_tmax)
    n = origin_tmax.shape[0]
    _check_rays_tensor(direction, n)
    if out is None:
        out = alloc_hits(n, origin_tmax.device)
    rays = _Rays(origin_tmax.data_ptr(), direction.data_ptr())
    q = Query(compute_surface_properties, max_footprint, use_tmax, image_width).c()
    _check(_lib.cbq_intersect_auto(dag.handle, ctypes.byref(rays), n, ctypes.byref(q), ctypes.byref(_hits_struct(out)),
                                   scratch.data_ptr(), scratch.numel(), _stream_ptr(stream)), "cbq_intersect_auto")
    return out


def autotune_launch(dag: Dag, origin_tmax, direction, scratch, out: dict, compute_surface_properties=True,
                    max_footprint=MAX_FOOTPRINT_DISABLED, use_tmax=False, repetitions: int = 3, stream=None,
                    image_width: int = 0):
    """Runs the native autotuner on these rays; returns (config dict, ms per launch)."""
    n = origin_tmax.shape[0]
    rays = _Rays(origin_tmax.data_ptr(), direction.data_ptr())
    q = Query(compute_surface_properties, max_footprint, use_tmax, image_width).c()
    best = LaunchConfig()
    ms = ctypes.c_float()
    _check(_lib.cbq_autotune(dag.handle, ctypes.byref(rays), n, ctypes.byref(q), ctypes.byref(_hits_struct(out)),
                             scratch.data_ptr(), scratch.numel(), repetitions, ctypes.byref(best), ctypes.byref(ms),
                             _stream_ptr(stream)), "cbq_autotune")
    return best.as_dict(), ms.value


def count_fetches(dag: Dag, origin_tmax, direction, compute_surface_properties=True,
                  max_footprint=MAX_FOOTPRINT_DISABLED, stream=None):
    import torch
    _check_rays_tensor(origin_tmax)
    n = origin_tmax.shape[0]
    _check_rays_tensor(direction, n)
    f = torch.empty(n, dtype=torch.int32, device=origin_tmax.device)
    rays = _Rays(origin_tmax.data_ptr(), direction.data_ptr())
    q = Query(compute_surface_properties, max_footprint, False).c()
    _check(_lib.cbq_count_fetches(dag.handle, ctypes.byref(rays), n, ctypes.byref(q), f.data_ptr(),
                                  _stream_ptr(stream)), "cbq_count_fetches")
    return f


def alloc_host_hits(n: int) -> dict:
    return {"hit": np.empty(n, np.uint8), "distance": np.empty(n, np.float32), "material": np.empty(n, np.uint32),
            "position": np.empty((n, 3), np.float32), "normal": np.empty((n, 3), np.float32),
            "voxel": np.empty((n, 3), np.int32), "status": np.empty(n, np.uint8)}


def intersect_volume_host(dag: Dag, origin_tmax: np.ndarray, direction: np.ndarray,
                          compute_surface_properties: bool = True, max_footprint: float = MAX_FOOTPRINT_DISABLED,
                          use_tmax: bool = False, out: dict | None = None, image_width: int = 0) -> dict:
    """Host-buffer form (cbq_intersect_host): copies in, traverses, copies out."""
    o = np.ascontiguousarray(origin_tmax, dtype=np.float32).reshape(-1, 4)
    d = np.ascontiguousarray(direction, dtype=np.float32).reshape(-1, 4)
    if o.shape != d.shape:
        raise ValueError("origin and direction arrays differ in length")
    n = o.shape[0]
    if out is None:
        out = alloc_host_hits(n)
    hits = _Hits(*[_np_ptr(out.get(k)) for k in HIT_FIELDS])
    q = Query(compute_surface_properties, max_footprint, use_tmax, image_width).c()
    _check(_lib.cbq_intersect_host(dag.handle, _np_ptr(o), _np_ptr(d), n, ctypes.byref(q), ctypes.byref(hits)),
           "cbq_intersect_host")
    return out


# ------------------------------------------------------------ serving

class _Request(ctypes.Structure):
    _fields_ = [("dag", ctypes.c_void_p), ("host_origin_tmax", ctypes.c_void_p), ("host_direction", ctypes.c_void_p),
                ("ray_count", ctypes.c_uint64), ("query", _Query), ("host_hits", _Hits)]


LAYOUT_REFERENCE = 0
LAYOUT_COMPACT = 1
SERVER_IN_PLACE = 0x1


class _ServerConfig(ctypes.Structure):
    _fields_ = [("device_memory_budget", ctypes.c_uint64), ("max_inflight_launches", ctypes.c_int32),
                ("max_batch_requests", ctypes.c_int32), ("max_batch_rays", ctypes.c_uint64),
                ("block", ctypes.c_int32), ("refill_min", ctypes.c_uint32), ("flags", ctypes.c_uint32)]


class _ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64), ("rays_completed", ctypes.c_uint64),
                ("launches", ctypes.c_uint64), ("queued", ctypes.c_uint64), ("inflight_launches", ctypes.c_uint64),
                ("mean_requests_per_launch", ctypes.c_double), ("latency_p50_us", ctypes.c_double),
                ("latency_p99_us", ctypes.c_double), ("latency_max_us", ctypes.c_double),
                ("latency_mean_us", ctypes.c_double), ("busy_seconds", ctypes.c_double),
                ("direct_requests", ctypes.c_uint64)]


_sig("cbq_server_create", [ctypes.POINTER(_ServerConfig), ctypes.POINTER(_P)])
_sig("cbq_server_submit", [_P, ctypes.POINTER(_Request), ctypes.POINTER(_U64)])
_sig("cbq_server_wait", [_P, _U64, ctypes.c_int64])
_sig("cbq_server_poll", [_P, _U64, ctypes.POINTER(ctypes.c_int32)])
_sig("cbq_server_cancel", [_P, _U64])
_sig("cbq_server_get_stats", [_P, ctypes.POINTER(_ServerStats)])
_sig("cbq_server_reset_stats", [_P])
_sig("cbq_server_destroy", [_P])


class _ReplayResult(ctypes.Structure):
    _fields_ = [("wall_seconds", ctypes.c_double), ("submitted", ctypes.c_uint64), ("failed", ctypes.c_uint64),
                ("backpressure", ctypes.c_uint64), ("lateness_p50_us", ctypes.c_double),
                ("lateness_p99_us", ctypes.c_double), ("lateness_max_us", ctypes.c_double),
                ("submit_p99_us", ctypes.c_double), ("submit_max_us", ctypes.c_double)]


_sig("cbq_server_replay", [_P, _P, _P, _U64, _U32, _P, ctypes.POINTER(_ReplayResult)])

# cbq_request as a numpy record, for building request traces without a Python
# loop per request (pointers as integers; 0 = NULL).
REQUEST_DTYPE = np.dtype([("dag", np.uint64), ("origin_tmax", np.uint64), ("direction", np.uint64),
                          ("ray_count", np.uint64), ("compute_surface", np.int32), ("max_footprint", np.float32),
                          ("flags", np.uint32), ("image_width", np.uint32)] +
                         [(k, np.uint64) for k in HIT_FIELDS])
assert REQUEST_DTYPE.itemsize == ctypes.sizeof(_Request)


class Server:
    """Continuous-batching request server over resident DAGs (cbq_server).

    submit() takes host numpy arrays and returns a ticket at once; the arrays
    are kept alive here until the ticket is waited for.  With in_place=True,
    requests whose arrays are all page-locked (e.g. from torch's pin_memory())
    are traversed in host memory without copies or device memory."""

    def __init__(self, device_memory_budget: int = 1 << 30, max_inflight_launches: int = 4,
                 max_batch_requests: int = 256, max_batch_rays: int = 4 << 20, block: int = 0, refill_min: int = 0,
                 in_place: bool = False):
        cfg = _ServerConfig(device_memory_budget, max_inflight_launches, max_batch_requests, max_batch_rays, block,
                            refill_min, SERVER_IN_PLACE if in_place else 0)
        h = _P()
        _check(_lib.cbq_server_create(ctypes.byref(cfg), ctypes.byref(h)), "cbq_server_create")
        self._h = h
        self._keep = {}

    def submit(self, dag: Dag, origin_tmax: np.ndarray, direction: np.ndarray, query: Query | None = None,
               out: dict | None = None):
        """Queues one request; returns (ticket, out) where `out` receives the hits."""
        o = np.ascontiguousarray(origin_tmax, dtype=np.float32).reshape(-1, 4)
        d = np.ascontiguousarray(direction, dtype=np.float32).reshape(-1, 4)
        n = o.shape[0]
        if out is None:
            out = alloc_host_hits(n)
        req = _Request(dag.handle, _np_ptr(o), _np_ptr(d), n, (query or Query()).c(),
                       _Hits(*[_np_ptr(out.get(k)) for k in HIT_FIELDS]))
        t = _U64()
        _check(_lib.cbq_server_submit(self._h, ctypes.byref(req), ctypes.byref(t)), "cbq_server_submit")
        self._keep[t.value] = (o, d, out, dag)
        return t.value, out

    def wait(self, ticket: int, timeout_us: int = -1) -> int:
        """Status of the request (0 = ok); raises CbqError on timeout or failure."""
        st = _lib.cbq_server_wait(self._h, ticket, timeout_us)
        if st != 5:  # not a timeout: the request is finished (or unknown)
            self._keep.pop(ticket, None)
        _check(st, "cbq_server_wait")
        return st

    def cancel(self, ticket: int) -> int:
        """Withdraws a request not yet launched; returns the status (0, 7 busy, 8 unknown)."""
        return _lib.cbq_server_cancel(self._h, ticket)

    def poll(self, ticket: int) -> bool:
        done = ctypes.c_int32()
        _check(_lib.cbq_server_poll(self._h, ticket, ctypes.byref(done)), "cbq_server_poll")
        return bool(done.value)

    def replay(self, requests: np.ndarray, arrival_s: np.ndarray, max_outstanding: int) -> dict:
        """Open-loop replay of a request trace from native threads
        (cbq_server_replay): requests[k] (a REQUEST_DTYPE record whose buffers
        the caller keeps alive) is submitted arrival_s[k] seconds after the
        start.  Returns the trace driver's result with per-request lateness (us)."""
        req = np.ascontiguousarray(requests, dtype=REQUEST_DTYPE)
        arr = np.ascontiguousarray(arrival_s, dtype=np.float64)
        if req.shape != arr.shape:
            raise ValueError("one arrival time per request")
        late = np.zeros(req.shape[0], np.float64)
        res = _ReplayResult()
        _check(_lib.cbq_server_replay(self._h, _np_ptr(req), _np_ptr(arr), req.shape[0], max_outstanding,
                                      _np_ptr(late), ctypes.byref(res)), "cbq_server_replay")
        out = {name: getattr(res, name) for name, _ in _ReplayResult._fields_}
        out["lateness_us"] = late
        return out

    def stats(self) -> dict:
        s = _ServerStats()
        _check(_lib.cbq_server_get_stats(self._h, ctypes.byref(s)), "cbq_server_get_stats")
        return {name: getattr(s, name) for name, _ in _ServerStats._fields_}

    def reset_stats(self) -> None:
        _check(_lib.cbq_server_reset_stats(self._h), "cbq_server_reset_stats")

    def close(self) -> None:
        if getattr(self, "_h", None) is not None:
            _lib.cbq_server_destroy(self._h)
            self._h = None
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------ pathtracer

class _PtMaterial(ctypes.Structure):
    _fields_ = [("albedo", ctypes.c_float * 3), ("emission", ctypes.c_float * 3)]


class _PtConfig(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int32), ("height", ctypes.c_int32), ("samples_per_pixel", ctypes.c_int32),
                ("bounces", ctypes.c_int32), ("eye", ctypes.c_double * 3), ("target", ctypes.c_double * 3),
                ("tan_half_fov", ctypes.c_double), ("max_footprint", ctypes.c_float),
                ("sun_direction", ctypes.c_float * 3), ("sun_colour", ctypes.c_float * 3),
                ("sky_colour", ctypes.c_float * 3), ("background", ctypes.c_float * 3), ("seed", ctypes.c_uint64),
                ("materials", ctypes.POINTER(_PtMaterial))]


class _PtStats(ctypes.Structure):
    _fields_ = [("extension_rays", ctypes.c_uint64), ("shadow_rays", ctypes.c_uint64),
                ("milliseconds", ctypes.c_double), ("kernel_launches", ctypes.c_uint64)]


PT_WAVE_FN = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p,
                              ctypes.c_void_p, ctypes.c_uint64, ctypes.POINTER(_Hits), ctypes.POINTER(_Query))
_sig("cbq_pathtrace", [_P, ctypes.POINTER(_PtConfig), _P, PT_WAVE_FN, _P, ctypes.POINTER(_PtStats), _P])
_sig("cbq_copy_to_host", [_P, _P, _U64])


def copy_to_host(device_ptr: int, shape, dtype) -> np.ndarray:
    """Copies a device buffer (a raw pointer) into a new numpy array."""
    out = np.empty(shape, dtype=dtype)
    _check(_lib.cbq_copy_to_host(_np_ptr(out), device_ptr, out.nbytes), "cbq_copy_to_host")
    return out


class WaveRecorder:
    """A pathtracer on_wave callback that copies every wave's rays and hits to
    the host: self.waves = [(kind, depth, sample, origin_tmax, direction, hits, query)]."""

    def __init__(self):
        self.waves = []

    def __call__(self, kind, depth, sample, o_ptr, d_ptr, n, hits, query):
        o = copy_to_host(o_ptr, (n, 4), np.float32)
        d = copy_to_host(d_ptr, (n, 4), np.float32)
        h = {"hit": copy_to_host(hits.hit, (n,), np.uint8)}
        if hits.material:
            h["material"] = copy_to_host(hits.material, (n,), np.uint32)
        if hits.position:
            h["position"] = copy_to_host(hits.position, (n, 3), np.float32)
        if hits.normal:
            h["normal"] = copy_to_host(hits.normal, (n, 3), np.float32)
        self.waves.append((kind, depth, sample, o, d, h,
                           (bool(query.compute_surface), float(query.max_footprint))))

# The reference demo's lighting (pathtracing_demo.cpp:84-104, :131): sun along
# normalize(1, -2, 10) with colour 0.1, sky colour 1.5, light-blue background.
SUN_DIRECTION = tuple(float(v) for v in np.array([1.0, -2.0, 10.0]) / np.linalg.norm([1.0, -2.0, 10.0]))


def pathtrace(dag: Dag, width: int, height: int, samples_per_pixel: int, bounces: int, eye, target,
              materials: np.ndarray, tan_half_fov: float = 0.57735026918962576, max_footprint: float = 0.0035,
              seed: int = 1, sun_direction=SUN_DIRECTION, sun_colour=(0.1, 0.1, 0.1), sky_colour=(1.5, 1.5, 1.5),
              background=(0.8, 0.8, 1.0), on_wave=None, stream=None):
    """Renders one frame; returns (image (height, width, 3) float32 CUDA tensor, stats dict).

    materials: (256, 2, 3) array of (albedo, emission) per material.
    on_wave(kind, depth, sample, origin_tmax_ptr, direction_ptr, n, hits, query) is called after
    every traversal wave with device pointers (kind 0 extension, 1 shadow)."""
    import torch
    mats = np.ascontiguousarray(materials, dtype=np.float32).reshape(256, 2, 3)
    arr = (_PtMaterial * 256)()
    for m in range(256):
        arr[m].albedo[:] = [float(v) for v in mats[m, 0]]
        arr[m].emission[:] = [float(v) for v in mats[m, 1]]
    cfg = _PtConfig(width, height, samples_per_pixel, bounces, (ctypes.c_double * 3)(*eye),
                    (ctypes.c_double * 3)(*target), tan_half_fov, max_footprint, (ctypes.c_float * 3)(*sun_direction),
                    (ctypes.c_float * 3)(*sun_colour), (ctypes.c_float * 3)(*sky_colour),
                    (ctypes.c_float * 3)(*background), seed, arr)
    image = torch.empty((height, width, 3), dtype=torch.float32, device="cuda")
    stats = _PtStats()
    cb = PT_WAVE_FN(lambda u, k, dp, s, o, d, n, h, q: on_wave(k, dp, s, o, d, n, h.contents, q.contents)) \
        if on_wave else PT_WAVE_FN()
    _check(_lib.cbq_pathtrace(dag.handle, ctypes.byref(cfg), image.data_ptr(), cb, None, ctypes.byref(stats),
                              _stream_ptr(stream)), "cbq_pathtrace")
    return image, {"extension_rays": stats.extension_rays, "shadow_rays": stats.shadow_rays,
                   "milliseconds": stats.milliseconds, "kernel_launches": stats.kernel_launches}


# ------------------------------------------------------------ batched form

class Batch:
    """Many volumes with their own ray batches in one persistent, graph-captured
    launch (cbq_batch).  `jobs` is a list of (Dag, origin_tmax, direction) with
    CUDA tensors; outputs are allocated per job (``self.outputs[i]``)."""

    def __init__(self, jobs, compute_surface_properties: bool = True,
                 max_footprint: float = MAX_FOOTPRINT_DISABLED, use_tmax: bool = False, outputs=None):
        self.jobs = list(jobs)
        self.outputs = outputs if outputs is not None else [alloc_hits(o.shape[0], o.device) for _, o, _ in self.jobs]
        arr = (_Job * max(1, len(self.jobs)))()
        for i, (dag, o, d) in enumerate(self.jobs):
            _check_rays_tensor(o)
            _check_rays_tensor(d, o.shape[0])
            arr[i].dag = dag.handle
            arr[i].rays = _Rays(o.data_ptr(), d.data_ptr())
            arr[i].ray_count = o.shape[0]
            arr[i].hits = _hits_struct(self.outputs[i])
        self._q = Query(compute_surface_properties, max_footprint, use_tmax).c()
        h = _P()
        _check(_lib.cbq_batch_create(arr, len(self.jobs), ctypes.byref(self._q), ctypes.byref(h)), "cbq_batch_create")
        self._h = h

    @property
    def total_rays(self) -> int:
        return self.config()["total_rays"]

    def config(self) -> dict:
        """The launch configuration (block, refill_min, steps, registers, stack,
        form) and the batch's ray count."""
        t = _U64()
        _check(_lib.cbq_batch_get_config(self._h, None, None, ctypes.byref(t)), "cbq_batch_get_config")
        c = _BatchConfig()
        _check(_lib.cbq_batch_get_launch_config(self._h, ctypes.byref(c)), "cbq_batch_get_launch_config")
        out = {name: getattr(c, name) for name, _ in _BatchConfig._fields_}
        out["total_rays"] = t.value
        return out

    def set_config(self, block: int = 0, refill_min: int = 0) -> None:
        _check(_lib.cbq_batch_set_config(self._h, block, refill_min), "cbq_batch_set_config")

    def set_launch_config(self, block: int = 128, refill_min: int = 8, steps: int = 8, registers: int = 0,
                          stack: int = STACK_LOCAL, form: int = FORM_PERSISTENT) -> None:
        c = _BatchConfig(block, refill_min, steps, registers, stack, form)
        _check(_lib.cbq_batch_set_launch_config(self._h, ctypes.byref(c)), "cbq_batch_set_launch_config")

    def autotune(self, repetitions: int = 3, stream=None) -> dict:
        _check(_lib.cbq_batch_autotune(self._h, _stream_ptr(stream), repetitions), "cbq_batch_autotune")
        return self.config()

    def launch(self, stream=None) -> None:
        """Replays the captured CUDA graph (captured on first use)."""
        _check(_lib.cbq_batch_launch(self._h, _stream_ptr(stream)), "cbq_batch_launch")

    def set_l2_persistence(self, dag: Dag | None, fraction: float) -> None:
        """Persisting L2 window over `dag`'s node store on the graph's kernel
        nodes (fraction of the device's persisting-L2 limit; 0 removes it)."""
        _check(_lib.cbq_batch_set_l2_persistence(self._h, dag.handle if dag is not None else None, fraction),
               "cbq_batch_set_l2_persistence")

    def launch_direct(self, stream=None) -> None:
        _check(_lib.cbq_batch_launch_direct(self._h, _stream_ptr(stream)), "cbq_batch_launch_direct")

    def destroy(self) -> None:
        if getattr(self, "_h", None) is not None:
            _lib.cbq_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass
