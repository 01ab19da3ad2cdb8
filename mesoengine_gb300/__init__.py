"""mesoengine_gb300 -- GB300-native voxel meshing and raymarching.

Python binding of the C ABI in include/meso.h (ctypes).  The compute path is
the CUDA library mesoengine_gb300/_lib/libmeso_gb300.so built for sm_103a;
there is no CPU fallback: loading fails loudly when the library is missing.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = _build.LIB

EMPTY_BRICK = 0xFFFFFFFF
SRC_GRID_U8, SRC_CHUNKS_U16, SRC_BRICKMAP, SRC_GRID_U16, SRC_CHUNKS_U8 = 0, 1, 2, 3, 4
RAY_SHADOW = 1
MAX_CHUNKS_PER_CALL = 1 << 20
REQ_RENDER, REQ_EDIT_REMESH_RENDER = 0, 1

STATUS = {
    0: "MESO_OK", 1: "MESO_ERR_INVALID_ARG", 2: "MESO_ERR_OOM", 3: "MESO_ERR_OVER_BUDGET",
    4: "MESO_ERR_OVERFLOW", 5: "MESO_ERR_TIMEOUT", 6: "MESO_ERR_CUDA", 7: "MESO_ERR_NOT_READY",
    8: "MESO_ERR_SHUTDOWN",
}

HIT_DTYPE = np.dtype(
    [("voxel", "<u8"), ("t", "<f4"), ("material", "<u2"), ("face", "u1"), ("shadow", "u1"),
     ("steps", "<u4"), ("shadow_steps", "<u4")]
)


class MesoError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


# ------------------------------------------------------------------ structs

class Config(ctypes.Structure):
    _fields_ = [
        ("chunk_edge", ctypes.c_uint32), ("brick_edge", ctypes.c_uint32), ("device", ctypes.c_int32),
        ("mesh_ctas_per_sm", ctypes.c_uint32), ("mesh_chunks_per_ticket", ctypes.c_uint32),
        ("ray_tile_w", ctypes.c_uint32), ("ray_tile_h", ctypes.c_uint32), ("ray_warps_per_cta", ctypes.c_uint32),
        ("hbm_budget_bytes", ctypes.c_uint64), ("tuning_path", ctypes.c_char_p),
    ]


class Terrain(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32), ("seed", ctypes.c_uint32),
        ("height_period", ctypes.c_uint32), ("height_octaves", ctypes.c_int32),
        ("height_base", ctypes.c_float), ("height_amp", ctypes.c_float),
        ("cave_period", ctypes.c_uint32), ("cave_threshold", ctypes.c_float),
    ]


class SceneInfo(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32),
        ("n_bricks", ctypes.c_uint64), ("brick_capacity", ctypes.c_uint64), ("device_bytes", ctypes.c_uint64),
        ("d_ptr", ctypes.c_void_p), ("d_occ", ctypes.c_void_p), ("d_mat", ctypes.c_void_p),
    ]


class MeshSource(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32), ("d_data", ctypes.c_void_p),
        ("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32), ("scene", ctypes.c_void_p),
    ]


class MeshOutput(ctypes.Structure):
    _fields_ = [
        ("d_quads", ctypes.c_void_p), ("capacity", ctypes.c_uint64), ("d_quad_count", ctypes.c_void_p),
        ("d_chunk_quad_counts", ctypes.c_void_p),
    ]


class MeshStoreInfo(ctypes.Structure):
    _fields_ = [
        ("n_chunks", ctypes.c_uint64), ("live_quads", ctypes.c_uint64), ("arena_quads", ctypes.c_uint64),
        ("arena_used", ctypes.c_uint64), ("compactions", ctypes.c_uint64), ("d_arena", ctypes.c_void_p),
        ("d_seg_offset", ctypes.c_void_p), ("d_seg_count", ctypes.c_void_p),
    ]


class Camera(ctypes.Structure):
    _fields_ = [
        ("origin_chunk", ctypes.c_int32 * 3), ("origin_frac", ctypes.c_float * 3),
        ("forward", ctypes.c_float * 3), ("right", ctypes.c_float * 3), ("up", ctypes.c_float * 3),
        ("tan_half_fov_y", ctypes.c_float), ("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
    ]


class SphereEdit(ctypes.Structure):
    _fields_ = [("center", ctypes.c_int32 * 3), ("radius", ctypes.c_int32), ("material", ctypes.c_uint16),
                ("pad", ctypes.c_uint16)]


class Request(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_uint32), ("scene_index", ctypes.c_uint32), ("camera", Camera), ("flags", ctypes.c_uint32),
        ("n_edits", ctypes.c_uint32), ("edits", ctypes.POINTER(SphereEdit)), ("user_tag", ctypes.c_uint64),
        ("dst_hits", ctypes.c_void_p),
    ]


class Completion(ctypes.Structure):
    _fields_ = [
        ("request_id", ctypes.c_uint64), ("user_tag", ctypes.c_uint64), ("status", ctypes.c_int32),
        ("n_dirty_chunks", ctypes.c_uint32), ("n_quads", ctypes.c_uint64), ("n_rays", ctypes.c_uint64),
        ("submit_s", ctypes.c_double), ("start_s", ctypes.c_double), ("done_s", ctypes.c_double),
        ("hit_checksum", ctypes.c_uint64), ("quad_checksum", ctypes.c_uint64),
    ]


class ServerConfig(ctypes.Structure):
    _fields_ = [
        ("max_inflight_batches", ctypes.c_uint32), ("max_batch_requests", ctypes.c_uint32),
        ("max_batch_rays", ctypes.c_uint64), ("hbm_budget_bytes", ctypes.c_uint64), ("keep_hits", ctypes.c_uint32),
        ("max_queue", ctypes.c_uint32), ("light", ctypes.c_float * 3), ("max_edit_quads", ctypes.c_uint64),
        ("keep_meshes", ctypes.c_uint32), ("reserved", ctypes.c_uint32),
    ]


VERTEX_DTYPE = np.dtype([("x", "<f4"), ("y", "<f4"), ("z", "<f4"), ("attr", "<u4")])

assert ctypes.sizeof(Camera) == 72
assert HIT_DTYPE.itemsize == 24

# ---------------------------------------------------------------- library

_lib = None

_SIGNATURES = {
    "meso_ctx_create": [ctypes.POINTER(Config), ctypes.POINTER(ctypes.c_void_p)],
    "meso_ctx_destroy": [ctypes.c_void_p],
    "meso_ctx_get_config": [ctypes.c_void_p, ctypes.POINTER(Config)],
    "meso_sync": [ctypes.c_void_p, ctypes.c_void_p],
    "meso_dev_alloc": [ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_void_p)],
    "meso_dev_free": [ctypes.c_void_p, ctypes.c_void_p],
    "meso_host_alloc_pinned": [ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_void_p)],
    "meso_host_free_pinned": [ctypes.c_void_p, ctypes.c_void_p],
    "meso_memcpy_h2d": [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p],
    "meso_memcpy_d2h": [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p],
    "meso_memset": [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t, ctypes.c_void_p],
    "meso_stream_create": [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)],
    "meso_stream_destroy": [ctypes.c_void_p, ctypes.c_void_p],
    "meso_event_create": [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)],
    "meso_event_destroy": [ctypes.c_void_p, ctypes.c_void_p],
    "meso_event_record": [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p],
    "meso_event_elapsed_ms": [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_float)],
    "meso_scene_create_terrain": [ctypes.c_void_p, ctypes.POINTER(Terrain), ctypes.c_uint64,
                                  ctypes.POINTER(ctypes.c_void_p)],
    "meso_scene_create_dense": [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                ctypes.c_uint64, ctypes.POINTER(ctypes.c_void_p)],
    "meso_scene_create_grid": [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                               ctypes.c_int32, ctypes.c_uint64, ctypes.POINTER(ctypes.c_void_p)],
    "meso_scene_count_solid": [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64)],
    "meso_scene_destroy": [ctypes.c_void_p, ctypes.c_void_p],
    "meso_mesh_store_create": [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)],
    "meso_mesh_store_update": [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32],
    "meso_mesh_store_get_info": [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(MeshStoreInfo)],
    "meso_mesh_store_gather": [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p,
                               ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64)],
    "meso_mesh_store_destroy": [ctypes.c_void_p, ctypes.c_void_p],
    "meso_scene_get_info": [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(SceneInfo)],
    "meso_scene_download": [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p],
    "meso_generate_dense_u8": [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_uint32,
                               ctypes.c_void_p, ctypes.c_void_p],
    "meso_generate_chunks_u16": [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_void_p,
                                 ctypes.c_void_p, ctypes.c_void_p],
    "meso_mesh_chunks": [ctypes.c_void_p, ctypes.POINTER(MeshSource), ctypes.c_void_p, ctypes.c_uint32,
                         ctypes.POINTER(MeshOutput), ctypes.c_void_p],
    "meso_mesh_chunks_per_launch": [ctypes.c_void_p, ctypes.POINTER(MeshSource), ctypes.c_void_p,
                                    ctypes.c_uint32, ctypes.POINTER(MeshOutput), ctypes.c_void_p],
    "meso_mesh_check": [ctypes.c_void_p, ctypes.POINTER(MeshOutput), ctypes.c_void_p,
                        ctypes.POINTER(ctypes.c_uint64)],
    "meso_mesh_host": [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                       ctypes.c_int32, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint64,
                       ctypes.POINTER(ctypes.c_uint64)],
    "meso_raymarch": [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(Camera), ctypes.c_uint32,
                      ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p],
    "meso_raymarch_per_view": [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(Camera),
                               ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p],
    "meso_raymarch_host": [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(Camera), ctypes.c_void_p,
                           ctypes.c_uint32, ctypes.c_void_p],
    "meso_raymarch_stats": [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(Camera),
                            ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p],
    "meso_edit_spheres": [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(SphereEdit), ctypes.c_uint32,
                          ctypes.c_void_p, ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint32), ctypes.c_void_p],
    "meso_server_create": [ctypes.c_void_p, ctypes.POINTER(ServerConfig), ctypes.POINTER(ctypes.c_void_p),
                           ctypes.c_uint32, ctypes.POINTER(ctypes.c_void_p)],
    "meso_server_submit": [ctypes.c_void_p, ctypes.POINTER(Request), ctypes.POINTER(ctypes.c_uint64)],
    "meso_server_poll": [ctypes.c_void_p, ctypes.POINTER(Completion), ctypes.c_uint32,
                         ctypes.POINTER(ctypes.c_uint32)],
    "meso_server_fetch_hits": [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_uint64],
    "meso_server_drain": [ctypes.c_void_p, ctypes.c_double],
    "meso_server_get_store": [ctypes.c_void_p, ctypes.c_uint32, ctypes.POINTER(ctypes.c_void_p)],
    "meso_server_destroy": [ctypes.c_void_p],
    "meso_autotune": [ctypes.c_void_p, ctypes.c_char_p],
    "meso_scene_save": [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char_p],
    "meso_scene_load": [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_uint64, ctypes.POINTER(ctypes.c_void_p)],
    "meso_quads_to_vertices": [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_uint32,
                               ctypes.c_void_p, ctypes.c_void_p],
    "meso_erode_mips": [ctypes.c_void_p, ctypes.POINTER(MeshSource), ctypes.c_void_p, ctypes.c_uint32,
                        ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p],
    "meso_capture_begin": [ctypes.c_void_p, ctypes.c_void_p],
    "meso_capture_end": [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)],
    "meso_graph_launch": [ctypes.c_void_p, ctypes.c_void_p],
    "meso_graph_destroy": [ctypes.c_void_p],
    "meso_selftest_bounded_wait": [ctypes.c_void_p, ctypes.c_uint32],
    "meso_measure_l2_read": [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32, ctypes.POINTER(ctypes.c_double)],
    "meso_raymarch_noalloc": [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(Camera),
                              ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p],
}


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Loads libmeso_gb300.so (building it in-tree first if needed)."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_missing:
        _build.build()
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"mesoengine_gb300: CUDA library missing at {LIB_PATH}")
    L = ctypes.CDLL(LIB_PATH)
    for name, args in _SIGNATURES.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    L.meso_last_error_string.restype = ctypes.c_char_p
    L.meso_last_error_string.argtypes = []
    L.meso_status_string.restype = ctypes.c_char_p
    L.meso_status_string.argtypes = [ctypes.c_int]
    L.meso_kernel_launches.restype = ctypes.c_uint64
    L.meso_kernel_launches.argtypes = [ctypes.c_void_p]
    L.meso_sm_count.restype = ctypes.c_int
    L.meso_sm_count.argtypes = [ctypes.c_void_p]
    L.meso_server_now.restype = ctypes.c_double
    L.meso_server_now.argtypes = [ctypes.c_void_p]
    _lib = L
    return L


def _check(rc: int) -> None:
    if rc != 0:
        raise MesoError(rc, (_lib.meso_last_error_string() or b"").decode())


def _np_ptr(a: np.ndarray) -> ctypes.c_void_p:
    return ctypes.c_void_p(a.ctypes.data)


# ---------------------------------------------------------------- objects

class DeviceBuffer:
    """Device allocation owned by a Context."""

    def __init__(self, ctx: "Context", nbytes: int):
        self.ctx = ctx
        self.nbytes = int(nbytes)
        p = ctypes.c_void_p()
        _check(_lib.meso_dev_alloc(ctx.handle, max(16, self.nbytes), ctypes.byref(p)))
        self.ptr = p.value

    def upload(self, arr: np.ndarray, stream=None) -> "DeviceBuffer":
        a = np.ascontiguousarray(arr)
        assert a.nbytes <= self.nbytes
        _check(_lib.meso_memcpy_h2d(self.ctx.handle, self.ptr, _np_ptr(a), a.nbytes, stream))
        _check(_lib.meso_sync(self.ctx.handle, stream))
        return self

    def download(self, dtype, count=None, stream=None) -> np.ndarray:
        dt = np.dtype(dtype)
        n = self.nbytes // dt.itemsize if count is None else int(count)
        out = np.empty(n, dtype=dt)
        if n:
            _check(_lib.meso_memcpy_d2h(self.ctx.handle, _np_ptr(out), self.ptr, n * dt.itemsize, stream))
        _check(_lib.meso_sync(self.ctx.handle, stream))
        return out

    def zero(self, stream=None) -> None:
        _check(_lib.meso_memset(self.ctx.handle, self.ptr, 0, self.nbytes, stream))

    def free(self) -> None:
        if self.ptr and _lib is not None:
            _lib.meso_dev_free(self.ctx.handle, self.ptr)
        self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class PinnedBuffer:
    """Page-locked host allocation owned by a Context."""

    def __init__(self, ctx: "Context", nbytes: int):
        self.ctx = ctx
        self.nbytes = int(nbytes)
        p = ctypes.c_void_p()
        _check(_lib.meso_host_alloc_pinned(ctx.handle, max(16, self.nbytes), ctypes.byref(p)))
        self.ptr = p.value

    def view(self, dtype, count=None) -> np.ndarray:
        dt = np.dtype(dtype)
        n = self.nbytes // dt.itemsize if count is None else int(count)
        buf = (ctypes.c_uint8 * (n * dt.itemsize)).from_address(self.ptr)
        return np.frombuffer(buf, dtype=dt, count=n)

    def free(self) -> None:
        if self.ptr and _lib is not None:
            _lib.meso_host_free_pinned(self.ctx.handle, self.ptr)
        self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Scene:
    def __init__(self, ctx: "Context", handle: int):
        self.ctx = ctx
        self.handle = handle

    def info(self) -> SceneInfo:
        i = SceneInfo()
        _check(_lib.meso_scene_get_info(self.ctx.handle, self.handle, ctypes.byref(i)))
        return i

    @property
    def dims(self):
        i = self.info()
        return (i.nx, i.ny, i.nz)

    def count_solid(self) -> int:
        """Solid voxels of the scene (counted on the device)."""
        n = ctypes.c_uint64()
        _check(_lib.meso_scene_count_solid(self.ctx.handle, self.handle, ctypes.byref(n)))
        return int(n.value)

    def download(self):
        """(ptr, occ[cap,8], mat[cap,512]) host copies."""
        i = self.info()
        nb = (i.nx // 8) * (i.ny // 8) * (i.nz // 8)
        ptr = np.empty(nb, dtype=np.uint32)
        occ = np.empty((max(1, i.brick_capacity), 8), dtype=np.uint64)
        mat = np.empty((max(1, i.brick_capacity), 512), dtype=np.uint16)
        _check(_lib.meso_scene_download(self.ctx.handle, self.handle, _np_ptr(ptr), _np_ptr(occ), _np_ptr(mat)))
        return ptr, occ[: i.brick_capacity], mat[: i.brick_capacity]

    def dense(self) -> np.ndarray:
        """Dense uint16 copy (small scenes only)."""
        nx, ny, nz = self.dims
        ptr, _, mat = self.download()
        out = np.zeros((nz // 8, 8, ny // 8, 8, nx // 8, 8), dtype=np.uint16)
        p = ptr.reshape(nz // 8, ny // 8, nx // 8)
        idx = np.nonzero(p != EMPTY_BRICK)
        for bz, by, bx in zip(*idx):
            out[bz, :, by, :, bx, :] = mat[p[bz, by, bx]].reshape(8, 8, 8)
        return out.reshape(nz, ny, nx)

    def save(self, path: str) -> None:
        _check(_lib.meso_scene_save(self.ctx.handle, self.handle, path.encode()))

    def edit(self, spheres, stream=None) -> np.ndarray:
        arr = (SphereEdit * max(1, len(spheres)))(*spheres)
        nx, ny, nz = self.dims
        cap = (nx // 32) * (ny // 32) * (nz // 32)
        dirty = np.empty(max(1, cap), dtype=np.uint32)  # the library writes the first n entries
        n = ctypes.c_uint32()
        _check(_lib.meso_edit_spheres(self.ctx.handle, self.handle, arr, len(spheres), _np_ptr(dirty), cap,
                                      ctypes.byref(n), stream))
        _check(_lib.meso_sync(self.ctx.handle, stream))
        return dirty[: n.value].copy()

    def destroy(self) -> None:
        if self.handle and _lib is not None:
            _lib.meso_scene_destroy(self.ctx.handle, self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class MeshStore:
    """The resident per-chunk mesh of a brick-map scene (meso_mesh_store)."""

    def __init__(self, ctx: "Context", scene: "Scene", handle=None):
        self.ctx = ctx
        self.scene = scene  # the store reads the scene: keep it alive
        self.owned = handle is None
        if handle is None:
            h = ctypes.c_void_p()
            _check(_lib.meso_mesh_store_create(ctx.handle, scene.handle, ctypes.byref(h)))
            handle = h.value
        self.handle = handle

    @classmethod
    def borrowed(cls, ctx: "Context", scene: "Scene", handle: int) -> "MeshStore":
        return cls(ctx, scene, handle)

    def update(self, chunks) -> None:
        c = np.ascontiguousarray(chunks, dtype=np.uint32)
        _check(_lib.meso_mesh_store_update(self.ctx.handle, self.handle, _np_ptr(c), c.size))

    def info(self) -> MeshStoreInfo:
        i = MeshStoreInfo()
        _check(_lib.meso_mesh_store_get_info(self.ctx.handle, self.handle, ctypes.byref(i)))
        return i

    def gather(self, chunks) -> np.ndarray:
        """Quads of the listed chunks in list order (chunk field = position in the list)."""
        c = np.ascontiguousarray(chunks, dtype=np.uint32)
        total = ctypes.c_uint64()
        # a size query: with capacity 0 the call reports the total (and
        # MESO_ERR_OVERFLOW when it is not zero)
        rc = _lib.meso_mesh_store_gather(self.ctx.handle, self.handle, _np_ptr(c), c.size, None, 0,
                                         ctypes.byref(total))
        if rc not in (0, 4):
            _check(rc)
        n = int(total.value)
        out = self.ctx.alloc(max(8, n * 8))
        _check(_lib.meso_mesh_store_gather(self.ctx.handle, self.handle, _np_ptr(c), c.size, out.ptr, n,
                                           ctypes.byref(total)))
        return out.download(np.uint64, n)

    def destroy(self) -> None:
        if self.handle and self.owned:
            _lib.meso_mesh_store_destroy(self.ctx.handle, self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class Context:
    """A device context: owns a stream and the device error flag."""

    def __init__(self, device: int = 0, tuning_path: str | None = None, **cfg):
        load()
        c = Config()
        c.device = device
        for k, v in cfg.items():
            setattr(c, k, v)
        self._tp = tuning_path.encode() if tuning_path else None
        c.tuning_path = self._tp
        h = ctypes.c_void_p()
        _check(_lib.meso_ctx_create(ctypes.byref(c), ctypes.byref(h)))
        self.handle = h.value

    # -- memory
    def alloc(self, nbytes: int) -> DeviceBuffer:
        return DeviceBuffer(self, nbytes)

    def to_device(self, arr: np.ndarray) -> DeviceBuffer:
        a = np.ascontiguousarray(arr)
        return DeviceBuffer(self, a.nbytes).upload(a)

    def sync(self, stream=None) -> None:
        _check(_lib.meso_sync(self.handle, stream))

    def stream(self):
        s = ctypes.c_void_p()
        _check(_lib.meso_stream_create(self.handle, ctypes.byref(s)))
        return s.value

    def event(self):
        e = ctypes.c_void_p()
        _check(_lib.meso_event_create(self.handle, ctypes.byref(e)))
        return e.value

    def record(self, ev, stream=None) -> None:
        _check(_lib.meso_event_record(self.handle, ev, stream))

    def elapsed_ms(self, a, b) -> float:
        ms = ctypes.c_float()
        _check(_lib.meso_event_elapsed_ms(self.handle, a, b, ctypes.byref(ms)))
        return float(ms.value)

    @property
    def kernel_launches(self) -> int:
        return int(_lib.meso_kernel_launches(self.handle))

    @property
    def sm_count(self) -> int:
        return int(_lib.meso_sm_count(self.handle))

    # -- scenes
    def scene_from_terrain(self, terrain: Terrain, spare_bricks: int = 0) -> Scene:
        h = ctypes.c_void_p()
        _check(_lib.meso_scene_create_terrain(self.handle, ctypes.byref(terrain), spare_bricks, ctypes.byref(h)))
        return Scene(self, h.value)

    def scene_from_dense(self, grid: np.ndarray, spare_bricks: int = 0) -> Scene:
        g = np.ascontiguousarray(grid, dtype=np.uint16)
        nz, ny, nx = g.shape
        h = ctypes.c_void_p()
        _check(_lib.meso_scene_create_dense(self.handle, _np_ptr(g), nx, ny, nz, spare_bricks, ctypes.byref(h)))
        return Scene(self, h.value)

    def scene_from_grid(self, kind: int, grid: "DeviceBuffer", dims, spare_bricks: int = 0) -> Scene:
        """Brick map of a dense device grid (SRC_GRID_U8 or SRC_GRID_U16), dims (nx, ny, nz)."""
        nx, ny, nz = dims
        h = ctypes.c_void_p()
        _check(_lib.meso_scene_create_grid(self.handle, kind, grid.ptr, nx, ny, nz, spare_bricks, ctypes.byref(h)))
        return Scene(self, h.value)

    # -- generators
    def generate_dense_u8(self, nx, ny, nz, seed=1, stream=None) -> DeviceBuffer:
        b = self.alloc(nx * ny * nz)
        _check(_lib.meso_generate_dense_u8(self.handle, nx, ny, nz, seed, b.ptr, stream))
        self.sync(stream)
        return b

    def generate_chunks_u16(self, n, seed0=1, stream=None):
        b = self.alloc(n * 65536)
        s = self.alloc(n * 4)
        _check(_lib.meso_generate_chunks_u16(self.handle, n, seed0, b.ptr, s.ptr, stream))
        self.sync(stream)
        return b, s

    # -- meshing
    def mesh(self, kind, data=None, coords=None, n=None, dims=(0, 0, 0), scene: Scene | None = None,
             capacity=None, per_launch=False, chunk_counts=False, stream=None, check=True):
        """Meshes chunks on the device; returns (quads uint64 array, per-chunk counts or None)."""
        src = MeshSource()
        src.kind = kind
        src.d_data = data.ptr if isinstance(data, DeviceBuffer) else None
        src.nx, src.ny, src.nz = dims
        src.scene = scene.handle if scene is not None else None
        coord_buf = None
        if coords is not None and kind in (SRC_CHUNKS_U16, SRC_CHUNKS_U8) and isinstance(data, DeviceBuffer):
            src.nx = data.nbytes // (65536 if kind == SRC_CHUNKS_U16 else 32768)
        if coords is not None:
            c = np.ascontiguousarray(coords, dtype=np.int32)
            coord_buf = self.to_device(c)
            n = c.shape[0] if n is None else n
        if capacity is None:  # worst case is a checkerboard: 6 * 16384 quads per chunk
            capacity = max(1024, n * (98304 if n <= 512 else 16384))
        qbuf = self.alloc(capacity * 8)
        cnt = self.alloc(8)
        ccnt = self.alloc(max(1, n) * 4) if chunk_counts else None
        out = MeshOutput(qbuf.ptr, capacity, cnt.ptr, ccnt.ptr if ccnt else None)
        fn = _lib.meso_mesh_chunks_per_launch if per_launch else _lib.meso_mesh_chunks
        _check(fn(self.handle, ctypes.byref(src), coord_buf.ptr if coord_buf else None, n, ctypes.byref(out),
                  stream))
        total = ctypes.c_uint64()
        rc = _lib.meso_mesh_check(self.handle, ctypes.byref(out), stream, ctypes.byref(total))
        if check:
            _check(rc)
        k = min(total.value, capacity)
        quads = qbuf.download(np.uint64, k)
        counts = ccnt.download(np.uint32, n) if ccnt else None
        return quads, counts

    def mesh_host(self, kind, data: np.ndarray, coords=None, dims=(0, 0, 0), capacity=None):
        d = np.ascontiguousarray(data)
        if kind in (SRC_CHUNKS_U16, SRC_CHUNKS_U8):
            n = d.shape[0] if coords is None else len(coords)
            dims = (d.shape[0], 0, 0)
        else:
            n = len(coords)
        c = None if coords is None else np.ascontiguousarray(coords, dtype=np.int32)
        capacity = max(1024, n * (98304 if n <= 512 else 16384)) if capacity is None else capacity
        out = np.empty(capacity, dtype=np.uint64)
        total = ctypes.c_uint64()
        _check(_lib.meso_mesh_host(self.handle, kind, _np_ptr(d), dims[0], dims[1], dims[2],
                                   _np_ptr(c) if c is not None else None, n, _np_ptr(out), capacity,
                                   ctypes.byref(total)))
        return out[: total.value]

    # -- raymarching
    def raymarch(self, scenes, cams, light=None, shadow=True, per_view=False, stream=None,
                 out: DeviceBuffer | None = None, download=True):
        scenes = scenes if isinstance(scenes, (list, tuple)) else [scenes]
        cams = cams if isinstance(cams, (list, tuple)) else [cams]
        if len(scenes) == 1 and len(cams) > 1:
            scenes = scenes * len(cams)
        sh = (ctypes.c_void_p * len(scenes))(*[s.handle for s in scenes])
        ca = (Camera * len(cams))(*cams)
        total = sum(c.width * c.height for c in cams)
        if out is None:
            out = self.alloc(total * 24)
        L = _light_arg(light)
        fn = _lib.meso_raymarch_per_view if per_view else _lib.meso_raymarch
        _check(fn(self.handle, sh, ca, len(cams), _np_ptr(L), RAY_SHADOW if shadow else 0, out.ptr, stream))
        if not download:
            return out
        self.sync(stream)
        return out.download(HIT_DTYPE, total)

    def raymarch_host(self, scene: Scene, cam: Camera, light=None, shadow=True, out_ptr=None) -> np.ndarray:
        """Host-buffer entry point; out_ptr (e.g. a PinnedBuffer.ptr) receives the hits."""
        L = _light_arg(light)
        hits = None
        if out_ptr is None:
            hits = np.empty(cam.width * cam.height, dtype=HIT_DTYPE)
            out_ptr = hits.ctypes.data
        _check(_lib.meso_raymarch_host(self.handle, scene.handle, ctypes.byref(cam), _np_ptr(L),
                                       RAY_SHADOW if shadow else 0, ctypes.c_void_p(out_ptr)))
        return hits

    def raymarch_stats(self, scenes, cams, light=None, shadow=True, out: DeviceBuffer | None = None):
        """(pointer fetches, occupied bricks entered, hits, rays) of one launch."""
        scenes = scenes if isinstance(scenes, (list, tuple)) else [scenes]
        cams = cams if isinstance(cams, (list, tuple)) else [cams]
        if len(scenes) == 1 and len(cams) > 1:
            scenes = scenes * len(cams)
        sh = (ctypes.c_void_p * len(scenes))(*[s.handle for s in scenes])
        ca = (Camera * len(cams))(*cams)
        total = sum(c.width * c.height for c in cams)
        if out is None:
            out = self.alloc(total * 24)
        L = _light_arg(light)
        counts = np.zeros(4, dtype=np.uint64)
        _check(_lib.meso_raymarch_stats(self.handle, sh, ca, len(cams), _np_ptr(L), RAY_SHADOW if shadow else 0,
                                        out.ptr, _np_ptr(counts)))
        return [int(v) for v in counts]

    def pinned(self, nbytes: int) -> PinnedBuffer:
        return PinnedBuffer(self, nbytes)

    def capture(self, fn, stream):
        """Captures the stream-ordered calls fn() issues on `stream` into a
        CUDA graph; returns a Graph whose launch() replays them."""
        _check(_lib.meso_capture_begin(self.handle, stream))
        try:
            fn()
        finally:
            g = ctypes.c_void_p()
            rc = _lib.meso_capture_end(self.handle, stream, ctypes.byref(g))
        _check(rc)
        return Graph(g.value)

    def scene_load(self, path: str, spare_bricks: int = 0) -> Scene:
        h = ctypes.c_void_p()
        _check(_lib.meso_scene_load(self.handle, path.encode(), spare_bricks, ctypes.byref(h)))
        return Scene(self, h.value)

    def quads_to_vertices(self, quads: np.ndarray, chunk_origins: np.ndarray) -> np.ndarray:
        """Returns VERTEX_DTYPE records, 4 per quad."""
        q = np.ascontiguousarray(quads, dtype=np.uint64)
        org = np.ascontiguousarray(chunk_origins, dtype=np.int32).reshape(-1, 3)
        dq, do = self.to_device(q if q.size else np.zeros(1, np.uint64)), self.to_device(org)
        out = self.alloc(max(1, q.size) * 64)
        _check(_lib.meso_quads_to_vertices(self.handle, dq.ptr, q.size, do.ptr, org.shape[0], out.ptr, None))
        self.sync()
        return out.download(VERTEX_DTYPE, 4 * q.size)

    def erode_mips(self, kind, data=None, coords=None, n=None, dims=(0, 0, 0), scene=None, depth=4) -> np.ndarray:
        """Erosion pyramid: uint32 words [n][depth][z][y] (bit x)."""
        src = MeshSource()
        src.kind = kind
        src.d_data = data.ptr if isinstance(data, DeviceBuffer) else None
        src.nx, src.ny, src.nz = dims
        src.scene = scene.handle if scene is not None else None
        cb = None
        if coords is not None:
            c = np.ascontiguousarray(coords, dtype=np.int32)
            cb = self.to_device(c)
            n = c.shape[0]
            if kind in (SRC_CHUNKS_U16, SRC_CHUNKS_U8) and isinstance(data, DeviceBuffer):
                src.nx = data.nbytes // (65536 if kind == SRC_CHUNKS_U16 else 32768)
        out = self.alloc(n * depth * 4096)
        _check(_lib.meso_erode_mips(self.handle, ctypes.byref(src), cb.ptr if cb else None, n, depth, out.ptr, None))
        self.sync()
        return out.download(np.uint32, n * depth * 1024).reshape(n, depth, 32, 32)

    def selftest_bounded_wait(self, limit_us: int) -> None:
        """Runs a device wait that must give up after limit_us; raises
        MesoError(MESO_ERR_TIMEOUT) when the failure path works."""
        _check(_lib.meso_selftest_bounded_wait(self.handle, limit_us))

    def measure_l2_read(self, nbytes: int = 32 << 20, passes: int = 50) -> float:
        """L2 read bandwidth in GB/s (an L2-resident buffer read `passes` times)."""
        g = ctypes.c_double()
        _check(_lib.meso_measure_l2_read(self.handle, nbytes, passes, ctypes.byref(g)))
        return g.value

    def mesh_store(self, scene: Scene) -> MeshStore:
        return MeshStore(self, scene)

    def autotune(self, path: str | None = None) -> None:
        _check(_lib.meso_autotune(self.handle, path.encode() if path else None))

    def config(self) -> dict:
        """The effective launch configuration (defaults, tuning file and autotuning applied)."""
        c = Config()
        _check(_lib.meso_ctx_get_config(self.handle, ctypes.byref(c)))
        return {k: getattr(c, k) for k in ("device", "mesh_ctas_per_sm", "mesh_chunks_per_ticket", "ray_tile_w",
                                            "ray_tile_h", "ray_warps_per_cta", "hbm_budget_bytes")}

    def close(self) -> None:
        if getattr(self, "handle", None) and _lib is not None:
            _lib.meso_ctx_destroy(self.handle)
        self.handle = None


class Graph:
    def __init__(self, handle):
        self.handle = handle

    def launch(self, stream=None) -> None:
        _check(_lib.meso_graph_launch(self.handle, stream))

    def destroy(self) -> None:
        if self.handle and _lib is not None:
            _lib.meso_graph_destroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


# ---------------------------------------------------------------- helpers

def light_dir(v=(0.3, 0.5, 0.8)) -> np.ndarray:
    a = np.asarray(v, dtype=np.float64)
    return (a / np.linalg.norm(a)).astype(np.float32)


_DEFAULT_LIGHT = None


def _light_arg(light):
    """The light direction as a float32 array (the default one built once)."""
    global _DEFAULT_LIGHT
    if light is None:
        if _DEFAULT_LIGHT is None:
            _DEFAULT_LIGHT = light_dir()
            _DEFAULT_LIGHT.setflags(write=False)
        return _DEFAULT_LIGHT
    return np.asarray(light, dtype=np.float32)


def camera(origin, target, width, height, fov_y_deg=60.0, up=(0.0, 0.0, 1.0)) -> Camera:
    """Pinhole camera at origin looking at target, z-up, rebased on its 32^3 chunk."""
    o = np.asarray(origin, dtype=np.float64)
    f = np.asarray(target, dtype=np.float64) - o
    f /= np.linalg.norm(f)
    r = np.cross(f, np.asarray(up, dtype=np.float64))
    if np.linalg.norm(r) < 1e-9:
        r = np.cross(f, np.array([0.0, 1.0, 0.0]))
    r /= np.linalg.norm(r)
    u = np.cross(r, f)
    ch = np.floor(o / 32.0).astype(np.int64)
    frac = o - ch * 32.0
    c = Camera()
    c.origin_chunk[:] = [int(v) for v in ch]
    c.origin_frac[:] = [float(v) for v in frac]
    c.forward[:] = [float(v) for v in f]
    c.right[:] = [float(v) for v in r]
    c.up[:] = [float(v) for v in u]
    c.tan_half_fov_y = float(np.tan(np.radians(fov_y_deg) / 2.0))
    c.width, c.height = int(width), int(height)
    return c


def terrain_preset(name: str, seed: int | None = None) -> Terrain:
    """Seeded terrain scenes: 'small' (128^3 test scene), 'scene1024' (the
    1024^3 raymarch scene, ~15% solid), 'serve512'/'serve1024'/'serve2048'
    (the served scenes, same recipe scaled), 'edit4096' (4096^3, ~2% solid)."""
    presets = {
        "small": (128, 2, 64, 32.0, 7.0),
        "scene1024": (1024, 2, 512, 256.0, 56.0),
        "serve512": (512, 11, 256, 128.0, 28.0),
        "serve1024": (1024, 12, 512, 256.0, 56.0),
        "serve1024b": (1024, 13, 512, 256.0, 56.0),
        "serve2048": (2048, 14, 1024, 512.0, 112.0),
        "edit4096": (4096, 9, 2048, 128.0, 16.0),
    }
    n, s, period, amp, base = presets[name]
    return Terrain(n, n, n, s if seed is None else seed, period, 6, base, amp, 48, 0.7)


# ---------------------------------------------------------------- serving

def hit_checksum(hits: np.ndarray) -> int:
    """Host restatement of the server's order-sensitive hit hash:
    sum_i mix64(w0 ^ mix64(w1 ^ mix64(w2 ^ (i*0x9E3779B97F4A7C15 + 1)))) mod 2^64,
    w0..w2 the three 64-bit words of hit i, mix64 the splitmix64 finaliser."""
    w = np.ascontiguousarray(hits).view(np.uint64).reshape(-1, 3)
    i = np.arange(w.shape[0], dtype=np.uint64)
    with np.errstate(over="ignore"):
        k = i * np.uint64(0x9E3779B97F4A7C15) + np.uint64(1)
        h = _mix64(w[:, 0] ^ _mix64(w[:, 1] ^ _mix64(w[:, 2] ^ k)))
        return int(np.sum(h, dtype=np.uint64))


def quad_checksum(quads: np.ndarray) -> int:
    """Order-insensitive quad hash: sum of mix64(q) mod 2^64."""
    with np.errstate(over="ignore"):
        return int(np.sum(_mix64(np.asarray(quads, dtype=np.uint64)), dtype=np.uint64))


def _mix64(x):
    x = np.asarray(x, dtype=np.uint64)
    with np.errstate(over="ignore"):
        x = x ^ (x >> np.uint64(30))
        x = x * np.uint64(0xBF58476D1CE4E5B9)
        x = x ^ (x >> np.uint64(27))
        x = x * np.uint64(0x94D049BB133111EB)
        x = x ^ (x >> np.uint64(31))
    return x


class Server:
    """Continuous-batching request server over resident scenes."""

    def __init__(self, ctx: Context, scenes, **cfg):
        self.ctx = ctx
        self.scenes = list(scenes)
        c = ServerConfig()
        for k, v in cfg.items():
            if k == "light":
                c.light[:] = list(v)
            else:
                setattr(c, k, v)
        arr = (ctypes.c_void_p * len(self.scenes))(*[s.handle for s in self.scenes])
        h = ctypes.c_void_p()
        _check(_lib.meso_server_create(ctx.handle, ctypes.byref(c), arr, len(self.scenes), ctypes.byref(h)))
        self.handle = h.value
        self._keep = {}

    def submit(self, scene_index: int, camera: Camera, shadow=False, edits=None, tag=0, dst=None) -> int:
        """dst: optional DeviceBuffer / PinnedBuffer (or raw pointer) that receives the request's hits."""
        r = Request()
        if dst is not None:
            r.dst_hits = dst if isinstance(dst, int) else dst.ptr
        r.kind = REQ_EDIT_REMESH_RENDER if edits is not None else REQ_RENDER
        r.scene_index = scene_index
        r.camera = camera
        r.flags = RAY_SHADOW if shadow else 0
        arr = None
        if edits:
            arr = (SphereEdit * len(edits))(*edits)
            r.n_edits = len(edits)
            r.edits = ctypes.cast(arr, ctypes.POINTER(SphereEdit))
        r.user_tag = tag
        rid = ctypes.c_uint64()
        _check(_lib.meso_server_submit(self.handle, ctypes.byref(r), ctypes.byref(rid)))
        return int(rid.value)

    def store(self, scene_index: int) -> "MeshStore":
        """The mesh store the server keeps for a scene (keep_meshes=1); owned by the server."""
        h = ctypes.c_void_p()
        _check(_lib.meso_server_get_store(self.handle, scene_index, ctypes.byref(h)))
        return MeshStore.borrowed(self.ctx, self.scenes[scene_index], h.value)

    def poll(self, max_n: int = 4096):
        buf = (Completion * max_n)()
        n = ctypes.c_uint32()
        _check(_lib.meso_server_poll(self.handle, buf, max_n, ctypes.byref(n)))
        return [buf[i] for i in range(n.value)]

    def drain(self, timeout_s: float = 60.0) -> None:
        _check(_lib.meso_server_drain(self.handle, timeout_s))

    def now(self) -> float:
        return float(_lib.meso_server_now(self.handle))

    def fetch_hits(self, request_id: int, n: int) -> np.ndarray:
        out = np.empty(n, dtype=HIT_DTYPE)
        _check(_lib.meso_server_fetch_hits(self.handle, request_id, _np_ptr(out), n))
        return out

    def close(self) -> None:
        if getattr(self, "handle", None) and _lib is not None:
            _lib.meso_server_destroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
