"""CPU oracle for the voxel meshing and raymarching hot paths (ctypes binding).

TEST INFRASTRUCTURE ONLY: the correctness checker and the timed CPU baseline.
Only the tests, the smoke check and the benchmark's CPU-baseline leg import
this package; the product library never does.

Parity status: unpinned by the reference, which implements neither greedy
meshing nor raymarching (it emits one imposter cube per surviving block,
Runtimes/Voxel/Chunk/ChunkPool.h:381-445).  The algorithms are clean-room
restatements of Lysenko 2012 (greedy meshing) and Amanatides & Woo 1987
(voxel traversal) on the reference's data conventions; see meso_oracle.h.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_LIB_PATH = os.path.join(_BUILD, "libmeso_oracle.so")
_SRC = os.path.join(_HERE, "meso_oracle.c")
_HDR = os.path.join(_HERE, "meso_oracle.h")

EMPTY_BRICK = 0xFFFFFFFF
SRC_GRID_U8, SRC_CHUNKS_U16, SRC_BRICKMAP, SRC_GRID_U16, SRC_CHUNKS_U8 = 0, 1, 2, 3, 4

HIT_DTYPE = np.dtype(
    [
        ("voxel", "<u8"),
        ("t", "<f4"),
        ("material", "<u2"),
        ("face", "u1"),
        ("shadow", "u1"),
        ("steps", "<u4"),
        ("shadow_steps", "<u4"),
    ]
)
assert HIT_DTYPE.itemsize == 24


def build(force: bool = False) -> str:
    """Compiles the oracle with gcc (FP contraction off) into oracle/_build."""
    os.makedirs(_BUILD, exist_ok=True)
    if (
        not force
        and os.path.exists(_LIB_PATH)
        and os.path.getmtime(_LIB_PATH) >= max(os.path.getmtime(_SRC), os.path.getmtime(_HDR))
    ):
        return _LIB_PATH
    tmp = _LIB_PATH + f".{os.getpid()}.tmp"
    cmd = [
        "gcc", "-O2", "-std=gnu11", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
        "-pthread", "-Wall", "-Wno-unused-function", "-o", tmp, _SRC, "-lm",
    ]
    subprocess.run(cmd, check=True)
    os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


class Terrain(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32),
        ("seed", ctypes.c_uint32),
        ("height_period", ctypes.c_uint32),
        ("height_octaves", ctypes.c_int32),
        ("height_base", ctypes.c_float),
        ("height_amp", ctypes.c_float),
        ("cave_period", ctypes.c_uint32),
        ("cave_threshold", ctypes.c_float),
    ]


class BrickMap(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32),
        ("ptr", ctypes.POINTER(ctypes.c_uint32)),
        ("occ", ctypes.POINTER(ctypes.c_uint64)),
        ("mat", ctypes.POINTER(ctypes.c_uint16)),
        ("n_bricks", ctypes.c_uint64),
        ("cap_bricks", ctypes.c_uint64),
    ]


class Source(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int),
        ("data", ctypes.c_void_p),
        ("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32),
        ("bm", ctypes.POINTER(BrickMap)),
    ]


class Camera(ctypes.Structure):
    _fields_ = [
        ("origin_chunk", ctypes.c_int32 * 3),
        ("origin_frac", ctypes.c_float * 3),
        ("forward", ctypes.c_float * 3),
        ("right", ctypes.c_float * 3),
        ("up", ctypes.c_float * 3),
        ("tan_half_fov_y", ctypes.c_float),
        ("width", ctypes.c_uint32),
        ("height", ctypes.c_uint32),
    ]


class Sphere(ctypes.Structure):
    _fields_ = [
        ("center", ctypes.c_int32 * 3),
        ("radius", ctypes.c_int32),
        ("material", ctypes.c_uint16),
        ("pad", ctypes.c_uint16),
    ]


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    path = build()
    L = ctypes.CDLL(path)
    P = ctypes.POINTER
    u32, i32, u64, f32, vp = ctypes.c_uint32, ctypes.c_int32, ctypes.c_uint64, ctypes.c_float, ctypes.c_void_p
    sig = {
        "mo_pcg3d": (u32, [u32, u32, u32]),
        "mo_lattice": (f32, [u32, u32, u32, u32]),
        "mo_vnoise3": (f32, [u32, u32, u32, u32, u32]),
        "mo_fbm2": (f32, [u32, u32, u32, ctypes.c_int, u32]),
        "mo_gen_dense_u8": (None, [ctypes.c_int] * 3 + [u32, vp]),
        "mo_chunk_solid_target": (u32, [u32]),
        "mo_chunk_material_count": (u32, [u32]),
        "mo_gen_chunks_u16": (None, [ctypes.c_int, u32, vp, vp]),
        "mo_terrain_height": (f32, [P(Terrain), u32, u32]),
        "mo_build_terrain": (ctypes.c_int, [P(Terrain), ctypes.c_int, P(BrickMap)]),
        "mo_build_from_dense_u16": (ctypes.c_int, [ctypes.c_int] * 3 + [vp, P(BrickMap)]),
        "mo_brickmap_free": (None, [P(BrickMap)]),
        "mo_brickmap_to_dense": (None, [P(BrickMap), vp]),
        "mo_pack_quad": (u64, [u32, ctypes.c_int] + [ctypes.c_int] * 5 + [ctypes.c_uint16]),
        "mo_mesh_chunk": (u64, [P(Source), vp, u32, vp, u64]),
        "mo_mesh_chunks_mt": (u64, [P(Source), vp, u32, ctypes.c_int, vp, u64]),
        "mo_count_faces": (u64, [P(Source), vp]),
        "mo_camera_ray": (None, [P(Camera), u32, u32, vp]),
        "mo_trace_ray": (None, [P(BrickMap), vp, vp, vp, vp, ctypes.c_int, vp]),
        "mo_raymarch_mt": (None, [P(BrickMap), P(Camera), u32, vp, ctypes.c_int, ctypes.c_int, vp]),
        "mo_raymarch_rows_mt": (None, [P(BrickMap), P(Camera), u32, u32, vp, ctypes.c_int, ctypes.c_int, vp]),
        "mo_edit_spheres": (ctypes.c_int, [P(BrickMap), P(Sphere), u32]),
        "mo_dirty_chunks": (u32, [P(BrickMap), P(Sphere), u32, vp, u32]),
        "mo_hardware_threads": (ctypes.c_int, []),
        "mo_erode_mips": (None, [vp, ctypes.c_int, ctypes.c_int, vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _ptr(a: np.ndarray) -> ctypes.c_void_p:
    return ctypes.c_void_p(a.ctypes.data)


# ---------------------------------------------------------------- generators

def gen_dense_u8(nx: int, ny: int, nz: int, seed: int = 1) -> np.ndarray:
    out = np.zeros((nz, ny, nx), dtype=np.uint8)
    lib().mo_gen_dense_u8(nx, ny, nz, seed, _ptr(out))
    return out


def gen_chunks_u16(n: int, seed0: int = 1):
    out = np.zeros((n, 32, 32, 32), dtype=np.uint16)
    solid = np.zeros(n, dtype=np.uint32)
    lib().mo_gen_chunks_u16(n, seed0, _ptr(out), _ptr(solid))
    return out, solid


def terrain(nx, ny, nz, seed, height_period, height_octaves, height_base, height_amp,
            cave_period=48, cave_threshold=0.7) -> Terrain:
    return Terrain(nx, ny, nz, seed, height_period, height_octaves, height_base, height_amp,
                   cave_period, cave_threshold)


class HostBrickMap:
    """Owns an oracle brick map; exposes numpy views of its arrays."""

    def __init__(self, bm: BrickMap):
        self.bm = bm

    @classmethod
    def from_terrain(cls, t: Terrain, nthreads: int = 0) -> "HostBrickMap":
        bm = BrickMap()
        rc = lib().mo_build_terrain(ctypes.byref(t), nthreads, ctypes.byref(bm))
        if rc != 0:
            raise RuntimeError(f"mo_build_terrain failed: {rc}")
        return cls(bm)

    @classmethod
    def from_dense(cls, grid: np.ndarray) -> "HostBrickMap":
        g = np.ascontiguousarray(grid, dtype=np.uint16)
        nz, ny, nx = g.shape
        bm = BrickMap()
        rc = lib().mo_build_from_dense_u16(nx, ny, nz, _ptr(g), ctypes.byref(bm))
        if rc != 0:
            raise RuntimeError(f"mo_build_from_dense_u16 failed: {rc}")
        return cls(bm)

    @classmethod
    def from_arrays(cls, dims, ptr: np.ndarray, occ: np.ndarray, mat: np.ndarray) -> "HostBrickMap":
        """Wraps existing arrays (e.g. a scene copied back from the device);
        the arrays stay owned by numpy."""
        obj = cls.__new__(cls)
        obj._keep = (np.ascontiguousarray(ptr, dtype=np.uint32), np.ascontiguousarray(occ, dtype=np.uint64),
                     np.ascontiguousarray(mat, dtype=np.uint16))
        bm = BrickMap()
        bm.nx, bm.ny, bm.nz = dims
        bm.ptr = obj._keep[0].ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))
        bm.occ = obj._keep[1].ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))
        bm.mat = obj._keep[2].ctypes.data_as(ctypes.POINTER(ctypes.c_uint16))
        bm.n_bricks = bm.cap_bricks = obj._keep[1].shape[0]
        obj.bm = bm
        obj._borrowed = True
        return obj

    @property
    def dims(self):
        return (self.bm.nx, self.bm.ny, self.bm.nz)

    @property
    def brick_dims(self):
        return (self.bm.nx // 8, self.bm.ny // 8, self.bm.nz // 8)

    def ptr(self) -> np.ndarray:
        bx, by, bz = self.brick_dims
        return np.ctypeslib.as_array(self.bm.ptr, shape=(bz * by * bx,)).copy()

    def occ(self) -> np.ndarray:
        n = int(self.bm.n_bricks)
        if n == 0:
            return np.zeros((0, 8), dtype=np.uint64)
        return np.ctypeslib.as_array(self.bm.occ, shape=(n * 8,)).reshape(n, 8).copy()

    def mat(self) -> np.ndarray:
        n = int(self.bm.n_bricks)
        if n == 0:
            return np.zeros((0, 512), dtype=np.uint16)
        return np.ctypeslib.as_array(self.bm.mat, shape=(n * 512,)).reshape(n, 512).copy()

    def dense(self) -> np.ndarray:
        nx, ny, nz = self.dims
        out = np.zeros((nz, ny, nx), dtype=np.uint16)
        lib().mo_brickmap_to_dense(ctypes.byref(self.bm), _ptr(out))
        return out

    def edit(self, spheres) -> None:
        arr = (Sphere * len(spheres))(*spheres)
        rc = lib().mo_edit_spheres(ctypes.byref(self.bm), arr, len(spheres))
        if rc != 0:
            raise RuntimeError("mo_edit_spheres failed")

    def dirty_chunks(self, spheres) -> np.ndarray:
        arr = (Sphere * max(1, len(spheres)))(*spheres)
        cx, cy, cz = self.bm.nx // 32, self.bm.ny // 32, self.bm.nz // 32
        out = np.zeros(cx * cy * cz, dtype=np.uint32)
        n = lib().mo_dirty_chunks(ctypes.byref(self.bm), arr, len(spheres), _ptr(out), out.size)
        return out[:n].copy()

    def __del__(self):
        if getattr(self, "_borrowed", False):
            return
        if getattr(self, "bm", None) is not None and _lib is not None:
            _lib.mo_brickmap_free(ctypes.byref(self.bm))
            self.bm = None


# ---------------------------------------------------------------- meshing

def _source(kind, data=None, dims=(0, 0, 0), bm: HostBrickMap | None = None) -> Source:
    s = Source()
    s.kind = kind
    s.data = ctypes.c_void_p(data.ctypes.data) if data is not None else None
    s.nx, s.ny, s.nz = dims
    s.bm = ctypes.pointer(bm.bm) if bm is not None else ctypes.POINTER(BrickMap)()
    return s


def mesh_chunks(kind, data=None, coords=None, n=None, bm=None, nthreads=0, dims=None) -> np.ndarray:
    """Meshes chunks and returns canonically sorted packed quads (uint64)."""
    if data is not None:
        data = np.ascontiguousarray(data)
    if kind in (SRC_CHUNKS_U16, SRC_CHUNKS_U8):
        n = data.shape[0] if n is None else n
        c = np.zeros((n, 3), dtype=np.int32)
        c[:, 0] = np.arange(n) if coords is None else np.asarray(coords)[:, 0]
        src = _source(kind, data)
    else:
        c = np.ascontiguousarray(np.asarray(coords, dtype=np.int32).reshape(-1, 3))
        n = c.shape[0]
        if kind == SRC_BRICKMAP:
            src = _source(kind, bm=bm)
        else:
            nz, ny, nx = data.shape if dims is None else dims[::-1]
            src = _source(kind, data, (nx, ny, nz))
    cap = 0
    total = lib().mo_mesh_chunks_mt(ctypes.byref(src), _ptr(c), n, nthreads, None, 0)
    out = np.zeros(max(1, total), dtype=np.uint64)
    cap = out.size
    total2 = lib().mo_mesh_chunks_mt(ctypes.byref(src), _ptr(c), n, nthreads, _ptr(out), cap)
    assert total2 == total
    return out[:total]


def count_faces(kind, data=None, coord=(0, 0, 0), bm=None) -> int:
    if data is not None:
        data = np.ascontiguousarray(data)
    if kind in (SRC_CHUNKS_U16, SRC_CHUNKS_U8):
        src = _source(kind, data)
    elif kind == SRC_BRICKMAP:
        src = _source(kind, bm=bm)
    else:
        nz, ny, nx = data.shape
        src = _source(kind, data, (nx, ny, nz))
    cc = np.asarray(coord, dtype=np.int32)
    return int(lib().mo_count_faces(ctypes.byref(src), _ptr(cc)))


def unpack_quads(q: np.ndarray) -> dict:
    q = np.asarray(q, dtype=np.uint64)
    f = lambda sh, bits: ((q >> np.uint64(sh)) & np.uint64((1 << bits) - 1)).astype(np.int64)
    return {
        "chunk": f(44, 20), "dir": f(41, 3), "z": f(36, 5), "y": f(31, 5), "x": f(26, 5),
        "w": f(21, 5) + 1, "h": f(16, 5) + 1, "material": f(0, 16),
    }


# ---------------------------------------------------------------- raymarching

def camera(origin, target, width, height, fov_y_deg=60.0, up=(0.0, 0.0, 1.0)) -> Camera:
    """Pinhole camera looking from origin at target (z-up), chunk-rebased origin."""
    return Camera(**camera_fields(origin, target, width, height, fov_y_deg, up))


def camera_fields(origin, target, width, height, fov_y_deg=60.0, up=(0.0, 0.0, 1.0)) -> dict:
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
    return {
        "origin_chunk": (ctypes.c_int32 * 3)(*[int(v) for v in ch]),
        "origin_frac": (ctypes.c_float * 3)(*[float(v) for v in frac]),
        "forward": (ctypes.c_float * 3)(*[float(v) for v in f]),
        "right": (ctypes.c_float * 3)(*[float(v) for v in r]),
        "up": (ctypes.c_float * 3)(*[float(v) for v in u]),
        "tan_half_fov_y": float(np.tan(np.radians(fov_y_deg) / 2.0)),
        "width": int(width),
        "height": int(height),
    }


def light_dir(v=(0.3, 0.5, 0.8)) -> np.ndarray:
    a = np.asarray(v, dtype=np.float64)
    return (a / np.linalg.norm(a)).astype(np.float32)


def raymarch(bm: HostBrickMap, cams, light=None, shadow=True, nthreads=0) -> np.ndarray:
    cams = list(cams) if isinstance(cams, (list, tuple)) else [cams]
    arr = (Camera * len(cams))(*cams)
    total = sum(c.width * c.height for c in cams)
    hits = np.zeros(total, dtype=HIT_DTYPE)
    L = light_dir() if light is None else np.asarray(light, dtype=np.float32)
    lib().mo_raymarch_mt(ctypes.byref(bm.bm), arr, len(cams), _ptr(L), int(shadow), nthreads, _ptr(hits))
    return hits


def trace_ray(bm: HostBrickMap, origin, direction, light=None, shadow=False):
    """Traces one ray from a world-space origin (chunk-rebased internally)."""
    o = np.asarray(origin, dtype=np.float64)
    ch = np.floor(o / 32.0).astype(np.int32)
    frac = (o - ch * 32.0).astype(np.float32)
    d = np.asarray(direction, dtype=np.float32)
    L = light_dir() if light is None else np.asarray(light, dtype=np.float32)
    h = np.zeros(1, dtype=HIT_DTYPE)
    lib().mo_trace_ray(ctypes.byref(bm.bm), _ptr(ch), _ptr(frac), _ptr(d), _ptr(L), int(shadow), _ptr(h))
    return h[0]


def raymarch_rows(bm: HostBrickMap, cam: Camera, row0: int, n_rows: int, light=None, shadow=True,
                  nthreads=0) -> np.ndarray:
    hits = np.zeros(cam.width * n_rows, dtype=HIT_DTYPE)
    L = light_dir() if light is None else np.asarray(light, dtype=np.float32)
    lib().mo_raymarch_rows_mt(ctypes.byref(bm.bm), ctypes.byref(cam), row0, n_rows, _ptr(L), int(shadow),
                              nthreads, _ptr(hits))
    return hits


def hardware_threads() -> int:
    return int(lib().mo_hardware_threads())


# ---------------------------------------------------------------- downstream

def erode_mips(occ: np.ndarray, depth: int) -> np.ndarray:
    """Erosion pyramid of one cubic chunk (occupancy [z][y][x]); returns
    [depth][z][y][x] uint8 (the reference's CalculateOccupancyErodeMipmaps)."""
    o = np.ascontiguousarray(occ != 0, dtype=np.uint8)
    R = o.shape[0]
    out = np.zeros((depth, R, R, R), dtype=np.uint8)
    lib().mo_erode_mips(_ptr(o), R, depth, _ptr(out))
    return out


def quads_to_vertices(quads: np.ndarray, chunk_origins: np.ndarray) -> np.ndarray:
    """Four corners per packed quad, counter-clockwise seen from outside:
    returns float32 positions [n, 4, 3] and uint32 attributes [n, 4]
    (material | dir << 16 | corner << 19), positions in world voxel units."""
    u = unpack_quads(quads)
    n = len(quads)
    org = np.asarray(chunk_origins, dtype=np.int64).reshape(-1, 3)[u["chunk"]] * 32
    d = u["dir"]
    a = d // 2
    plus = (d % 2) == 0
    loc = np.stack([u["x"], u["y"], u["z"]], 1)
    ua = np.where(a == 0, 1, 0)
    va = np.where(a == 2, 1, 2)
    pa = loc[np.arange(n), a] + plus
    u0 = loc[np.arange(n), ua]
    v0 = loc[np.arange(n), va]
    natural = np.where(a == 1, ~plus, plus)
    pos = np.zeros((n, 4, 3), dtype=np.int64)
    attr = np.zeros((n, 4), dtype=np.uint32)
    for k in range(4):
        c = np.where(natural, k, (4 - k) % 4)
        cu = np.where((c == 1) | (c == 2), u0 + u["w"], u0)
        cv = np.where(c >= 2, v0 + u["h"], v0)
        p = np.zeros((n, 3), dtype=np.int64)
        p[np.arange(n), a] = pa
        p[np.arange(n), ua] = cu
        p[np.arange(n), va] = cv
        pos[:, k] = p + org
        attr[:, k] = (u["material"] | (d << 16) | (k << 19)).astype(np.uint32)
    return pos.astype(np.float32), attr
