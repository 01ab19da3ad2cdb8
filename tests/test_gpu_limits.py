"""Argument limits and degenerate inputs at the C ABI: every bad call is
rejected with MESO_ERR_INVALID_ARG before anything is launched, and tiny or
one-pixel workloads still match the oracle."""
import ctypes

import numpy as np
import pytest

import oracle
import mesoengine_gb300 as meso

pytestmark = pytest.mark.gpu

INVALID_ARG = 1


def test_mesh_rejects_oversized_and_malformed_calls(ctx):
    L = meso.load()
    data, _ = ctx.generate_chunks_u16(2, seed0=3)
    q, cnt = ctx.alloc(1024 * 8), ctx.alloc(8)
    out = meso.MeshOutput(q.ptr, 1024, cnt.ptr, None)
    src = meso.MeshSource()
    src.kind = meso.SRC_CHUNKS_U16
    src.d_data = data.ptr
    # more chunks than one call may carry
    assert L.meso_mesh_chunks(ctx.handle, ctypes.byref(src), None, meso.MAX_CHUNKS_PER_CALL + 1,
                              ctypes.byref(out), None) == INVALID_ARG
    # unknown source kind
    bad = meso.MeshSource()
    bad.kind = 99
    bad.d_data = data.ptr
    assert L.meso_mesh_chunks(ctx.handle, ctypes.byref(bad), None, 1, ctypes.byref(out), None) == INVALID_ARG
    # grid dims that are not multiples of 32
    g = meso.MeshSource()
    g.kind = meso.SRC_GRID_U8
    g.d_data = data.ptr
    g.nx, g.ny, g.nz = 48, 32, 32
    coords = ctx.to_device(np.zeros((1, 3), np.int32))
    assert L.meso_mesh_chunks(ctx.handle, ctypes.byref(g), coords.ptr, 1, ctypes.byref(out), None) == INVALID_ARG
    # a chunk array that is not 16-byte aligned
    mis = meso.MeshSource()
    mis.kind = meso.SRC_CHUNKS_U16
    mis.d_data = data.ptr + 8
    assert L.meso_mesh_chunks(ctx.handle, ctypes.byref(mis), None, 1, ctypes.byref(out), None) == INVALID_ARG
    ctx.sync()


def test_scene_and_camera_limits(ctx):
    with pytest.raises(meso.MesoError) as e:
        ctx.scene_from_dense(np.zeros((32, 32, 48), np.uint16))  # nx = 48
    assert e.value.status == INVALID_ARG
    with pytest.raises(meso.MesoError) as e:
        ctx.scene_from_terrain(meso.Terrain(16384, 32, 32, 1, 64, 3, 8.0, 8.0, 16, 0.7))
    assert e.value.status == INVALID_ARG
    scene = ctx.scene_from_dense(np.zeros((32, 32, 32), np.uint16))
    for w, h in [(0, 8), (8, 0), (16385, 1)]:
        with pytest.raises(meso.MesoError) as e:
            ctx.raymarch(scene, meso.camera((-8.0, -8.0, 40.0), (16.0, 16.0, 16.0), w, h))
        assert e.value.status == INVALID_ARG
    # shadow rays need a light direction
    L = meso.load()
    hits = ctx.alloc(64 * 24)
    cam = meso.camera((-8.0, -8.0, 40.0), (16.0, 16.0, 16.0), 8, 8)
    sh = (ctypes.c_void_p * 1)(scene.handle)
    assert L.meso_raymarch(ctx.handle, sh, ctypes.byref(cam), 1, None, meso.RAY_SHADOW, hits.ptr, None) == INVALID_ARG
    scene.destroy()


def test_downstream_limits(ctx):
    L = meso.load()
    q = ctx.to_device(np.zeros(4, np.uint64))
    org = ctx.to_device(np.zeros((1, 3), np.int32))
    out = ctx.alloc(4 * 64 + 16)
    assert L.meso_quads_to_vertices(ctx.handle, q.ptr, 4, org.ptr, 1, out.ptr + 8, None) == INVALID_ARG
    data, _ = ctx.generate_chunks_u16(1, seed0=5)
    src = meso.MeshSource()
    src.kind = meso.SRC_CHUNKS_U16
    src.d_data = data.ptr
    mips = ctx.alloc(9 * 4096)
    for depth in (0, 9):
        assert L.meso_erode_mips(ctx.handle, ctypes.byref(src), None, 1, depth, mips.ptr, None) == INVALID_ARG
    ctx.sync()


def test_l2_read_measurement(ctx):
    # the L2 probe reads an L2-resident buffer: faster than the HBM copy peak
    g = ctx.measure_l2_read(32 << 20, 20)
    assert g > 3000.0
    L = meso.load()
    out = ctypes.c_double()
    for nbytes, passes in [(1 << 10, 10), ((64 << 20) + 16, 10), ((1 << 20) + 8, 10), (1 << 20, 0), (1 << 20, 1001)]:
        assert L.meso_measure_l2_read(ctx.handle, nbytes, passes, ctypes.byref(out)) == INVALID_ARG


def test_degenerate_workloads_match_oracle(ctx):
    # one solid voxel in the corner of a 32^3 scene; a 1x1 and a 1x7 image
    g = np.zeros((32, 32, 32), np.uint16)
    g[0, 0, 0] = 5
    scene = ctx.scene_from_dense(g)
    bm = oracle.HostBrickMap.from_dense(g)
    for w, h in [(1, 1), (1, 7), (7, 1)]:
        o, tg = (-3.0, -2.0, 4.0), (0.5, 0.5, 0.5)
        got = ctx.raymarch(scene, meso.camera(o, tg, w, h))
        ref = oracle.raymarch(bm, oracle.camera(o, tg, w, h))
        assert np.array_equal(got.view(np.uint8), ref.view(np.uint8))
    q, _ = ctx.mesh(meso.SRC_BRICKMAP, coords=np.zeros((1, 3), np.int32), scene=scene)
    assert np.array_equal(np.sort(q), oracle.mesh_chunks(oracle.SRC_BRICKMAP, coords=np.zeros((1, 3), np.int32), bm=bm))
    assert len(q) == 6
    scene.destroy()
