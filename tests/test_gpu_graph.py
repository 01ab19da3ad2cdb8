"""CUDA-graph capture of the batched mesher and the multi-view raymarch:
replays give the same results as direct calls."""
import ctypes

import numpy as np
import pytest

import mesoengine_gb300 as meso

pytestmark = pytest.mark.gpu


def test_graph_replay_mesh_and_raymarch(ctx):
    L = meso.load()
    st = ctx.stream()
    n = 96
    data, _ = ctx.generate_chunks_u16(n, seed0=5)
    ref, _ = ctx.mesh(meso.SRC_CHUNKS_U16, data, n=n)
    cap = n * 16384
    qbuf, cnt = ctx.alloc(cap * 8), ctx.alloc(8)
    src = meso.MeshSource()
    src.kind = meso.SRC_CHUNKS_U16
    src.d_data = data.ptr
    out = meso.MeshOutput(qbuf.ptr, cap, cnt.ptr, None)
    scene = ctx.scene_from_terrain(meso.terrain_preset("small"))
    cams = [meso.camera((-40.0 + 9 * i, -30.0, 140.0), (64.0, 64.0, 20.0), 64, 40) for i in range(3)]
    ref_hits = ctx.raymarch(scene, cams)
    hits = ctx.alloc(sum(c.width * c.height for c in cams) * 24)
    sh = (ctypes.c_void_p * 3)(*([scene.handle] * 3))
    ca = (meso.Camera * 3)(*cams)
    light = meso.light_dir()

    def work():
        meso._check(L.meso_mesh_chunks(ctx.handle, ctypes.byref(src), None, n, ctypes.byref(out), st))
        meso._check(L.meso_raymarch(ctx.handle, sh, ca, 3, light.ctypes.data, meso.RAY_SHADOW, hits.ptr, st))

    g = ctx.capture(work, st)
    for _ in range(3):
        qbuf.zero(st)
        hits.zero(st)
        g.launch(st)
        ctx.sync(st)
        total = int(cnt.download(np.uint64, 1, stream=st)[0])
        q = qbuf.download(np.uint64, total, stream=st)
        assert np.array_equal(np.sort(q), np.sort(ref))
        assert np.array_equal(hits.download(meso.HIT_DTYPE, ref_hits.shape[0], stream=st).view(np.uint8),
                              ref_hits.view(np.uint8))
    g.destroy()


def test_graph_replay_raymarch_view_table(ctx):
    """More than 32 views take the device view-table path (per-call table,
    descriptors written by kernels whose parameters the graph keeps by
    value); replays after the capturing call has returned give the direct
    call's hits."""
    L = meso.load()
    st = ctx.stream()
    scene = ctx.scene_from_terrain(meso.terrain_preset("small"))
    rng = np.random.default_rng(11)
    cams = [meso.camera((rng.uniform(-60, -20), rng.uniform(-60, 190), rng.uniform(60, 160)),
                        (rng.uniform(30, 100), rng.uniform(30, 100), rng.uniform(0, 30)),
                        int(rng.integers(8, 40)), int(rng.integers(8, 30))) for _ in range(70)]
    ref = ctx.raymarch(scene, cams)
    hits = ctx.alloc(ref.shape[0] * 24)
    light = meso.light_dir()

    def work():
        sh = (ctypes.c_void_p * len(cams))(*([scene.handle] * len(cams)))
        ca = (meso.Camera * len(cams))(*cams)
        meso._check(L.meso_raymarch(ctx.handle, sh, ca, len(cams), light.ctypes.data, meso.RAY_SHADOW, hits.ptr, st))

    g = ctx.capture(work, st)
    for _ in range(2):
        hits.zero(st)
        g.launch(st)
        ctx.sync(st)
        assert np.array_equal(hits.download(meso.HIT_DTYPE, ref.shape[0], stream=st).view(np.uint8),
                              ref.view(np.uint8))
    g.destroy()
