"""Erosion pyramid, quad -> vertex expansion and brick-map files on the GPU,
against the oracle."""
import ctypes
import os
import tempfile

import numpy as np
import pytest

import oracle
import mesoengine_gb300 as meso

pytestmark = pytest.mark.gpu


def _bits_to_dense(words):
    """[depth][z][y] uint32 words (bit x) -> [depth][z][y][x] uint8."""
    w = np.asarray(words, dtype=np.uint32)
    return ((w[..., None] >> np.arange(32, dtype=np.uint32)) & 1).astype(np.uint8)


def test_erode_mips_chunk_array_matches_reference_loop(ctx):
    n = 24
    dev, _ = ctx.generate_chunks_u16(n, seed0=31)
    host = dev.download(np.uint16).reshape(n, 32, 32, 32)
    solid = np.zeros((1, 32, 32, 32), np.uint16)
    solid[0, 4:28, 2:30, 5:31] = 3
    both = np.concatenate([host, solid])
    got = ctx.erode_mips(meso.SRC_CHUNKS_U16, ctx.to_device(both), n=both.shape[0], depth=4)
    for i in range(both.shape[0]):
        ref = oracle.erode_mips(both[i], 4)
        assert np.array_equal(_bits_to_dense(got[i]), ref), i
    assert _bits_to_dense(got[-1])[3].sum() > 0


def test_erode_mips_u8_chunks_with_index_list(ctx):
    # uint8 chunk arrays take the 16-byte load path too; an index list picks
    # chunks out of order and repeats one
    rng = np.random.default_rng(5)
    chunks = ((rng.random((6, 32, 32, 32)) < 0.8) * rng.integers(1, 255, (6, 32, 32, 32))).astype(np.uint8)
    chunks[2] = 0
    chunks[3, 1:31, 1:31, 1:31] = 9
    idx = np.array([[3], [0], [5], [3], [2]], dtype=np.int32)
    got = ctx.erode_mips(meso.SRC_CHUNKS_U8, ctx.to_device(chunks), coords=idx, depth=4)
    for i, c in enumerate(idx[:, 0]):
        assert np.array_equal(_bits_to_dense(got[i]), oracle.erode_mips(chunks[c], 4)), i


def test_erode_mips_grid_and_brickmap(ctx):
    g = ctx.generate_dense_u8(64, 64, 64, seed=3)
    grid = g.download(np.uint8).reshape(64, 64, 64)
    coords = np.array([(x, y, z) for z in range(2) for y in range(2) for x in range(2)], dtype=np.int32)
    got = ctx.erode_mips(meso.SRC_GRID_U8, g, coords=coords, dims=(64, 64, 64), depth=3)
    scene = ctx.scene_from_dense(grid.astype(np.uint16))
    got_b = ctx.erode_mips(meso.SRC_BRICKMAP, coords=coords, scene=scene, depth=3)
    for i, (x, y, z) in enumerate(coords):
        chunk = grid[32 * z:32 * z + 32, 32 * y:32 * y + 32, 32 * x:32 * x + 32]
        ref = oracle.erode_mips(chunk, 3)
        assert np.array_equal(_bits_to_dense(got[i]), ref)
        assert np.array_equal(_bits_to_dense(got_b[i]), ref)


def test_quads_to_vertices_matches_oracle(ctx):
    n = 16
    dev, _ = ctx.generate_chunks_u16(n, seed0=77)
    q, _ = ctx.mesh(meso.SRC_CHUNKS_U16, dev, n=n)
    origins = np.array([(i % 4, (i // 4) % 4, i // 16 - 3) for i in range(n)], dtype=np.int32)
    v = ctx.quads_to_vertices(q, origins)
    pos, attr = oracle.quads_to_vertices(q, origins)
    assert v.shape[0] == 4 * len(q)
    got = np.stack([v["x"], v["y"], v["z"]], 1).reshape(-1, 4, 3)
    assert np.array_equal(got, pos)
    assert np.array_equal(v["attr"].reshape(-1, 4), attr)


def test_scene_file_roundtrip(ctx):
    t = meso.terrain_preset("small")
    scene = ctx.scene_from_terrain(t, spare_bricks=2048)
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "s.meso")
        scene.save(path)
        back = ctx.scene_load(path)
        for a, b in zip(scene.download(), back.download()):
            assert np.array_equal(a[: len(b)], b)
        # after edits the pool order is no longer canonical; the file is
        sp = [meso.SphereEdit((ctypes.c_int32 * 3)(60, 60, 20), 9, 0, 0),
              meso.SphereEdit((ctypes.c_int32 * 3)(20, 90, 40), 6, 777, 0)]
        scene.edit(sp)
        scene.save(path)
        back2 = ctx.scene_load(path, spare_bricks=16)
        assert np.array_equal(back2.dense(), scene.dense())
        cam = meso.camera((-40.0, -30.0, 140.0), (64.0, 64.0, 20.0), 48, 32)
        assert np.array_equal(ctx.raymarch(back2, cam).view(np.uint8), ctx.raymarch(scene, cam).view(np.uint8))
        bm = oracle.HostBrickMap.from_dense(scene.dense())
        ptr, occ, mat = back2.download()
        assert np.array_equal(ptr, bm.ptr())
        assert np.array_equal(occ[: bm.bm.n_bricks], bm.occ())
        with open(path, "r+b") as f:
            f.write(b"NOTMESO!")
        with pytest.raises(meso.MesoError):
            ctx.scene_load(path)
