"""The resident per-chunk mesh store: after batches of sphere edits, each
chunk's segment holds exactly the oracle's greedy quads for that chunk of
the edited scene (bit-exact after the canonical sort)."""
import ctypes

import numpy as np
import pytest

import oracle
import mesoengine_gb300 as meso

pytestmark = pytest.mark.gpu


def _oracle_terrain(t):
    return oracle.terrain(t.nx, t.ny, t.nz, t.seed, t.height_period, t.height_octaves, t.height_base,
                          t.height_amp, t.cave_period, t.cave_threshold)


def _spheres(n, seed, dims, rmax=20):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        c = [int(rng.integers(-8, d + 8)) for d in dims]
        m = 0 if rng.random() < 0.5 else int(rng.integers(1, 65536))
        out.append((c, int(rng.integers(2, rmax + 1)), m))
    return out


def _coords(dims):
    cx, cy, cz = dims[0] // 32, dims[1] // 32, dims[2] // 32
    idx = np.arange(cx * cy * cz, dtype=np.int64)
    return np.stack([idx % cx, (idx // cx) % cy, idx // (cx * cy)], 1).astype(np.int32)


def _assert_store_matches(store, bm, dims):
    n = (dims[0] // 32) * (dims[1] // 32) * (dims[2] // 32)
    got = np.sort(store.gather(np.arange(n)))
    ref = oracle.mesh_chunks(oracle.SRC_BRICKMAP, coords=_coords(dims), bm=bm)
    assert got.shape == ref.shape
    assert np.array_equal(got, ref)
    info = store.info()
    assert info.live_quads == len(ref)
    assert info.arena_used <= info.arena_quads


def test_store_follows_edits(ctx):
    t = meso.terrain_preset("small")
    scene = ctx.scene_from_terrain(t, spare_bricks=8192)
    bm = oracle.HostBrickMap.from_terrain(_oracle_terrain(t))
    dims = (t.nx, t.ny, t.nz)
    store = ctx.mesh_store(scene)
    _assert_store_matches(store, bm, dims)
    for seed in (3, 4, 5, 6):
        sp = _spheres(24, seed, dims)
        dirty = scene.edit([meso.SphereEdit((ctypes.c_int32 * 3)(*c), r, m, 0) for c, r, m in sp])
        bm.edit([oracle.Sphere((ctypes.c_int32 * 3)(*c), r, m, 0) for c, r, m in sp])
        store.update(dirty)
        _assert_store_matches(store, bm, dims)
    store.destroy()


def test_store_repacks_when_full(ctx):
    """Edits that grow most chunks' quad counts push the bump pointer past a
    small arena; the store repacks (and grows) it and stays exact."""
    t = meso.terrain_preset("small")
    scene = ctx.scene_from_terrain(t, spare_bricks=1 << 16)
    bm = oracle.HostBrickMap.from_terrain(_oracle_terrain(t))
    dims = (t.nx, t.ny, t.nz)
    store = ctx.mesh_store(scene)
    # many small random-material spheres raise every touched chunk's count
    rng = np.random.default_rng(17)
    for _ in range(6):
        sp = [([int(rng.integers(0, d)) for d in dims], int(rng.integers(2, 6)), int(rng.integers(1, 65536)))
              for _ in range(160)]
        dirty = scene.edit([meso.SphereEdit((ctypes.c_int32 * 3)(*c), r, m, 0) for c, r, m in sp])
        bm.edit([oracle.Sphere((ctypes.c_int32 * 3)(*c), r, m, 0) for c, r, m in sp])
        store.update(dirty)
    assert store.info().compactions >= 1
    _assert_store_matches(store, bm, dims)
    # an update of no chunks, of unchanged chunks and of a list with repeats
    # keeps everything
    store.update([])
    store.update(np.arange(8))
    store.update(np.array([3, 9, 3, 3, 40, 9], np.uint32))
    _assert_store_matches(store, bm, dims)
    store.destroy()


def test_store_of_empty_scene_and_emptied_scene(ctx):
    """A scene with no solid voxel has an empty store; a scene whose every
    solid voxel is removed by edits ends with an empty store; refilling it
    brings the quads back, each time equal to the oracle."""
    g = np.zeros((64, 64, 64), np.uint16)
    scene = ctx.scene_from_dense(g, spare_bricks=4096)
    bm = oracle.HostBrickMap.from_dense(g)
    store = ctx.mesh_store(scene)
    assert store.info().live_quads == 0
    assert store.gather(np.arange(8)).size == 0
    fill = [((32, 32, 32), 20, 77), ((10, 50, 20), 6, 5)]
    dirty = scene.edit([meso.SphereEdit((ctypes.c_int32 * 3)(*c), r, m, 0) for c, r, m in fill])
    bm.edit([oracle.Sphere((ctypes.c_int32 * 3)(*c), r, m, 0) for c, r, m in fill])
    store.update(dirty)
    _assert_store_matches(store, bm, (64, 64, 64))
    clear = [((32, 32, 32), 60, 0)]
    dirty = scene.edit([meso.SphereEdit((ctypes.c_int32 * 3)(*c), r, m, 0) for c, r, m in clear])
    bm.edit([oracle.Sphere((ctypes.c_int32 * 3)(*c), r, m, 0) for c, r, m in clear])
    store.update(dirty)
    assert store.info().live_quads == 0
    _assert_store_matches(store, bm, (64, 64, 64))
    store.destroy()
