"""Sphere edits on a device brick map, dirty chunks and remeshing, against the oracle."""
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
        r = int(rng.integers(2, rmax + 1))
        m = 0 if rng.random() < 0.5 else int(rng.integers(1, 65536))
        out.append((c, r, m))
    return out


def _dev(sp):
    return [meso.SphereEdit((ctypes.c_int32 * 3)(*c), r, m, 0) for c, r, m in sp]


def _host(sp):
    return [oracle.Sphere((ctypes.c_int32 * 3)(*c), r, m, 0) for c, r, m in sp]


def _coords(idx, dims):
    cx, cy = dims[0] // 32, dims[1] // 32
    idx = np.asarray(idx, dtype=np.int64)
    return np.stack([idx % cx, (idx // cx) % cy, idx // (cx * cy)], 1).astype(np.int32)


def test_edits_dirty_remesh_render(ctx):
    t = meso.terrain_preset("small")
    scene = ctx.scene_from_terrain(t, spare_bricks=8192)
    bm = oracle.HostBrickMap.from_terrain(_oracle_terrain(t))
    dims = (t.nx, t.ny, t.nz)
    for step, seed in enumerate([3, 4, 5]):
        sp = _spheres(24, seed, dims)
        dirty = scene.edit(_dev(sp))
        bm.edit(_host(sp))
        odirty = bm.dirty_chunks(_host(sp))
        assert np.array_equal(dirty, odirty)
        dense = scene.dense()
        assert np.array_equal(dense, bm.dense()), f"content differs after edit batch {step}"
        # emptiness of the pointer grid follows content (empty bricks unlinked)
        ptr = scene.download()[0]
        occupied = dense.reshape(16, 8, 16, 8, 16, 8).any(axis=(1, 3, 5)).ravel()
        assert np.array_equal(ptr != meso.EMPTY_BRICK, occupied)
        # remesh of the dirty chunks
        coords = _coords(dirty, dims)
        q, _ = ctx.mesh(meso.SRC_BRICKMAP, coords=coords, scene=scene)
        ref = oracle.mesh_chunks(oracle.SRC_BRICKMAP, coords=coords, bm=bm)
        assert np.array_equal(np.sort(q), ref)
        # render after the edit
        cam = meso.camera((-40.0, -30.0, 140.0), (64.0, 64.0, 20.0), 64, 40)
        got = ctx.raymarch(scene, cam)
        exp = oracle.raymarch(bm, oracle.camera((-40.0, -30.0, 140.0), (64.0, 64.0, 20.0), 64, 40))
        for f in ("voxel", "material", "face", "shadow", "steps", "shadow_steps"):
            assert np.array_equal(got[f], exp[f]), f
        assert np.array_equal(got["t"].view(np.uint32), exp["t"].view(np.uint32))


def test_edit_pool_exhaustion_reports_oom(ctx):
    g = np.zeros((64, 64, 64), np.uint16)
    g[0, 0, 0] = 1
    scene = ctx.scene_from_dense(g, spare_bricks=0)
    with pytest.raises(meso.MesoError) as e:
        scene.edit(_dev([([40, 40, 40], 10, 7)]))
    assert e.value.status == 2  # MESO_ERR_OOM
    # the scene stays usable: removing the one voxel that was there works
    scene.edit(_dev([([0, 0, 0], 1, 0)]))
    assert scene.dense()[0:2, 0:2, 0:2].max() == 0


def test_edit_remove_everything_unlinks_bricks(ctx):
    rng = np.random.default_rng(9)
    g = ((rng.random((64, 64, 64)) < 0.2) * 5).astype(np.uint16)
    scene = ctx.scene_from_dense(g)
    scene.edit(_dev([([32, 32, 32], 60, 0)]))
    ptr = scene.download()[0]
    assert (ptr == meso.EMPTY_BRICK).all()
    assert scene.info().n_bricks == 0


def test_large_edits_match_oracle(ctx):
    # spheres whose boxes cover most of the grid take the bitmap path for the
    # touched bricks and dirty chunks; small ones beside them the sorted path
    t = meso.terrain_preset("small")
    scene = ctx.scene_from_terrain(t, spare_bricks=1 << 16)
    bm = oracle.HostBrickMap.from_terrain(_oracle_terrain(t))
    dims = (t.nx, t.ny, t.nz)
    for sp in ([([64, 64, 40], 90, 0)], [([20, 100, 10], 70, 513), ([5, 5, 5], 3, 9)], [([64, 64, 64], 200, 77)]):
        dirty = scene.edit(_dev(sp))
        bm.edit(_host(sp))
        assert np.array_equal(dirty, bm.dirty_chunks(_host(sp)))
        assert np.array_equal(scene.dense(), bm.dense())
