"""GPU scene build and raymarching against the CPU oracle.

Hit voxel, face, material, shadow flag and step counts are compared bit for
bit; the hit distance t within 1e-6 relative (it is in fact bit-identical:
both sides evaluate the same sequence of correctly rounded FP32 operations).
"""
import ctypes

import numpy as np
import pytest

import oracle
import mesoengine_gb300 as meso

pytestmark = pytest.mark.gpu
T_RTOL = 1e-6


def _oracle_terrain(t: meso.Terrain):
    return oracle.terrain(t.nx, t.ny, t.nz, t.seed, t.height_period, t.height_octaves, t.height_base,
                          t.height_amp, t.cave_period, t.cave_threshold)


def assert_hits_equal(got, ref):
    assert got.shape == ref.shape
    for f in ("voxel", "material", "face", "shadow", "steps", "shadow_steps"):
        bad = np.nonzero(got[f] != ref[f])[0]
        assert bad.size == 0, f"{f} differs at {bad[:8]}: {got[f][bad[:8]]} vs {ref[f][bad[:8]]}"
    hit = np.isfinite(ref["t"])
    assert np.array_equal(np.isfinite(got["t"]), hit)
    np.testing.assert_allclose(got["t"][hit], ref["t"][hit], rtol=T_RTOL, atol=0)


@pytest.fixture(scope="module")
def small(ctx):
    t = meso.terrain_preset("small")
    scene = ctx.scene_from_terrain(t)
    bm = oracle.HostBrickMap.from_terrain(_oracle_terrain(t))
    return t, scene, bm


def test_terrain_build_bit_exact(small):
    t, scene, bm = small
    ptr, occ, mat = scene.download()
    assert np.array_equal(ptr, bm.ptr())
    assert np.array_equal(occ, bm.occ())
    assert np.array_equal(mat, bm.mat())


def test_terrain_256_bit_exact(ctx):
    t = meso.Terrain(256, 256, 256, 5, 128, 6, 14.0, 64.0, 48, 0.7)
    scene = ctx.scene_from_terrain(t)
    bm = oracle.HostBrickMap.from_terrain(_oracle_terrain(t))
    ptr, occ, mat = scene.download()
    assert np.array_equal(ptr, bm.ptr())
    assert np.array_equal(occ, bm.occ())
    assert np.array_equal(mat, bm.mat())


def test_dense_scene_roundtrip(ctx):
    rng = np.random.default_rng(1)
    g = ((rng.random((64, 64, 96)) < 0.05) * rng.integers(1, 9, (64, 64, 96))).astype(np.uint16)
    s = ctx.scene_from_dense(g)
    assert np.array_equal(s.dense(), g)
    bm = oracle.HostBrickMap.from_dense(g)
    ptr, occ, mat = s.download()
    assert np.array_equal(ptr, bm.ptr())
    assert np.array_equal(occ, bm.occ())


@pytest.mark.parametrize("shadow", [True, False])
def test_raymarch_small_matches_oracle(ctx, small, shadow):
    t, scene, bm = small
    cam = meso.camera((-40.0, -30.0, 140.0), (64.0, 64.0, 20.0), 96, 64)
    ocam = oracle.camera((-40.0, -30.0, 140.0), (64.0, 64.0, 20.0), 96, 64)
    got = ctx.raymarch(scene, cam, shadow=shadow)
    ref = oracle.raymarch(bm, ocam, shadow=shadow)
    assert (ref["voxel"] != np.uint64(2**64 - 1)).sum() > 100
    assert_hits_equal(got, ref)


def test_raymarch_edge_cameras(ctx, small):
    t, scene, bm = small
    cases = [
        ((64.5, 64.5, 200.0), (64.5, 64.5, 0.0)),      # straight down, axis aligned
        ((-50.0, 64.25, 10.0), (200.0, 64.25, 10.0)),   # along +x at low height
        ((60.0, 60.0, 60.0), (10.0, 100.0, 5.0)),       # origin inside the grid
        ((300.0, 300.0, 300.0), (400.0, 400.0, 400.0)),  # looking away: all miss
        ((32.0, -64.0, 40.0), (32.0, 200.0, 40.0)),     # origin on a chunk boundary
    ]
    for o, tg in cases:
        cam = meso.camera(o, tg, 40, 24)
        ocam = oracle.camera(o, tg, 40, 24)
        assert_hits_equal(ctx.raymarch(scene, cam), oracle.raymarch(bm, ocam))


def test_multi_view_equals_per_view(ctx, small):
    t, scene, bm = small
    cams = [meso.camera((-40.0 + 7 * i, -30.0, 140.0 - 3 * i), (64.0, 64.0, 20.0), 48 + 8 * i, 32) for i in range(5)]
    a = ctx.raymarch(scene, cams)
    b = ctx.raymarch(scene, cams, per_view=True)
    assert np.array_equal(a.view(np.uint8), b.view(np.uint8))
    off = 0
    for i, c in enumerate(cams):
        oc = oracle.camera((-40.0 + 7 * i, -30.0, 140.0 - 3 * i), (64.0, 64.0, 20.0), 48 + 8 * i, 32)
        n = c.width * c.height
        assert_hits_equal(a[off:off + n], oracle.raymarch(bm, oc))
        off += n


def test_raymarch_host_entry(ctx, small):
    t, scene, bm = small
    cam = meso.camera((-20.0, 150.0, 90.0), (64.0, 64.0, 10.0), 64, 48)
    ocam = oracle.camera((-20.0, 150.0, 90.0), (64.0, 64.0, 10.0), 64, 48)
    assert_hits_equal(ctx.raymarch_host(scene, cam), oracle.raymarch(bm, ocam))


@pytest.mark.parametrize("w,height", [(40, 1), (40, 389), (40, 1100), (96, 72), (160, 37), (256, 256)])
def test_raymarch_host_pinned_direct(ctx, small, w, height):
    # a page-locked output is written by the kernel directly (no device
    # buffer, no copy); every byte of it must be overwritten.  Widths that
    # are multiples of 32 put four whole tiles side by side in most CTAs,
    # which then write whole 32-pixel rows; the others (and the CTAs of the
    # last, partial tile row) write tile by tile
    t, scene, bm = small
    cam = meso.camera((-20.0, 150.0, 90.0), (64.0, 64.0, 10.0), w, height)
    ocam = oracle.camera((-20.0, 150.0, 90.0), (64.0, 64.0, 10.0), w, height)
    buf = ctx.pinned(w * height * meso.HIT_DTYPE.itemsize)
    buf.view(np.uint8)[:] = 0xAB
    ctx.raymarch_host(scene, cam, out_ptr=buf.ptr)
    got = buf.view(meso.HIT_DTYPE, w * height).copy()
    buf.free()
    assert_hits_equal(got, oracle.raymarch(bm, ocam))


@pytest.fixture(scope="module")
def sparse(ctx):
    # 256 x 192 x 128 voxels (x, y, z), a few boxes: most 32^3 cells empty
    rng = np.random.default_rng(3)
    g = np.zeros((128, 192, 256), np.uint16)  # [z][y][x]
    for _ in range(30):
        c = rng.integers(0, (128, 192, 256))
        r = rng.integers(1, 7, 3)
        g[max(c[0] - r[0], 0):c[0] + r[0], max(c[1] - r[1], 0):c[1] + r[1], max(c[2] - r[2], 0):c[2] + r[2]] = \
            rng.integers(1, 200)
    return ctx.scene_from_dense(g, spare_bricks=4096), oracle.HostBrickMap.from_dense(g)


def test_empty_cell_jumps_match_oracle(ctx, sparse):
    # the timed kernel crosses empty 4x4x4-brick cells in one jump and adds
    # their brick steps arithmetically; hits, t and both step counts must be
    # those of the brick-by-brick walk, including exact ties (the centre ray
    # of the first camera runs along (1,1,1) through cell corners)
    scene, bm = sparse
    poses = [((-64.0, -64.0, -64.0), (64.0, 64.0, 64.0)), ((-32.0, 96.0, 300.0), (96.0, 96.0, 0.0)),
             ((0.0, 0.0, 0.0), (255.0, 191.0, 127.0)), ((128.0, -10.0, 64.0), (128.0, 300.0, 64.0)),
             ((300.0, 250.0, 200.0), (10.0, 20.0, 5.0)), ((32.0, 32.0, 32.0), (33.0, 200.0, 100.0))]
    rng = np.random.default_rng(11)
    for _ in range(10):
        o = rng.uniform(-150, 400, 3)
        poses.append((tuple(o), tuple(rng.uniform(0, (256, 192, 128)))))
    for o, tg in poses:
        cam = meso.camera(o, tg, 48, 40)
        assert_hits_equal(ctx.raymarch(scene, cam), oracle.raymarch(bm, oracle.camera(o, tg, 48, 40)))


def test_empty_cell_map_follows_edits(ctx, sparse):
    # carve whole cells empty and fill empty ones, then render
    scene, bm = sparse
    sp = [((80, 80, 60), 40, 0), ((200, 40, 100), 12, 7), ((20, 150, 20), 9, 300), ((128, 96, 64), 30, 0)]
    scene.edit([meso.SphereEdit((ctypes.c_int32 * 3)(*c), r, m, 0) for c, r, m in sp])
    bm.edit([oracle.Sphere((ctypes.c_int32 * 3)(*c), r, m, 0) for c, r, m in sp])
    for o, tg in [((-64.0, -64.0, -64.0), (128.0, 96.0, 64.0)), ((300.0, 250.0, 200.0), (80.0, 80.0, 60.0))]:
        cam = meso.camera(o, tg, 64, 48)
        assert_hits_equal(ctx.raymarch(scene, cam), oracle.raymarch(bm, oracle.camera(o, tg, 64, 48)))


def test_many_views_of_two_scenes_match_oracle(ctx, small, sparse):
    # 40 views (more than the 32 passed as kernel parameters, so the view
    # table in device memory is used) of two scenes of different sizes in
    # one launch; every view against the oracle of its scene
    t, s_small, bm_small = small
    s_sparse, bm_sparse = sparse
    rng = np.random.default_rng(23)
    scenes, cams, refs = [], [], []
    for i in range(40):
        big = i % 2 == 1
        dims = (256, 192, 128) if big else (128, 128, 128)
        o = tuple(rng.uniform(-120, 380, 3))
        tg = tuple(rng.uniform(0, dims))
        w, h = int(rng.integers(8, 48)), int(rng.integers(8, 40))
        scenes.append(s_sparse if big else s_small)
        cams.append(meso.camera(o, tg, w, h))
        refs.append(oracle.raymarch(bm_sparse if big else bm_small, oracle.camera(o, tg, w, h)))
    got = ctx.raymarch(scenes, cams)
    off = 0
    for c, ref in zip(cams, refs):
        n = c.width * c.height
        assert_hits_equal(got[off:off + n], ref)
        off += n


def test_all_cell_levels_match_oracle(ctx):
    # 1024 x 512 x 1024 terrain below z ~ 300: the 512^3-voxel cells above
    # z = 512 are empty, so rays take jumps of every size (512^3, 128^3 and
    # 32^3 voxels) and brick steps; the oracle walks brick by brick over the
    # same arrays copied back from the device
    t = meso.Terrain(1024, 512, 1024, 21, 256, 6, 40.0, 200.0, 48, 0.7)
    scene = ctx.scene_from_terrain(t)
    ptr, occ, mat = scene.download()
    bm = oracle.HostBrickMap.from_arrays((1024, 512, 1024), ptr, occ, mat)
    poses = [((-200.0, -100.0, 1100.0), (600.0, 300.0, 100.0)), ((512.0, 256.0, 1500.0), (512.0, 257.0, 0.0)),
             ((1300.0, 700.0, 900.0), (-100.0, -50.0, 700.0)), ((10.0, 10.0, 1000.0), (1000.0, 500.0, 20.0)),
             ((-300.0, 256.0, 512.0), (1400.0, 256.0, 512.0))]
    for o, tg in poses:
        cam = meso.camera(o, tg, 64, 48)
        assert_hits_equal(ctx.raymarch(scene, cam), oracle.raymarch(bm, oracle.camera(o, tg, 64, 48)))
    scene.destroy()


def test_matches_golden_fixture(ctx, small):
    import os
    golden = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    t, scene, bm = small
    hits = ctx.raymarch(scene, meso.camera((-40.0, -30.0, 140.0), (64.0, 64.0, 20.0), 96, 64))
    ref = np.load(os.path.join(golden, "hits_terrain128_96x64.npy"))
    assert np.array_equal(hits.view(np.uint8), ref.view(np.uint8))


# The small plain case: the dense 256^3 uint8 value-noise grid (3 octaves,
# seed 1), one 640x360 pinhole camera with a 60 degree vertical field of
# view (the reference's default, Runtimes/Instance/VoxelWindowsInstance.h:22),
# origin outside the grid aimed at its centre, marched to the first hit.
CFG1_ORIGIN, CFG1_TARGET = (-160.0, -96.0, 384.0), (128.0, 128.0, 128.0)


@pytest.fixture(scope="module")
def dense256(ctx):
    d = ctx.generate_dense_u8(256, 256, 256, seed=1)
    host = oracle.gen_dense_u8(256, 256, 256, 1)
    assert np.array_equal(d.download(np.uint8).reshape(256, 256, 256), host)
    scene = ctx.scene_from_grid(meso.SRC_GRID_U8, d, (256, 256, 256))
    bm = oracle.HostBrickMap.from_dense(host.astype(np.uint16))
    return scene, bm, host


def test_grid_u8_scene_build_bit_exact(dense256):
    scene, bm, host = dense256
    ptr, occ, mat = scene.download()
    assert np.array_equal(ptr, bm.ptr())
    assert np.array_equal(occ, bm.occ())
    assert np.array_equal(mat, bm.mat())
    assert np.array_equal(scene.dense(), host.astype(np.uint16))


@pytest.mark.parametrize("shadow", [False, True])
def test_raymarch_dense256_u8_640x360_matches_oracle(ctx, dense256, shadow):
    scene, bm, _ = dense256
    got = ctx.raymarch(scene, meso.camera(CFG1_ORIGIN, CFG1_TARGET, 640, 360), shadow=shadow)
    ref = oracle.raymarch(bm, oracle.camera(CFG1_ORIGIN, CFG1_TARGET, 640, 360), shadow=shadow)
    assert np.isfinite(ref["t"]).sum() > 640 * 360 // 10  # the grid fills about a fifth of the frame
    assert_hits_equal(got, ref)


def test_grid_u16_scene_equals_host_dense(ctx):
    rng = np.random.default_rng(3)
    g = ((rng.random((64, 96, 64)) < 0.1) * rng.integers(1, 65536, (64, 96, 64))).astype(np.uint16)
    d = ctx.to_device(g)
    a = ctx.scene_from_grid(meso.SRC_GRID_U16, d, (64, 96, 64))
    b = ctx.scene_from_dense(g)
    for x, y in zip(a.download(), b.download()):
        assert np.array_equal(x, y)
    with pytest.raises(meso.MesoError):
        ctx.scene_from_grid(meso.SRC_CHUNKS_U16, d, (64, 96, 64))


def test_scene_count_solid(ctx, small):
    t, scene, bm = small
    assert scene.count_solid() == int(np.count_nonzero(bm.dense()))
