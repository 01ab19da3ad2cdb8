"""GPU scene build and raymarching against the CPU oracle.

Hit voxel, face, material, shadow flag and step counts are compared bit for
bit; the hit distance t within 1e-6 relative (it is in fact bit-identical:
both sides evaluate the same sequence of correctly rounded FP32 operations).
"""
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


@pytest.mark.parametrize("height", [1, 389, 1100])
def test_raymarch_host_pinned_direct(ctx, small, height):
    # a page-locked output is written by the kernel directly (no device
    # buffer, no copy); every byte of it must be overwritten
    t, scene, bm = small
    w = 40
    cam = meso.camera((-20.0, 150.0, 90.0), (64.0, 64.0, 10.0), w, height)
    ocam = oracle.camera((-20.0, 150.0, 90.0), (64.0, 64.0, 10.0), w, height)
    buf = ctx.pinned(w * height * meso.HIT_DTYPE.itemsize)
    buf.view(np.uint8)[:] = 0xAB
    ctx.raymarch_host(scene, cam, out_ptr=buf.ptr)
    got = buf.view(meso.HIT_DTYPE, w * height).copy()
    buf.free()
    assert_hits_equal(got, oracle.raymarch(bm, ocam))


def test_matches_golden_fixture(ctx, small):
    import os
    golden = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    t, scene, bm = small
    hits = ctx.raymarch(scene, meso.camera((-40.0, -30.0, 140.0), (64.0, 64.0, 20.0), 96, 64))
    ref = np.load(os.path.join(golden, "hits_terrain128_96x64.npy"))
    assert np.array_equal(hits.view(np.uint8), ref.view(np.uint8))
