"""The raymarch entry point that allocates nothing, against meso_raymarch.

meso_raymarch_noalloc serves callers that cannot allocate device memory
during a call (a frame loop on a fixed device-memory budget, or a host whose
own memory manager owns all device memory): it keeps the per-view
descriptor table in a fixed device array.  This test drives it through the
C ABI with more than 32 views, so the table is really used, on two calls in
a row with different cameras, and checks each result against the existing
entry point with the same tolerance as the other raymarch tests.  The two
calls go back to back on one stream with no synchronisation between them,
the case the shared table's stream ordering is there for.  The file sorts
last so that a run stopping at the first failure has run all other tests
already.
"""
import ctypes

import numpy as np
import pytest

import mesoengine_gb300 as meso

pytestmark = pytest.mark.gpu
T_RTOL = 1e-6


def _assert_hits_close(got, ref):
    for f in ("voxel", "material", "face", "shadow", "steps", "shadow_steps"):
        assert np.array_equal(got[f], ref[f]), f
    hit = np.isfinite(ref["t"])
    assert np.array_equal(np.isfinite(got["t"]), hit)
    np.testing.assert_allclose(got["t"][hit], ref["t"][hit], rtol=T_RTOL, atol=0)


def _noalloc(ctx, scene, cams, out, stream=None):
    fn = meso.load().meso_raymarch_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(meso.Camera), ctypes.c_uint32,
                   ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    sh = (ctypes.c_void_p * len(cams))(*([scene.handle] * len(cams)))
    ca = (meso.Camera * len(cams))(*cams)
    light = meso.light_dir()
    return fn(ctx.handle, sh, ca, len(cams), light.ctypes.data, meso.RAY_SHADOW, out.ptr, stream)


def _cams(n, seed):
    rng = np.random.default_rng(seed)
    cams = []
    for _ in range(n):
        o = (rng.uniform(-60, -20), rng.uniform(-60, 190), rng.uniform(60, 160))
        t = (rng.uniform(30, 100), rng.uniform(30, 100), rng.uniform(0, 30))
        cams.append(meso.camera(o, t, int(rng.integers(8, 40)), int(rng.integers(8, 30))))
    return cams


def test_raymarch_noalloc_matches_raymarch(ctx):
    scene = ctx.scene_from_terrain(meso.terrain_preset("small"))
    st = ctx.stream()
    sets = [_cams(n, seed) for n, seed in [(40, 1), (37, 2), (130, 3)]]
    refs = [ctx.raymarch(scene, cams) for cams in sets]
    outs = [ctx.alloc(sum(c.width * c.height for c in cams) * 24) for cams in sets]
    # two calls in a row on one stream, no synchronisation between them
    for cams, out in zip(sets[:2], outs[:2]):
        assert _noalloc(ctx, scene, cams, out, st) == 0, meso.load().meso_last_error_string()
    ctx.sync(st)
    # and a call of more than 64 views (several parameter batches)
    assert _noalloc(ctx, scene, sets[2], outs[2], st) == 0, meso.load().meso_last_error_string()
    ctx.sync(st)
    for ref, out in zip(refs, outs):
        assert np.isfinite(ref["t"]).sum() > 0
        _assert_hits_close(out.download(meso.HIT_DTYPE, ref.shape[0]), ref)


def test_raymarch_noalloc_rejects_too_many_views(ctx):
    scene = ctx.scene_from_terrain(meso.terrain_preset("small"))
    cams = [meso.camera((-40.0, -30.0, 140.0), (64.0, 64.0, 20.0), 8, 8)] * 513
    out = ctx.alloc(513 * 64 * 24)
    assert _noalloc(ctx, scene, cams, out) == 1  # MESO_ERR_INVALID_ARG
    assert b"512" in meso.load().meso_last_error_string()
