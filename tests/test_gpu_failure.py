"""The device failure path without a device fault: a bounded wait that cannot
succeed gives up, the host reads MESO_ERR_TIMEOUT, and the context keeps
working (meshing and raymarching still match the oracle)."""
import time

import numpy as np
import pytest

import oracle
import mesoengine_gb300 as meso

pytestmark = pytest.mark.gpu

TIMEOUT = 5  # MESO_ERR_TIMEOUT


@pytest.mark.parametrize("limit_us", [2000, 100000])
def test_bounded_wait_gives_up_and_context_stays_usable(ctx, limit_us):
    t0 = time.perf_counter()
    with pytest.raises(meso.MesoError) as e:
        ctx.selftest_bounded_wait(limit_us)
    dt = time.perf_counter() - t0
    assert e.value.status == TIMEOUT
    assert dt >= limit_us * 1e-6 * 0.9
    assert dt < limit_us * 1e-6 + 5.0
    # the flag was consumed: the next sync is clean
    ctx.sync()
    # and the context still meshes and raymarches correctly
    data, _ = ctx.generate_chunks_u16(4, seed0=7)
    q, _ = ctx.mesh(meso.SRC_CHUNKS_U16, data, n=4)
    host = data.download(np.uint16).reshape(4, 32, 32, 32)
    assert np.array_equal(np.sort(q), oracle.mesh_chunks(oracle.SRC_CHUNKS_U16, host))
    g = np.zeros((64, 64, 64), np.uint16)
    g[10:30, 20:40, 5:50] = 3
    scene = ctx.scene_from_dense(g)
    cam = meso.camera((-40.0, -30.0, 90.0), (32.0, 32.0, 20.0), 32, 24)
    got = ctx.raymarch(scene, cam)
    ref = oracle.raymarch(oracle.HostBrickMap.from_dense(g), oracle.camera((-40.0, -30.0, 90.0), (32.0, 32.0, 20.0), 32, 24))
    assert np.array_equal(got.view(np.uint8), ref.view(np.uint8))


def test_bounded_wait_rejects_bad_limits(ctx):
    for bad in (0, 2_000_000):
        with pytest.raises(meso.MesoError) as e:
            ctx.selftest_bounded_wait(bad)
        assert e.value.status == 1  # MESO_ERR_INVALID_ARG
