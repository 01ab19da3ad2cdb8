"""The autotuner: it writes its choice as JSON, a new context reads it back
through meso_config.tuning_path, and the tuned context's quads and hits are
still bit-exact against the oracle."""
import json

import numpy as np
import pytest

import oracle
import mesoengine_gb300 as meso

pytestmark = pytest.mark.gpu


def test_autotune_roundtrip_and_parity(tmp_path):
    path = str(tmp_path / "tuning.json")
    a = meso.Context(0)
    try:
        a.autotune(path)
        tuned = a.config()
    finally:
        a.close()
    with open(path) as f:
        j = json.load(f)
    assert j["ray_tile_w"] in (4, 8, 16, 32) and j["ray_warps_per_cta"] in (1, 2, 4)
    assert j["mesh_ctas_per_sm"] in (1, 2) and j["mesh_chunks_per_ticket"] in (1, 2, 4)
    assert j["ray_ms_1280x720"] > 0 and j["mesh_ms_1024_chunks"] > 0
    for k in ("ray_tile_w", "ray_warps_per_cta", "mesh_ctas_per_sm", "mesh_chunks_per_ticket"):
        assert tuned[k] == j[k], k
    ctx = meso.Context(0, tuning_path=path)
    try:
        got = ctx.config()
        for k in ("ray_tile_w", "ray_warps_per_cta", "mesh_ctas_per_sm", "mesh_chunks_per_ticket"):
            assert got[k] == j[k], k
        assert got["ray_tile_h"] * got["ray_tile_w"] == 32
        # meshing on the tuned context
        dev, _ = ctx.generate_chunks_u16(64, seed0=7)
        host, _ = oracle.gen_chunks_u16(64, 7)
        q, _ = ctx.mesh(meso.SRC_CHUNKS_U16, dev, n=64)
        assert np.array_equal(np.sort(q), oracle.mesh_chunks(oracle.SRC_CHUNKS_U16, host))
        # raymarching on the tuned context
        t = meso.terrain_preset("small")
        scene = ctx.scene_from_terrain(t)
        bm = oracle.HostBrickMap.from_terrain(
            oracle.terrain(t.nx, t.ny, t.nz, t.seed, t.height_period, t.height_octaves, t.height_base,
                           t.height_amp, t.cave_period, t.cave_threshold))
        cam = ((-40.0, -30.0, 140.0), (64.0, 64.0, 20.0), 100, 60)
        hits = ctx.raymarch(scene, meso.camera(*cam))
        ref = oracle.raymarch(bm, oracle.camera(*cam))
        assert np.array_equal(hits.view(np.uint8), ref.view(np.uint8))
        scene.destroy()
    finally:
        ctx.close()


def test_explicit_config_overrides_tuning_file(tmp_path):
    path = tmp_path / "t.json"
    path.write_text(json.dumps({"ray_tile_w": 16, "ray_warps_per_cta": 2, "mesh_ctas_per_sm": 1,
                                "mesh_chunks_per_ticket": 4}))
    ctx = meso.Context(0, tuning_path=str(path), ray_tile_w=4)
    try:
        c = ctx.config()
        assert (c["ray_tile_w"], c["ray_tile_h"], c["ray_warps_per_cta"]) == (4, 8, 2)
        assert (c["mesh_ctas_per_sm"], c["mesh_chunks_per_ticket"]) == (1, 4)
    finally:
        ctx.close()
