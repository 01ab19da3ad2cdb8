"""Serving loop: every result is the same alone and in the mix.

Render requests of different sizes and scenes are batched into shared
launches; edit+remesh+render requests are serialised per scene in arrival
order.  Running the same request list one request at a time (submit, drain)
and all at once must give identical per-request hit hashes, quad hashes and
dirty-chunk counts; the kept hits equal a direct raymarch of the request.
"""
import ctypes

import numpy as np
import pytest

import mesoengine_gb300 as meso

pytestmark = pytest.mark.gpu


def _scenes(ctx):
    a = ctx.scene_from_terrain(meso.terrain_preset("small"), spare_bricks=4096)
    b = ctx.scene_from_terrain(meso.Terrain(256, 256, 128, 21, 128, 6, 10.0, 48.0, 48, 0.7), spare_bricks=4096)
    return [a, b]


def _requests(seed, n=24, edits=True):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        sc = int(rng.integers(0, 2))
        size = [(16, 16), (40, 24), (96, 64), (128, 72)][int(rng.integers(0, 4))]
        o = (float(rng.uniform(-60, -10)), float(rng.uniform(-60, 60)), float(rng.uniform(90, 160)))
        tg = (float(rng.uniform(40, 90)), float(rng.uniform(40, 90)), float(rng.uniform(0, 30)))
        ed = None
        if edits and rng.random() < 0.3:
            ed = []
            for _ in range(int(rng.integers(1, 6))):
                c = (ctypes.c_int32 * 3)(*[int(v) for v in rng.integers(0, 120, 3)])
                m = 0 if rng.random() < 0.5 else int(rng.integers(1, 65535))
                ed.append(meso.SphereEdit(c, int(rng.integers(2, 12)), m, 0))
        out.append((sc, meso.camera(o, tg, *size), bool(rng.random() < 0.5), ed))
    return out


def _run(ctx, reqs, one_by_one, keep_hits=False):
    scenes = _scenes(ctx)
    srv = meso.Server(ctx, scenes, max_inflight_batches=3, max_batch_rays=1 << 20, keep_hits=int(keep_hits),
                      max_edit_quads=1 << 20)
    res = {}
    ids = []
    for i, (sc, cam, shadow, ed) in enumerate(reqs):
        ids.append(srv.submit(sc, cam, shadow=shadow, edits=ed, tag=i))
        if one_by_one:
            srv.drain()
    srv.drain()
    for c in srv.poll():
        res[c.user_tag] = c
    hits = {}
    if keep_hits:
        for i, rid in enumerate(ids):
            cam = reqs[i][1]
            hits[i] = srv.fetch_hits(rid, cam.width * cam.height)
    srv.close()
    return res, hits


def test_render_results_equal_alone_and_in_mix(ctx):
    reqs = _requests(1, edits=False)
    alone, _ = _run(ctx, reqs, True)
    mix, hits = _run(ctx, reqs, False, keep_hits=True)
    scenes = _scenes(ctx)
    for i, (sc, cam, shadow, _) in enumerate(reqs):
        assert alone[i].status == 0 and mix[i].status == 0
        assert alone[i].hit_checksum == mix[i].hit_checksum
        direct = ctx.raymarch(scenes[sc], cam, shadow=shadow)
        assert np.array_equal(hits[i].view(np.uint8), direct.view(np.uint8))
        assert mix[i].hit_checksum == meso.hit_checksum(direct)
        assert mix[i].n_rays == cam.width * cam.height + np.count_nonzero(direct["shadow_steps"])


def test_delivery_to_every_destination_kind(ctx):
    """Delivered hits and their checksums do not depend on where they go.
    The raymarch kernel stores a request's hits straight into device memory
    or device-mapped page-locked host memory (aligned to 8 bytes); any other
    destination (pageable host memory, an address off the 8-byte grid) gets
    a copy from the batch buffer.  Batches mix all kinds; every delivered
    buffer equals a direct raymarch, bit for bit, and every completion's
    checksum and ray count equal the host hash of those hits."""
    reqs = _requests(5, n=30, edits=False)
    scenes = _scenes(ctx)
    srv = meso.Server(ctx, scenes, max_inflight_batches=2, max_batch_rays=1 << 20)
    keep, dsts = [], []
    for i, (sc, cam, shadow, _) in enumerate(reqs):
        nb = cam.width * cam.height * 24
        kind = i % 6
        if kind in (0, 1):  # device memory, at 0 and 8 bytes into an allocation
            b = ctx.alloc(nb + 16)
            ptr = b.ptr + 8 * kind
            read = (lambda b=b, k=kind, nb=nb: b.download(np.uint8, nb + 8 * k)[8 * k:])
        elif kind in (2, 3, 4):  # page-locked host memory at 0, 8 and 4 bytes in
            b = ctx.pinned(nb + 16)
            off = (0, 8, 4)[kind - 2]
            ptr = b.ptr + off
            read = (lambda b=b, o=off, nb=nb: b.view(np.uint8, nb + o)[o:].copy())
        else:  # pageable host memory
            b = np.zeros(nb + 16, np.uint8)
            ptr = b.ctypes.data
            read = (lambda b=b, nb=nb: b[:nb].copy())
        keep.append(b)
        dsts.append(read)
        srv.submit(sc, cam, shadow=shadow, tag=i, dst=ptr)
    srv.drain()
    comp = {c.user_tag: c for c in srv.poll()}
    srv.close()
    for i, (sc, cam, shadow, _) in enumerate(reqs):
        c = comp[i]
        assert c.status == 0
        direct = ctx.raymarch(scenes[sc], cam, shadow=shadow)
        got = dsts[i]()
        assert np.array_equal(got, direct.view(np.uint8).reshape(-1)), f"request {i} (kind {i % 6})"
        assert c.hit_checksum == meso.hit_checksum(direct)
        assert c.n_rays == cam.width * cam.height + np.count_nonzero(direct["shadow_steps"])


def test_edits_serialised_per_scene(ctx):
    reqs = _requests(2)
    assert any(r[3] for r in reqs)
    alone, _ = _run(ctx, reqs, True)
    mix, _ = _run(ctx, reqs, False)
    for i, r in enumerate(reqs):
        a, m = alone[i], mix[i]
        assert a.status == 0 and m.status == 0, (a.status, m.status)
        assert (a.hit_checksum, a.quad_checksum, a.n_quads, a.n_dirty_chunks) == \
               (m.hit_checksum, m.quad_checksum, m.n_quads, m.n_dirty_chunks)
        if r[3]:
            assert m.n_dirty_chunks > 0


def test_admission_rejects_oversize_and_overflowing_queue(ctx):
    scenes = _scenes(ctx)
    srv = meso.Server(ctx, scenes, max_inflight_batches=1, max_batch_requests=1, max_batch_rays=64 * 64,
                      max_queue=2)
    big = srv.submit(0, meso.camera((-40.0, -30.0, 140.0), (64.0, 64.0, 20.0), 128, 128))
    cam = meso.camera((-40.0, -30.0, 140.0), (64.0, 64.0, 20.0), 64, 64)
    ids = [srv.submit(0, cam, shadow=True) for _ in range(400)]
    srv.drain()
    comp = {c.request_id: c for c in srv.poll()}
    srv.close()
    assert comp[big].status == 3  # MESO_ERR_OVER_BUDGET: can never fit a slot
    st = [comp[i].status for i in ids]
    assert st.count(0) >= 2 and st.count(3) >= 1 and set(st) <= {0, 3}
    for i in ids:
        c = comp[i]
        assert c.done_s >= c.submit_s


def _oracle_terrain(t):
    import oracle
    return oracle.terrain(t.nx, t.ny, t.nz, t.seed, t.height_period, t.height_octaves, t.height_base,
                          t.height_amp, t.cave_period, t.cave_threshold)


def test_served_edits_equal_oracle_replay(ctx):
    """The served edit path -- sphere edits, the forked remesh and render,
    the mesh store update, delivery into caller-owned buffers -- against a
    sequential replay on the oracle: every delivered render equals the
    oracle's raymarch of the scene as of that request (bit for bit), every
    remesh's dirty count and quad hash equal the oracle's, and the server's
    mesh store ends equal to the oracle's mesh of the final scene."""
    import oracle
    t = meso.terrain_preset("small")
    scene = ctx.scene_from_terrain(t, spare_bricks=8192)
    bm = oracle.HostBrickMap.from_terrain(_oracle_terrain(t))
    reqs = [r for r in _requests(31, n=40) if r[0] == 0]
    assert sum(1 for r in reqs if r[3]) >= 3
    srv = meso.Server(ctx, [scene], max_inflight_batches=3, max_batch_rays=1 << 20, max_edit_quads=1 << 20,
                      keep_meshes=1)
    outs, ids = [], []
    for i, (_, cam, shadow, ed) in enumerate(reqs):
        outs.append(ctx.alloc(cam.width * cam.height * 24))
        ids.append(srv.submit(0, cam, shadow=shadow, edits=ed, tag=i, dst=outs[-1]))
    srv.drain()
    comp = {c.user_tag: c for c in srv.poll()}
    cx = t.nx // 32
    for i, (_, cam, shadow, ed) in enumerate(reqs):
        c = comp[i]
        assert c.status == 0
        if ed:
            sp = [oracle.Sphere((ctypes.c_int32 * 3)(*e.center), e.radius, e.material, 0) for e in ed]
            dirty = bm.dirty_chunks(sp)
            bm.edit(sp)
            assert c.n_dirty_chunks == len(dirty)
            coords = np.stack([dirty % cx, (dirty // cx) % cx, dirty // (cx * cx)], 1).astype(np.int32)
            q = oracle.mesh_chunks(oracle.SRC_BRICKMAP, coords=coords, bm=bm)
            assert c.n_quads == len(q) and c.quad_checksum == meso.quad_checksum(q)
        ref = oracle.raymarch(bm, _oracle_cam(cam), shadow=shadow)
        got = outs[i].download(meso.HIT_DTYPE, cam.width * cam.height)
        assert np.array_equal(got.view(np.uint8), ref.view(np.uint8)), f"request {i}"
    n = (t.nx // 32) * (t.ny // 32) * (t.nz // 32)
    idx = np.arange(n)
    coords = np.stack([idx % cx, (idx // cx) % cx, idx // (cx * cx)], 1).astype(np.int32)
    got = np.sort(srv.store(0).gather(idx))
    assert np.array_equal(got, oracle.mesh_chunks(oracle.SRC_BRICKMAP, coords=coords, bm=bm))
    srv.close()


def _oracle_cam(cam):
    """The oracle's camera with the same fields as a meso camera."""
    import oracle
    return oracle.Camera.from_buffer_copy(bytes(cam))  # the two structs share one layout


def test_served_store_repaired_after_overflow(ctx):
    """An edit whose remesh overflows the server's quad buffer (max_edit_quads
    far too small) reports MESO_ERR_OVERFLOW for its quad count, and its
    placement into the mesh store fails on the device; the server places
    those chunks again before the scene's next request, so the store still
    equals the oracle's mesh of the edited scene."""
    import oracle
    t = meso.terrain_preset("small")
    scene = ctx.scene_from_terrain(t, spare_bricks=8192)
    bm = oracle.HostBrickMap.from_terrain(_oracle_terrain(t))
    srv = meso.Server(ctx, [scene], max_inflight_batches=2, max_batch_rays=1 << 16, max_edit_quads=256,
                      keep_meshes=1)
    cam = meso.camera((-40.0, -30.0, 140.0), (64.0, 64.0, 20.0), 32, 24)
    eds = []
    for k in range(3):
        ed = [meso.SphereEdit((ctypes.c_int32 * 3)(20 + 40 * k, 60, 30), 14, 0 if k == 1 else 700 + k, 0),
              meso.SphereEdit((ctypes.c_int32 * 3)(90, 20 + 30 * k, 25), 9, 1234 + k, 0)]
        eds.append(ed)
        srv.submit(0, cam, edits=ed, tag=k)
    srv.drain()
    comp = {c.user_tag: c for c in srv.poll()}
    assert any(c.status == 4 for c in comp.values())  # MESO_ERR_OVERFLOW: the remesh did not fit 256 quads
    for ed in eds:
        bm.edit([oracle.Sphere((ctypes.c_int32 * 3)(*e.center), e.radius, e.material, 0) for e in ed])
    cx = t.nx // 32
    idx = np.arange((t.nx // 32) * (t.ny // 32) * (t.nz // 32))
    coords = np.stack([idx % cx, (idx // cx) % cx, idx // (cx * cx)], 1).astype(np.int32)
    assert np.array_equal(np.sort(srv.store(0).gather(idx)),
                          oracle.mesh_chunks(oracle.SRC_BRICKMAP, coords=coords, bm=bm))
    srv.close()


def test_served_stores_of_two_scenes(ctx):
    """keep_meshes with two resident scenes: edits of either scene, mixed in
    one stream, leave each scene's store equal to the oracle's mesh of that
    scene after its own edits."""
    import oracle
    scenes = _scenes(ctx)
    presets = [meso.terrain_preset("small"), meso.Terrain(256, 256, 128, 21, 128, 6, 10.0, 48.0, 48, 0.7)]
    bms = [oracle.HostBrickMap.from_terrain(_oracle_terrain(t)) for t in presets]
    reqs = _requests(44, n=30)
    srv = meso.Server(ctx, scenes, max_inflight_batches=3, max_batch_rays=1 << 20, max_edit_quads=1 << 20,
                      keep_meshes=1)
    for i, (sc, cam, shadow, ed) in enumerate(reqs):
        srv.submit(sc, cam, shadow=shadow, edits=ed, tag=i)
        if ed:
            bms[sc].edit([oracle.Sphere((ctypes.c_int32 * 3)(*e.center), e.radius, e.material, 0) for e in ed])
    srv.drain()
    assert all(c.status == 0 for c in srv.poll())
    assert sum(1 for r in reqs if r[3] and r[0] == 0) > 0 and sum(1 for r in reqs if r[3] and r[0] == 1) > 0
    for k, t in enumerate(presets):
        cx, cy, cz = t.nx // 32, t.ny // 32, t.nz // 32
        idx = np.arange(cx * cy * cz)
        coords = np.stack([idx % cx, (idx // cx) % cy, idx // (cx * cy)], 1).astype(np.int32)
        assert np.array_equal(np.sort(srv.store(k).gather(idx)),
                              oracle.mesh_chunks(oracle.SRC_BRICKMAP, coords=coords, bm=bms[k]))
    srv.close()
