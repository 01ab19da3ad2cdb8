"""GPU greedy meshing against the CPU oracle (bit-exact after canonical sort).

Quads are packed uint64 whose numeric order is the canonical
(chunk, dir, z, y, x) order, so parity is np.sort(gpu) == oracle.
"""
import numpy as np
import pytest

import oracle
import mesoengine_gb300 as meso

pytestmark = pytest.mark.gpu


def _sorted(q):
    return np.sort(np.asarray(q, dtype=np.uint64))


def _kat_chunks():
    c = np.zeros((6, 32, 32, 32), np.uint16)
    c[0, 5, 6, 7] = 3                                  # single voxel -> 6 unit quads
    c[1] = 9                                           # full chunk -> 6 quads of 32x32
    z, y, x = np.indices((32, 32, 32))
    c[2] = ((x + y + z) % 2 == 0) * 1                  # checkerboard -> no merges
    c[3] = (x // 4 % 3 + 1) * (z < 20)                 # material stripes
    c[4, :, :, 31] = 7                                 # wall on the +x border
    c[5] = np.where((x * 7 + y * 13 + z * 5) % 11 < 5, (x + y) % 3 + 1, 0)
    return c


def test_kat_chunks_u16(ctx):
    c = _kat_chunks()
    ref = oracle.mesh_chunks(oracle.SRC_CHUNKS_U16, c)
    q, counts = ctx.mesh(meso.SRC_CHUNKS_U16, ctx.to_device(c), n=c.shape[0], chunk_counts=True)
    assert np.array_equal(_sorted(q), ref)
    per = np.bincount(oracle.unpack_quads(ref)["chunk"], minlength=c.shape[0])
    assert np.array_equal(counts, per)
    assert per[0] == 6 and per[1] == 6 and per[2] == 6 * 16384


def _component_chunks():
    """Patterns built to exercise the order-independent peeling: isolated
    faces, two-face components (dominoes, both orientations), L- and
    T-shaped three- and four-face components, long runs, and the extreme
    material values 1 and 65535."""
    rng = np.random.default_rng(77)
    z, y, x = np.indices((32, 32, 32))
    c = np.zeros((12, 32, 32, 32), np.uint16)
    # dominoes along x and along y on a sparse lattice, distinct materials
    c[0] = np.where((x % 4 < 2) & (y % 3 == 0) & (z % 3 == 0), 1 + (x // 4 + 7 * y + 31 * z) % 60000, 0)
    c[1] = np.where((y % 4 < 2) & (x % 3 == 0) & (z % 3 == 0), 1 + (y // 4 + 7 * x + 31 * z) % 60000, 0)
    # vertical dominoes (two voxels along z) and L-shapes
    c[2] = np.where((z % 4 < 2) & (x % 3 == 0) & (y % 3 == 0), 65535, 0)
    c[3] = np.where(((x % 5 == 0) & (y % 5 < 2) | (x % 5 < 2) & (y % 5 == 0)) & (z % 4 == 1), 5, 0)
    # random materials from a small palette on random occupancy
    for k, (p, m) in enumerate([(0.05, 2), (0.3, 2), (0.6, 3), (0.9, 1)]):
        occ = rng.random((32, 32, 32)) < p
        c[4 + k] = np.where(occ, rng.integers(1, m + 1, (32, 32, 32)), 0)
    # full slabs with a stripe of another material, and a hollow box
    c[8] = np.where(z < 16, 1 + (x == 10) * 65534, 0)
    c[9] = np.where((x > 2) & (x < 29) & (y > 2) & (y < 29) & (z > 2) & (z < 29), 4, 0)
    c[9][5:27, 5:27, 5:27] = 0
    # alternating 2-wide bands (domino-rich) and a sparse mix of everything
    c[10] = np.where(((x // 2 + y // 2 + z) % 2 == 0), 1 + ((x // 2) % 2), 0)
    c[11] = np.where(rng.random((32, 32, 32)) < 0.15, rng.integers(1, 65536, (32, 32, 32)), 0)
    return c


def test_component_patterns_match_oracle(ctx):
    c = _component_chunks()
    ref = oracle.mesh_chunks(oracle.SRC_CHUNKS_U16, c)
    q, counts = ctx.mesh(meso.SRC_CHUNKS_U16, ctx.to_device(c), n=c.shape[0], chunk_counts=True)
    assert np.array_equal(_sorted(q), ref)
    assert np.array_equal(counts, np.bincount(oracle.unpack_quads(ref)["chunk"], minlength=c.shape[0]))
    # the same chunks through the uint8 path (materials folded into 1..255)
    c8 = np.where(c > 0, 1 + (c.astype(np.uint32) % 255), 0).astype(np.uint8)
    q8, _ = ctx.mesh(meso.SRC_CHUNKS_U8, ctx.to_device(c8), n=c8.shape[0])
    assert np.array_equal(_sorted(q8), oracle.mesh_chunks(oracle.SRC_CHUNKS_U8, c8))


def test_ctas_per_sm_settings_agree():
    # one or two persistent 16-warp CTAs per SM give the same quads
    c16 = _component_chunks()[:8]
    c8 = np.where(c16 > 0, 1 + (c16.astype(np.uint32) % 255), 0).astype(np.uint8)
    ref16 = oracle.mesh_chunks(oracle.SRC_CHUNKS_U16, c16)
    ref8 = oracle.mesh_chunks(oracle.SRC_CHUNKS_U8, c8)
    for cps in (1, 2):
        cx = meso.Context(0, mesh_ctas_per_sm=cps)
        try:
            d16, d8 = cx.to_device(c16), cx.to_device(c8)
            q16, _ = cx.mesh(meso.SRC_CHUNKS_U16, d16, n=c16.shape[0])
            q8, _ = cx.mesh(meso.SRC_CHUNKS_U8, d8, n=c8.shape[0])
            d16.free()
            d8.free()
            assert np.array_equal(_sorted(q16), ref16)
            assert np.array_equal(_sorted(q8), ref8)
        finally:
            cx.close()
    with pytest.raises(meso.MesoError) as e:
        meso.Context(0, mesh_ctas_per_sm=3)
    assert e.value.status == 1


def test_generated_chunks_match_oracle(ctx):
    n = 48
    dev, solid = ctx.generate_chunks_u16(n, seed0=1)
    host, hsolid = oracle.gen_chunks_u16(n, 1)
    got = dev.download(np.uint16).reshape(n, 32, 32, 32)
    assert np.array_equal(got, host)
    assert np.array_equal(solid.download(np.uint32), hsolid)
    assert np.array_equal((host > 0).reshape(n, -1).sum(1), hsolid)


def test_chunks_u16_batched_and_per_launch(ctx):
    n = 64
    dev, _ = ctx.generate_chunks_u16(n, seed0=101)
    host = dev.download(np.uint16).reshape(n, 32, 32, 32)
    ref = oracle.mesh_chunks(oracle.SRC_CHUNKS_U16, host)
    q1, _ = ctx.mesh(meso.SRC_CHUNKS_U16, dev, n=n)
    q2, _ = ctx.mesh(meso.SRC_CHUNKS_U16, dev, n=n, per_launch=True)
    assert np.array_equal(_sorted(q1), ref)
    assert np.array_equal(_sorted(q2), ref)


def test_chunk_index_list(ctx):
    n = 16
    dev, _ = ctx.generate_chunks_u16(n, seed0=7)
    host = dev.download(np.uint16).reshape(n, 32, 32, 32)
    order = np.array([5, 3, 3, 15, 0], dtype=np.int32)
    ref = oracle.mesh_chunks(oracle.SRC_CHUNKS_U16, host[order])
    q, _ = ctx.mesh(meso.SRC_CHUNKS_U16, dev, coords=order.reshape(-1, 1))
    assert np.array_equal(_sorted(q), ref)


def test_dense_u8_grid_with_neighbours(ctx):
    # the small plain case: 256^3 uint8, 512 chunks, faces see across chunks
    g_dev = ctx.generate_dense_u8(256, 256, 256, seed=1)
    grid = g_dev.download(np.uint8).reshape(256, 256, 256)
    assert np.array_equal(grid, oracle.gen_dense_u8(256, 256, 256, 1))
    coords = np.array([(x, y, z) for z in range(8) for y in range(8) for x in range(8)], dtype=np.int32)
    ref = oracle.mesh_chunks(oracle.SRC_GRID_U8, grid, coords=coords)
    q, _ = ctx.mesh(meso.SRC_GRID_U8, g_dev, coords=coords, dims=(256, 256, 256))
    assert np.array_equal(_sorted(q), ref)


def test_dense_u16_grid(ctx):
    rng = np.random.default_rng(3)
    g = (rng.random((64, 96, 64)) < 0.3) * rng.integers(1, 4, (64, 96, 64))
    g = g.astype(np.uint16)
    coords = np.array([(x, y, z) for z in range(2) for y in range(3) for x in range(2)], dtype=np.int32)
    ref = oracle.mesh_chunks(oracle.SRC_GRID_U16, g, coords=coords)
    q, _ = ctx.mesh(meso.SRC_GRID_U16, ctx.to_device(g), coords=coords, dims=(64, 96, 64))
    assert np.array_equal(_sorted(q), ref)


def test_overflow_reports_need(ctx):
    c = _kat_chunks()[2:3]  # checkerboard: 98304 quads
    with pytest.raises(meso.MesoError) as e:
        ctx.mesh(meso.SRC_CHUNKS_U16, ctx.to_device(c), n=1, capacity=1000)
    assert e.value.status == 4
    q, _ = ctx.mesh(meso.SRC_CHUNKS_U16, ctx.to_device(c), n=1, capacity=1000, check=False)
    assert len(q) == 1000


def test_empty_input(ctx):
    c = np.zeros((3, 32, 32, 32), np.uint16)
    q, counts = ctx.mesh(meso.SRC_CHUNKS_U16, ctx.to_device(c), n=3, chunk_counts=True)
    assert len(q) == 0 and counts.tolist() == [0, 0, 0]
    q0, _ = ctx.mesh(meso.SRC_CHUNKS_U16, ctx.to_device(c), n=0)
    assert len(q0) == 0


def test_mesh_host_entry(ctx):
    c = _kat_chunks()
    ref = oracle.mesh_chunks(oracle.SRC_CHUNKS_U16, c)
    q = ctx.mesh_host(meso.SRC_CHUNKS_U16, c)
    assert np.array_equal(_sorted(q), ref)


def test_mesh_host_slices(ctx):
    """A host chunk array longer than one slice (1024 chunks) is meshed in
    slices whose uploads overlap the previous slice's launch; the quads carry
    the chunks' indices in the whole array and equal the one-launch device
    path's, with the output in pageable memory (copied back at the end) and
    in page-locked memory (written by the kernel), for uint16 and uint8
    chunks; a buffer too small reports the count it needed."""
    import ctypes
    n = 1300
    dev, _ = ctx.generate_chunks_u16(n, seed0=7)
    host16 = dev.download(np.uint16, n * 32768).reshape(n, 32, 32, 32)
    ref16, _ = ctx.mesh(meso.SRC_CHUNKS_U16, dev, n=n)
    ref16 = _sorted(ref16)
    assert np.array_equal(_sorted(ctx.mesh_host(meso.SRC_CHUNKS_U16, host16)), ref16)
    cap = len(ref16) + 100
    pin = ctx.pinned(cap * 8)
    total = ctypes.c_uint64()
    meso._check(meso._lib.meso_mesh_host(ctx.handle, meso.SRC_CHUNKS_U16, host16.ctypes.data, n, 0, 0, None, n,
                                         pin.ptr, cap, ctypes.byref(total)))
    assert total.value == len(ref16)
    assert np.array_equal(np.sort(pin.view(np.uint64, total.value)), ref16)
    pin.free()
    host8 = (host16 % 251).astype(np.uint8)
    d8 = ctx.to_device(host8)
    ref8, _ = ctx.mesh(meso.SRC_CHUNKS_U8, d8, n=n)
    assert np.array_equal(_sorted(ctx.mesh_host(meso.SRC_CHUNKS_U8, host8)), _sorted(ref8))
    small = np.empty(1000, dtype=np.uint64)
    rc = meso._lib.meso_mesh_host(ctx.handle, meso.SRC_CHUNKS_U16, host16.ctypes.data, n, 0, 0, None, n,
                                  small.ctypes.data, 1000, ctypes.byref(total))
    assert rc == 4 and total.value == len(ref16)  # MESO_ERR_OVERFLOW with the count needed


def test_brickmap_chunks(ctx):
    t = meso.terrain_preset("small")
    scene = ctx.scene_from_terrain(t)
    dense = scene.dense()
    bm = oracle.HostBrickMap.from_dense(dense)
    coords = np.array([(x, y, z) for z in range(4) for y in range(4) for x in range(4)], dtype=np.int32)
    ref = oracle.mesh_chunks(oracle.SRC_BRICKMAP, coords=coords, bm=bm)
    q, _ = ctx.mesh(meso.SRC_BRICKMAP, coords=coords, scene=scene)
    assert len(ref) > 0
    assert np.array_equal(_sorted(q), ref)


def test_brickmap_counts_with_empty_repeated_and_bad_chunks(ctx):
    """A short list (one chunk per queue ticket): empty chunks get count 0
    without being meshed, repeated chunks are meshed again, and an
    out-of-range coordinate gets count 0 and raises the invalid-argument
    flag."""
    t = meso.terrain_preset("small")
    scene = ctx.scene_from_terrain(t)
    bm = oracle.HostBrickMap.from_dense(scene.dense())
    allc = [(x, y, z) for z in range(4) for y in range(4) for x in range(4)]
    rng = np.random.default_rng(5)
    good = [allc[i] for i in rng.integers(0, 64, 90)] + allc  # > 32, with repeats and empty chunks
    coords = np.array(good + [(9, 0, 0)] + good[:7], dtype=np.int32)
    with pytest.raises(meso.MesoError, match="outside"):
        ctx.mesh(meso.SRC_BRICKMAP, coords=coords, scene=scene)
    q, counts = ctx.mesh(meso.SRC_BRICKMAP, coords=coords, scene=scene, chunk_counts=True, check=False)
    ok = np.array([i for i in range(len(coords)) if i != len(good)])
    ref = oracle.mesh_chunks(oracle.SRC_BRICKMAP, coords=coords[ok], bm=bm)
    ref_counts = np.bincount((ref >> np.uint64(44)).astype(np.int64), minlength=len(ok))
    assert counts[len(good)] == 0
    assert np.array_equal(counts[ok], ref_counts)
    # quads carry the index in the call: map the oracle's indices back
    chunk = (ref >> np.uint64(44)).astype(np.int64)
    remapped = (ref & np.uint64((1 << 44) - 1)) | (ok[chunk].astype(np.uint64) << np.uint64(44))
    assert np.array_equal(_sorted(q), np.sort(remapped))
    assert (counts == 0).sum() > 1  # empty chunks among them


def test_brickmap_long_list_tickets(ctx):
    """A list long enough that every CTA takes several list entries per
    ticket (through a stride permutation of the list) and tests them
    together against the scene's per-chunk cell map: 3,000 entries with
    every chunk of the scene many times over, air chunks among them, and two
    out-of-range coordinates.  Quads, per-entry counts and the flag equal
    the oracle's, entry by entry."""
    t = meso.terrain_preset("small")
    scene = ctx.scene_from_terrain(t)
    bm = oracle.HostBrickMap.from_dense(scene.dense())
    allc = np.array([(x, y, z) for z in range(4) for y in range(4) for x in range(4)], dtype=np.int32)
    rng = np.random.default_rng(17)
    coords = allc[rng.integers(0, 64, 3000)]
    bad = [777, 2222]
    coords[bad[0]] = (4, 0, 0)
    coords[bad[1]] = (0, -1, 0)
    with pytest.raises(meso.MesoError, match="outside"):
        ctx.mesh(meso.SRC_BRICKMAP, coords=coords, scene=scene)
    q, counts = ctx.mesh(meso.SRC_BRICKMAP, coords=coords, scene=scene, chunk_counts=True, check=False)
    ok = np.array([i for i in range(len(coords)) if i not in bad])
    ref = oracle.mesh_chunks(oracle.SRC_BRICKMAP, coords=coords[ok], bm=bm)
    chunk = (ref >> np.uint64(44)).astype(np.int64)
    assert np.array_equal(counts[ok], np.bincount(chunk, minlength=len(ok)))
    assert counts[bad[0]] == 0 and counts[bad[1]] == 0
    remapped = (ref & np.uint64((1 << 44) - 1)) | (ok[chunk].astype(np.uint64) << np.uint64(44))
    assert np.array_equal(_sorted(q), np.sort(remapped))
    assert (counts[ok] == 0).sum() > 100  # air chunks among them


def test_matches_golden_fixture(ctx):
    import os
    golden = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    dev, _ = ctx.generate_chunks_u16(8, seed0=1)
    q, _ = ctx.mesh(meso.SRC_CHUNKS_U16, dev, n=8)
    assert np.array_equal(_sorted(q), np.load(os.path.join(golden, "quads_chunks_u16_seed1_n8.npy")))
    g = ctx.generate_dense_u8(64, 64, 64, seed=1)
    coords = np.array([(x, y, z) for z in range(2) for y in range(2) for x in range(2)], dtype=np.int32)
    q2, _ = ctx.mesh(meso.SRC_GRID_U8, g, coords=coords, dims=(64, 64, 64))
    assert np.array_equal(_sorted(q2), np.load(os.path.join(golden, "quads_dense_u8_64_seed1.npy")))


def test_grid_and_brickmap_sources_agree():
    """The same non-cubic content (96 x 64 x 128 voxels, clustered solids,
    a few materials) meshed from a dense uint16 grid, from a brick-map scene
    built from it, and folded to uint8 from a dense uint8 grid: all three see
    neighbours across chunk borders, so their quads equal each other's and
    the oracle's."""
    import mesoengine_gb300 as m
    cx = m.Context(0)
    try:
        rng = np.random.default_rng(31)
        z, y, x = np.indices((128, 64, 96))
        field = np.sin(x / 7.0) + np.cos(y / 5.0) + np.sin(z / 9.0) + rng.random((128, 64, 96)) * 0.8
        g = np.where(field > 1.2, 1 + (x // 8 + y // 16 + z // 32) % 4, 0).astype(np.uint16)
        coords = np.array([(i, j, k) for k in range(4) for j in range(2) for i in range(3)], dtype=np.int32)
        ref = oracle.mesh_chunks(oracle.SRC_GRID_U16, g, coords=coords)
        assert len(ref) > 1000
        d = cx.to_device(g)
        q_grid, _ = cx.mesh(meso.SRC_GRID_U16, d, coords=coords, dims=(96, 64, 128))
        scene = cx.scene_from_dense(g)
        q_bm, _ = cx.mesh(meso.SRC_BRICKMAP, coords=coords, scene=scene)
        g8 = g.astype(np.uint8)
        d8 = cx.to_device(g8)
        q8, _ = cx.mesh(meso.SRC_GRID_U8, d8, coords=coords, dims=(96, 64, 128))
        assert np.array_equal(_sorted(q_grid), ref)
        assert np.array_equal(_sorted(q_bm), ref)
        assert np.array_equal(_sorted(q8), oracle.mesh_chunks(oracle.SRC_GRID_U8, g8, coords=coords))
        # materials 1..4 survive the uint8 fold, so the quads are the same words
        assert np.array_equal(_sorted(q8), ref)
        scene.destroy()
        d.free()
        d8.free()
    finally:
        cx.close()
