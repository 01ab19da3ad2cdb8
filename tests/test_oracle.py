"""CPU oracle: known-answer cases, properties and the committed golden fixtures.

The reference has no greedy mesher, no raymarcher and no tests or golden
vectors, so parity is pinned here by hand-computed cases (one voxel, a full
chunk, a checkerboard, axis-aligned rays) and by fixtures written by
tests/golden/make_golden.py.
"""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
MISS = np.uint64(2**64 - 1)


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def golden():
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        return json.load(f)


def mesh1(c):
    return oracle.mesh_chunks(oracle.SRC_CHUNKS_U16, c[None].astype(np.uint16))


# ----------------------------------------------------------------- meshing KATs

def test_single_voxel_six_unit_quads():
    c = np.zeros((32, 32, 32), np.uint16)
    c[5, 6, 7] = 3  # z, y, x
    u = oracle.unpack_quads(mesh1(c))
    assert u["dir"].tolist() == [0, 1, 2, 3, 4, 5]
    assert set(u["x"]) == {7} and set(u["y"]) == {6} and set(u["z"]) == {5}
    assert set(u["w"]) == {1} and set(u["h"]) == {1} and set(u["material"]) == {3}


def test_full_chunk_six_full_quads():
    c = np.full((32, 32, 32), 9, np.uint16)
    u = oracle.unpack_quads(mesh1(c))
    assert len(u["dir"]) == 6
    assert set(u["w"]) == {32} and set(u["h"]) == {32}
    # +X face sits on x = 31, -X on x = 0, and so on
    assert u["x"][0] == 31 and u["x"][1] == 0 and u["y"][2] == 31 and u["z"][4] == 31


def test_checkerboard_has_no_merges():
    z, y, x = np.indices((32, 32, 32))
    c = ((x + y + z) % 2 == 0).astype(np.uint16)
    q = mesh1(c)
    assert len(q) == 6 * 16384
    u = oracle.unpack_quads(q)
    assert (u["w"] == 1).all() and (u["h"] == 1).all()


def test_material_boundary_splits_quads():
    c = np.zeros((32, 32, 32), np.uint16)
    c[0, 0, :16] = 1
    c[0, 0, 16:] = 2
    u = oracle.unpack_quads(mesh1(c))
    top = u["dir"] == 4  # +Z faces of the row: two runs of 16
    assert sorted(u["w"][top].tolist()) == [16, 16]
    assert sorted(u["material"][top].tolist()) == [1, 2]


def test_greedy_scan_order_width_first():
    # an L shape: the greedy widens along u first, then grows along v
    c = np.zeros((32, 32, 32), np.uint16)
    c[0, 0, 0:4] = 5
    c[0, 1, 0:2] = 5
    u = oracle.unpack_quads(mesh1(c))
    top = np.nonzero(u["dir"] == 4)[0]  # Z faces: u = x, v = y
    got = sorted(zip(u["x"][top], u["y"][top], u["w"][top], u["h"][top]))
    assert got == [(0, 0, 4, 1), (0, 1, 2, 1)]


def test_quads_cover_exposed_faces_exactly():
    chunks, _ = oracle.gen_chunks_u16(24, 11)
    q = oracle.mesh_chunks(oracle.SRC_CHUNKS_U16, chunks)
    u = oracle.unpack_quads(q)
    area = np.bincount(u["chunk"], weights=u["w"] * u["h"], minlength=24).astype(int)
    faces = [oracle.count_faces(oracle.SRC_CHUNKS_U16, chunks, (i, 0, 0)) for i in range(24)]
    assert area.tolist() == faces
    # quads of one direction and slice are disjoint and inside the chunk
    for i in range(4):
        sel = u["chunk"] == i
        cover = np.zeros((6, 32, 32, 32), np.int32)
        for d, x, y, z, w, h in zip(*(u[k][sel] for k in ("dir", "x", "y", "z", "w", "h"))):
            if d < 2:
                assert y + w <= 32 and z + h <= 32
                cover[d, z:z + h, y:y + w, x] += 1
            elif d < 4:
                assert x + w <= 32 and z + h <= 32
                cover[d, z:z + h, y, x:x + w] += 1
            else:
                assert x + w <= 32 and y + h <= 32
                cover[d, z, y:y + h, x:x + w] += 1
        assert cover.max() <= 1


def test_grid_neighbours_hide_faces():
    g = np.zeros((64, 32, 32), np.uint16)  # z, y, x: two chunks stacked along z
    g[31, 0, 0] = 1
    g[32, 0, 0] = 1
    q = oracle.mesh_chunks(oracle.SRC_GRID_U16, g, coords=[(0, 0, 0), (0, 0, 1)])
    u = oracle.unpack_quads(q)
    # the shared face across the chunk border is hidden on both sides
    assert not ((u["chunk"] == 0) & (u["dir"] == 4)).any()
    assert not ((u["chunk"] == 1) & (u["dir"] == 5)).any()
    assert len(q) == 10


# ----------------------------------------------------------- raymarching KATs

def _bm_dense(g):
    return oracle.HostBrickMap.from_dense(g.astype(np.uint16))


def _ray(bm, origin, d, shadow=False, light=None):
    return oracle.trace_ray(bm, origin, d, light=light, shadow=shadow)


def test_axis_ray_hits_known_voxel():
    g = np.zeros((64, 64, 64), np.uint16)
    g[10, 20, 40] = 7  # z, y, x
    bm = _bm_dense(g)
    h = _ray(bm, (-5.5, 20.5, 10.5), (1.0, 0.0, 0.0))
    assert h["voxel"] == 40 + 20 * 64 + 10 * 64 * 64
    assert h["face"] == 1  # entered through its -X face
    assert h["material"] == 7
    assert h["t"] == np.float32(45.5)
    # bricks along x: 0..4 empty (5 coarse steps into brick 5), then x 40 is the
    # first voxel of brick 5: no fine step
    assert h["steps"] == (5 << 16) | 0


def test_axis_ray_fine_steps_inside_occupied_brick():
    g = np.zeros((64, 64, 64), np.uint16)
    g[10, 20, 45] = 2
    bm = _bm_dense(g)
    h = _ray(bm, (-5.5, 20.5, 10.5), (1.0, 0.0, 0.0))
    assert h["voxel"] == 45 + 20 * 64 + 10 * 64 * 64
    assert h["steps"] == (5 << 16) | 5  # x 40 -> 45 inside brick 5
    assert h["t"] == np.float32(50.5)


def test_ray_missing_grid_and_ray_from_inside():
    g = np.zeros((32, 32, 32), np.uint16)
    g[0, 0, 0] = 1
    bm = _bm_dense(g)
    miss = _ray(bm, (-10.0, -10.0, -10.0), (-1.0, 0.0, 0.0))
    assert miss["voxel"] == MISS and np.isinf(miss["t"]) and miss["face"] == 6 and miss["steps"] == 0
    inside = _ray(bm, (0.5, 0.5, 0.5), (0.0, 0.0, 1.0))
    assert inside["voxel"] == 0 and inside["face"] == 6 and inside["t"] == 0.0


def test_shadow_ray_occluded_and_lit():
    g = np.zeros((64, 64, 64), np.uint16)
    g[0, :, :] = 3           # floor at z = 0
    g[20:24, 28:36, 28:36] = 4  # a block above (32, 32)
    bm = _bm_dense(g)
    L = oracle.light_dir((0.0, 0.0, 1.0))

    def trace(o):
        return _ray(bm, o, (0.0, 0.0, -1.0), shadow=True, light=L)

    under = trace((32.5, 32.5, 10.5))   # below the block: floor hit, shadowed
    assert under["voxel"] == 32 + 32 * 64 and under["shadow"] == 1
    open_ = trace((5.5, 5.5, 10.5))    # away from the block: lit
    assert open_["voxel"] == 5 + 5 * 64 and open_["shadow"] == 0


def test_hits_agree_with_dense_sampling():
    t = oracle.terrain(64, 64, 64, 4, 32, 6, 4.0, 16.0, 48, 0.7)
    bm = oracle.HostBrickMap.from_terrain(t)
    dense = bm.dense()
    cam = oracle.camera((-20.0, -15.0, 70.0), (32.0, 32.0, 8.0), 24, 16)
    h = oracle.raymarch(bm, cam)
    o = np.array(cam.origin_chunk) * 32 + np.array(cam.origin_frac)
    d = np.zeros(3, np.float32)
    for k in np.nonzero(h["voxel"] != MISS)[0][:60]:
        py, px = divmod(int(k), cam.width)
        oracle.lib().mo_camera_ray(cam, px, py, d.ctypes.data)
        v = int(h["voxel"][k])
        x, y, z = v % 64, (v // 64) % 64, v // 4096
        assert dense[z, y, x] > 0
        ts = np.linspace(0.0, float(h["t"][k]) - 1e-3, 2000)
        p = np.floor(o[None] + d[None].astype(np.float64) * ts[:, None]).astype(int)
        ok = ((p >= 0) & (p < 64)).all(1)
        assert not (dense[p[ok, 2], p[ok, 1], p[ok, 0]] > 0).any()


# ------------------------------------------------------------------- goldens

def test_goldens_chunks_and_quads():
    gd = golden()
    chunks, solid = oracle.gen_chunks_u16(8, 1)
    assert sha(chunks) == gd["chunks_u16_seed1_n8_sha256"]
    assert solid.tolist() == gd["chunks_u16_seed1_n8_solid"]
    q = oracle.mesh_chunks(oracle.SRC_CHUNKS_U16, chunks)
    assert np.array_equal(q, np.load(os.path.join(GOLDEN, "quads_chunks_u16_seed1_n8.npy")))


def test_goldens_dense_grid():
    gd = golden()
    grid = oracle.gen_dense_u8(64, 64, 64, 1)
    assert sha(grid) == gd["dense_u8_64_seed1_sha256"]
    coords = np.array([(x, y, z) for z in range(2) for y in range(2) for x in range(2)], dtype=np.int32)
    q = oracle.mesh_chunks(oracle.SRC_GRID_U8, grid, coords=coords)
    assert np.array_equal(q, np.load(os.path.join(GOLDEN, "quads_dense_u8_64_seed1.npy")))


def test_goldens_terrain_and_hits():
    gd = golden()
    bm = oracle.HostBrickMap.from_terrain(oracle.terrain(128, 128, 128, 2, 64, 6, 7.0, 32.0, 48, 0.7))
    assert int(bm.bm.n_bricks) == gd["terrain128_bricks"]
    assert sha(bm.ptr()) == gd["terrain128_ptr_sha256"]
    assert sha(bm.occ()) == gd["terrain128_occ_sha256"]
    assert sha(bm.mat()) == gd["terrain128_mat_sha256"]
    h = oracle.raymarch(bm, oracle.camera((-40.0, -30.0, 140.0), (64.0, 64.0, 20.0), 96, 64))
    ref = np.load(os.path.join(GOLDEN, "hits_terrain128_96x64.npy"))
    assert np.array_equal(h.view(np.uint8), ref.view(np.uint8))


def test_edits_and_dirty_chunks():
    import ctypes
    g = np.zeros((64, 64, 64), np.uint16)
    bm = oracle.HostBrickMap.from_dense(g)
    sp = [oracle.Sphere((ctypes.c_int32 * 3)(10, 10, 10), 3, 5, 0),
          oracle.Sphere((ctypes.c_int32 * 3)(11, 10, 10), 1, 0, 0)]
    bm.edit(sp)
    d = bm.dense()
    z, y, x = np.indices(d.shape)
    s0 = (x - 10) ** 2 + (y - 10) ** 2 + (z - 10) ** 2 <= 9
    s1 = (x - 11) ** 2 + (y - 10) ** 2 + (z - 10) ** 2 <= 1
    assert np.array_equal(d > 0, s0 & ~s1)
    assert (d[s0 & ~s1] == 5).all()
    assert bm.dirty_chunks(sp).tolist() == [0]
    # a sphere near a chunk border dirties the neighbour through the one-voxel halo
    sp2 = [oracle.Sphere((ctypes.c_int32 * 3)(30, 5, 5), 1, 9, 0)]
    assert bm.dirty_chunks(sp2).tolist() == [0, 1]


def test_generators_are_deterministic():
    a, _ = oracle.gen_chunks_u16(3, 77)
    b, _ = oracle.gen_chunks_u16(3, 77)
    assert np.array_equal(a, b)
    assert oracle.lib().mo_pcg3d(1, 2, 3) == oracle.lib().mo_pcg3d(1, 2, 3)
    v = oracle.lib().mo_vnoise3(5, 6, 7, 64, 1)
    assert 0.0 <= v < 1.0


# ------------------------------------------------------ downstream restatements

def test_erosion_pyramid_of_a_solid_chunk():
    occ = np.ones((32, 32, 32), np.uint8)
    m = oracle.erode_mips(occ, 5)
    for d in range(5):
        z, y, x = np.indices((32, 32, 32))
        expect = ((x >= d) & (x <= 31 - d) & (y >= d) & (y <= 31 - d) & (z >= d) & (z <= 31 - d)) if d else occ > 0
        assert np.array_equal(m[d] > 0, expect), d


def test_erosion_needs_all_26_neighbours():
    occ = np.zeros((32, 32, 32), np.uint8)
    occ[9:12, 9:12, 9:12] = 1          # a 3^3 block: only its centre is enclosed
    m = oracle.erode_mips(occ, 3)
    assert m[1].sum() == 1 and m[1][10, 10, 10] == 1
    assert m[2].sum() == 0
    occ[9, 9, 9] = 0                    # remove one corner: the centre is no longer enclosed
    assert oracle.erode_mips(occ, 2)[1].sum() == 0


def test_quad_vertices_known_corners():
    q = np.array([oracle.lib().mo_pack_quad(0, 4, 2, 3, 5, 4, 2, 9),   # +Z at z=5, x 2..6, y 3..5
                  oracle.lib().mo_pack_quad(1, 1, 7, 0, 0, 1, 1, 3)],  # -X at x=7 of chunk 1
                 dtype=np.uint64)
    pos, attr = oracle.quads_to_vertices(q, [(0, 0, 0), (1, 0, 2)])
    assert pos[0].tolist() == [[2, 3, 6], [6, 3, 6], [6, 5, 6], [2, 5, 6]]
    # -X: plane x = 7 (+32 origin), reversed corner order
    assert pos[1].tolist() == [[39, 0, 64], [39, 0, 65], [39, 1, 65], [39, 1, 64]]
    assert (attr[0] & 0xFFFF).tolist() == [9] * 4 and ((attr[1] >> 16) & 7).tolist() == [1] * 4
    # counter-clockwise seen from outside: (p1 - p0) x (p2 - p0) is along the normal
    for i, normal in ((0, (0, 0, 1)), (1, (-1, 0, 0))):
        n = np.cross(pos[i, 1] - pos[i, 0], pos[i, 2] - pos[i, 0])
        assert np.array_equal(np.sign(n), np.array(normal))
