"""Writes the golden fixtures of the CPU oracle (run from the repo root).

The reference MesoEngine has neither a greedy mesher nor a raymarcher and no
tests, so these fixtures pin the oracle itself: any later change to the
oracle's noise, scene generators, mesher or traversal shows up as a diff
against them, and the GPU tests compare the device results to the same files.

    python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
import oracle  # noqa: E402


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main():
    out = {}
    chunks, solid = oracle.gen_chunks_u16(8, 1)
    out["chunks_u16_seed1_n8_sha256"] = sha(chunks)
    out["chunks_u16_seed1_n8_solid"] = [int(v) for v in solid]
    quads = oracle.mesh_chunks(oracle.SRC_CHUNKS_U16, chunks)
    np.save(os.path.join(HERE, "quads_chunks_u16_seed1_n8.npy"), quads)
    grid = oracle.gen_dense_u8(64, 64, 64, 1)
    out["dense_u8_64_seed1_sha256"] = sha(grid)
    coords = np.array([(x, y, z) for z in range(2) for y in range(2) for x in range(2)], dtype=np.int32)
    gq = oracle.mesh_chunks(oracle.SRC_GRID_U8, grid, coords=coords)
    np.save(os.path.join(HERE, "quads_dense_u8_64_seed1.npy"), gq)
    t = oracle.terrain(128, 128, 128, 2, 64, 6, 7.0, 32.0, 48, 0.7)
    bm = oracle.HostBrickMap.from_terrain(t)
    out["terrain128_ptr_sha256"] = sha(bm.ptr())
    out["terrain128_occ_sha256"] = sha(bm.occ())
    out["terrain128_mat_sha256"] = sha(bm.mat())
    out["terrain128_bricks"] = int(bm.bm.n_bricks)
    cam = oracle.camera((-40.0, -30.0, 140.0), (64.0, 64.0, 20.0), 96, 64)
    hits = oracle.raymarch(bm, cam)
    np.save(os.path.join(HERE, "hits_terrain128_96x64.npy"), hits)
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print("wrote goldens:", sorted(out))


if __name__ == "__main__":
    main()
