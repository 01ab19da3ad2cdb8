"""A compiled C++ host calls the library through include/meso.hpp: the
program (tests/cpp/meso_caller.cpp) is built with g++ against
libmeso_gb300.so, renders the golden view (compared byte for byte with the
committed golden hits inside the program), meshes the scene, edits it and
keeps a mesh store current; its quads are compared here with the oracle's."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle
import mesoengine_gb300 as meso

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_caller(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    lib = meso.LIB_PATH
    assert os.path.exists(lib)
    exe = str(tmp_path / "meso_caller")
    subprocess.run([gxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "meso_caller.cpp"), "-o", exe, lib,
                    "-Wl,-rpath," + os.path.dirname(lib)], check=True)
    cam = meso.camera((-40.0, -30.0, 140.0), (64.0, 64.0, 20.0), 96, 64)
    (tmp_path / "camera.bin").write_bytes(bytes(cam))
    golden = np.load(os.path.join(ROOT, "tests", "golden", "hits_terrain128_96x64.npy"))
    (tmp_path / "hits.bin").write_bytes(np.ascontiguousarray(golden).tobytes())
    r = subprocess.run([exe, str(tmp_path / "camera.bin"), str(tmp_path / "hits.bin"), str(tmp_path)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    t = oracle.terrain(128, 128, 128, 2, 64, 6, 7.0, 32.0, 48, 0.7)
    bm = oracle.HostBrickMap.from_terrain(t)
    idx = np.arange(64)
    coords = np.stack([idx % 4, (idx // 4) % 4, idx // 16], 1).astype(np.int32)
    before = np.fromfile(tmp_path / "quads_before.bin", dtype=np.uint64)
    assert np.array_equal(before, oracle.mesh_chunks(oracle.SRC_BRICKMAP, coords=coords, bm=bm))
    sp = [oracle.Sphere((ctypes.c_int32 * 3)(11 * k % 128, 37 * k % 128, 5 + 3 * k), 3 + k % 7,
                        0 if k % 3 == 0 else 100 + 977 * k, 0) for k in range(12)]
    bm.edit(sp)
    after = np.fromfile(tmp_path / "quads_after.bin", dtype=np.uint64)
    assert np.array_equal(after, oracle.mesh_chunks(oracle.SRC_BRICKMAP, coords=coords, bm=bm))
