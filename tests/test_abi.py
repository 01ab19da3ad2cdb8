"""The C ABI: the library builds, loads, and exports every entry point that
include/meso.h declares; C struct layouts match the Python binding.  No GPU
is needed (no compute call is made)."""
import ctypes
import os
import re
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "meso.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(meso_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_entry_points():
    names = declared_functions()
    for n in ("meso_ctx_create", "meso_mesh_chunks", "meso_raymarch", "meso_edit_spheres", "meso_server_create",
              "meso_autotune", "meso_raymarch_noalloc"):
        assert n in names


def test_library_exports_every_declared_symbol():
    import mesoengine_gb300 as meso
    meso._build.build()
    lib = ctypes.CDLL(meso.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", meso.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (meso_[a-z0-9_]+)", out))
    assert set(declared_functions()) <= exported


def test_context_creation_fails_cleanly_without_a_gpu():
    import mesoengine_gb300 as meso
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(meso.MesoError) as e:
        meso.Context(0)
    assert e.value.status in (1, 6)


def test_struct_layouts_match_binding():
    import mesoengine_gb300 as meso
    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "meso.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(meso_camera), sizeof(meso_hit), sizeof(meso_terrain),
         sizeof(meso_mesh_source), sizeof(meso_mesh_output), sizeof(meso_sphere_edit), sizeof(meso_request),
         sizeof(meso_completion), sizeof(meso_config), sizeof(meso_scene_info));
  return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "l.c")
        exe = os.path.join(d, "l")
        open(c, "w").write(src)
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        sizes = [int(v) for v in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()]
    py = [ctypes.sizeof(meso.Camera), meso.HIT_DTYPE.itemsize, ctypes.sizeof(meso.Terrain),
          ctypes.sizeof(meso.MeshSource), ctypes.sizeof(meso.MeshOutput), ctypes.sizeof(meso.SphereEdit),
          ctypes.sizeof(meso.Request), ctypes.sizeof(meso.Completion), ctypes.sizeof(meso.Config),
          ctypes.sizeof(meso.SceneInfo)]
    assert sizes == py


def test_product_does_not_use_the_oracle():
    import mesoengine_gb300 as meso
    out = subprocess.run(["ldd", meso.LIB_PATH], capture_output=True, text=True).stdout
    assert "oracle" not in out
    pkg = os.path.join(ROOT, "mesoengine_gb300")
    for sub in ("csrc", ""):
        d = os.path.join(pkg, sub)
        for f in os.listdir(d):
            if f.endswith((".cu", ".h", ".cpp", ".py")):
                text = open(os.path.join(d, f)).read()
                assert "meso_oracle" not in text and "import oracle" not in text, f


def test_cpp_wrapper_header_compiles():
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "w.cpp")
        open(c, "w").write('#include "meso.hpp"\nint main() { return 0; }\n')
        subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-I", os.path.join(ROOT, "include"), c],
                       check=True)
