"""The C++ wrapper (include/tpdsplat.hpp) compiles against the C ABI with g++
and renders the same frame as the Python binding, bit for bit."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import torpedo_gb300 as T
from torpedo_gb300 import _lib as L
from torpedo_gb300 import configs

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "cpp" / "engine_render.cpp"


def _build(tmp: Path) -> Path:
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not found")
    lib = L.lib_path()
    exe = tmp / "engine_render"
    cmd = [gxx, "-std=c++17", "-O1", "-Wall", "-Werror", "-I", str(ROOT / "include"), str(SRC), "-o", str(exe),
           "-L", str(lib.parent), "-ltpdsplat", f"-Wl,-rpath,{lib.parent}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_cpp_wrapper_compiles_and_links(tmp_path):
    _build(tmp_path)


@pytest.mark.gpu
def test_cpp_wrapper_frame_equals_python(cuda, tmp_path):
    exe = _build(tmp_path)
    out = tmp_path / "img.f32"
    r = subprocess.run([str(exe), str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    img_cpp = np.fromfile(out, dtype=np.float32).reshape(256, 256, 3)
    eng = T.GaussianEngine()
    eng.compile(configs.scene("cfg0").records)
    eng.set_camera(configs.cameras("cfg0")[0])
    eng.raster_frame()
    img_py = eng.read_image()[0]
    eng.close()
    np.testing.assert_array_equal(img_cpp, img_py)
