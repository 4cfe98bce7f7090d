"""Compiles the reference's own host C++ into oracle/_ref/libtpdref.so.

Recipe for the checker only (outputs go to oracle/_ref/, git-ignored): the
reference's math headers, Camera.cpp, PerspectiveCamera.cpp,
GaussianGeometry.cpp with its vendored miniply.cpp, and the body of
GaussianEngine::getHigherMSB, compiled from where they lie in the reference
tree. GaussianEngine.h itself includes Vulkan headers that are not present,
so that one function body is extracted into oracle/_ref/gen_higher_msb.cpp.
The reference's shaders (Slang) cannot be built here: there is no slangc and
no Vulkan on these machines.
"""
from __future__ import annotations

import os
import re
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
LIB = OUT / "libtpdref.so"
REF = Path(os.environ.get("TPD_REFERENCE_ROOT", "/root/reference")) / "torpedo"


def available() -> bool:
    return (REF / "rendering" / "src" / "Camera.cpp").exists()


def _extract_higher_msb() -> Path:
    text = (REF / "volumetric/include/torpedo/volumetric/GaussianEngine.h").read_text()
    m = re.search(r"constexpr uint32_t tpd::GaussianEngine::getHigherMSB\(const uint32_t n\) noexcept \{\n(.*?)\n\}",
                  text, re.S)
    if not m:
        raise RuntimeError("getHigherMSB not found in GaussianEngine.h")
    gen = OUT / "gen_higher_msb.cpp"
    gen.write_text("#include <cstdint>\n// generated from GaussianEngine.h by oracle/build_ref.py\n"
                   "uint32_t ref_higher_msb_impl(const uint32_t n) {\n" + m.group(1) + "\n}\n")
    return gen


def build(force: bool = False) -> Path:
    if not available():
        raise RuntimeError(f"reference sources not found under {REF}")
    OUT.mkdir(exist_ok=True)
    if LIB.exists() and not force:
        return LIB
    gen = _extract_higher_msb()
    inc = [f"-I{REF / d / 'include'}" for d in ("math", "rendering", "extension", "volumetric")]
    srcs = [HERE / "ref_glue.cpp", gen, REF / "rendering/src/Camera.cpp", REF / "extension/src/PerspectiveCamera.cpp",
            REF / "volumetric/src/GaussianGeometry.cpp", REF / "volumetric/src/miniply.cpp"]
    cmd = ["g++", "-std=c++23", "-O2", "-fPIC", "-shared", "-include", "cstdint", "-include", "cstring",
           "-include", "algorithm", *inc, f"-I{REF / 'volumetric/src'}", *map(str, srcs), "-o", str(LIB)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference build failed:\n{r.stderr[-4000:]}")
    return LIB


if __name__ == "__main__":
    print(build(force=True))
