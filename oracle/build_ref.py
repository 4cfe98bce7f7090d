"""Compiles the reference's own code into oracle/_ref/libtpdref.so.

Recipe for the checker only (outputs go to oracle/_ref/, git-ignored):
  - host C++: the reference's math headers, Camera.cpp, PerspectiveCamera.cpp,
    GaussianGeometry.cpp with its vendored miniply.cpp, and the body of
    GaussianEngine::getHigherMSB, compiled from where they lie in the
    reference tree (GaussianEngine.h itself includes Vulkan headers that are
    not present, so that one function body is extracted into
    oracle/_ref/gen_higher_msb.cpp);
  - the compute shaders: there is no slangc and no Vulkan on these machines,
    so oracle/slang_to_cpp.py translates the Slang source of the nine
    shaders and their module token by token into C++
    (oracle/_ref/gen/*.inc), and oracle/ref_shaders.cpp runs them on the CPU
    with the dispatch sequence of GaussianEngine::rasterFrame
    (oracle/slang_cpu.h gives the language's types and execution model).
"""
from __future__ import annotations

import os
import re
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
LIB = OUT / "libtpdref.so"
# The reference checkout: TPD_REFERENCE_ROOT, else where the build container
# mounts it (read-only). This recipe is the one place that names it; where it
# is absent (the GPU machines) nothing is built and the committed fixtures
# stand in for it.
REFERENCE_ROOT = Path(os.environ.get("TPD_REFERENCE_ROOT", "/root/reference"))
REF = REFERENCE_ROOT / "torpedo"


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


SHADERS = REF / "volumetric" / "assets" / "gaussian"


def _compile(src: Path, obj: Path, flags: list[str]) -> subprocess.CompletedProcess:
    return subprocess.run(["g++", "-O2", "-fPIC", "-c", *flags, str(src), "-o", str(obj)], capture_output=True,
                          text=True)


def build(force: bool = False) -> Path:
    if not available():
        raise RuntimeError(f"reference sources not found under {REF}")
    OUT.mkdir(exist_ok=True)
    if LIB.exists() and not force:
        return LIB
    from concurrent.futures import ThreadPoolExecutor

    from oracle import slang_to_cpp

    gen = _extract_higher_msb()
    slang_to_cpp.generate(SHADERS, OUT / "gen")
    inc = [f"-I{REF / d / 'include'}" for d in ("math", "rendering", "extension", "volumetric")]
    host = ["-std=c++23", "-include", "cstdint", "-include", "cstring", "-include", "algorithm", *inc,
            f"-I{REF / 'volumetric/src'}"]
    # the shaders: IEEE single precision, no contraction, threads for workgroups
    shader = ["-std=c++23", "-ffp-contract=off", "-fno-strict-aliasing", "-pthread", f"-I{HERE}", f"-I{OUT / 'gen'}"]
    # GaussianPoint::random seeds itself from std::random_device: the forced
    # header makes that seed settable (see seeded_random_device.h)
    seeded = [*host, f"-I{HERE}", "-include", str(HERE / "seeded_random_device.h")]
    units = [(HERE / "ref_glue.cpp", [*host, f"-I{HERE}"]), (gen, host), (REF / "rendering/src/Camera.cpp", host),
             (REF / "extension/src/PerspectiveCamera.cpp", host), (REF / "volumetric/src/GaussianGeometry.cpp", seeded),
             (REF / "volumetric/src/miniply.cpp", host), (HERE / "ref_shaders.cpp", shader)]
    objs = [OUT / f"{src.stem}.o" for src, _ in units]
    with ThreadPoolExecutor(max_workers=len(units)) as ex:
        results = list(ex.map(lambda u: _compile(u[0][0], u[1], u[0][1]), zip(units, objs)))
    for (src, _), r in zip(units, results):
        if r.returncode != 0:
            raise RuntimeError(f"reference build failed on {src.name}:\n{r.stderr[-4000:]}")
    r = subprocess.run(["g++", "-shared", "-pthread", *map(str, objs), "-o", str(LIB)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference link failed:\n{r.stderr[-4000:]}")
    return LIB


if __name__ == "__main__":
    print(build(force=True))
