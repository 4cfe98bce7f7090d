"""Builds libtpdsplat.so in-tree (torpedo_gb300/_build/) with nvcc for sm_103a.

Each translation unit compiles in parallel; the library is relinked only when
a source or header is newer than it.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = OUT / "libtpdsplat.so"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
          "-I", str(CSRC), "-I", str(INCLUDE)]

# per-file extra flags: the preprocess transcribes the shader's operation
# order, so no multiply may be fused into an add there.
SOURCES = {
    "preprocess.cu": ["--fmad=false"],
    "keygen.cu": [],
    "sort.cu": [],
    "blend.cu": [],
    "backward.cu": [],
    "engine.cu": [],
    "scan_static.cu": [],
    "host_util.cpp": ["-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-pthread"],
}


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(path).exists():
        raise RuntimeError("nvcc not found; CUDA 13 toolkit required to build libtpdsplat")
    return path


def _headers_mtime() -> float:
    files = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h"))
    return max((f.stat().st_mtime for f in files), default=0.0)


def _compile(src: str, flags: list[str], hdr_mtime: float, verbose: bool) -> Path:
    s = CSRC / src
    obj = OUT / (src + ".o")
    if obj.exists() and obj.stat().st_mtime >= max(s.stat().st_mtime, hdr_mtime):
        return obj
    cmd = [nvcc(), *ARCH, *COMMON, *flags, "-c", str(s), "-o", str(obj)]
    if src.endswith(".cpp"):
        cmd = [nvcc(), *COMMON, *flags, "-x", "c++", "-c", str(s), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    if verbose and (r.stdout or r.stderr):
        print(r.stdout, r.stderr)
    return obj


def build(verbose: bool = False, force: bool = False) -> Path:
    """TPD_CHECKED=1 in the environment adds -DTPD_CHECKED (extra debug checks)."""
    OUT.mkdir(exist_ok=True)
    flags = "checked" if os.environ.get("TPD_CHECKED") == "1" else "release"
    stamp = OUT / "flavour"
    if not stamp.exists() or stamp.read_text() != flags:
        force = True
        stamp.write_text(flags)
    if flags == "checked":
        COMMON.append("-DTPD_CHECKED")
    if force:
        for o in OUT.glob("*.o"):
            o.unlink()
    hdr = _headers_mtime()
    with ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda kv: _compile(kv[0], kv[1], hdr, verbose), SOURCES.items()))
    newest = max(o.stat().st_mtime for o in objs)
    if force or not LIB.exists() or LIB.stat().st_mtime < newest:
        tmp = OUT / "libtpdsplat.so.tmp"
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys

    print(build(verbose=True, force="--force" in sys.argv))
