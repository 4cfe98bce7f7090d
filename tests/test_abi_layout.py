"""The ctypes mirrors of the C ABI's structs have the C layout: a small C
program built with the host compiler against include/tpdsplat.h prints the
size of each struct and the offset of each field the Python side declares,
and they must agree (tpd_settings_init fills the whole C struct, so a short
mirror would be written past its end)."""
import shutil
import subprocess
from pathlib import Path

import ctypes as C
import pytest

from torpedo_gb300 import _lib as L

ROOT = Path(__file__).resolve().parents[1]
STRUCTS = {"tpd_settings": L.Settings, "tpd_frame_stats": L.FrameStats, "tpd_view": L.View}


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no host C compiler")
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "tpdsplat.h"', "int main(void) {"]
    for cname, py in STRUCTS.items():
        lines.append(f'    printf("{cname} size %zu\\n", sizeof({cname}));')
        for field, _ in py._fields_:
            lines.append(f'    printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines += ["    return 0;", "}"]
    d = tmp_path_factory.mktemp("abi")
    src, exe = d / "layout.c", d / "layout"
    src.write_text("\n".join(lines) + "\n")
    subprocess.run([cc, "-std=c11", f"-I{ROOT / 'include'}", str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    layout = {}
    for line in out.splitlines():
        name, key, value = line.split()
        layout[(name, key)] = int(value)
    return layout


@pytest.mark.parametrize("cname", sorted(STRUCTS))
def test_struct_size_and_field_offsets(c_layout, cname):
    py = STRUCTS[cname]
    assert C.sizeof(py) == c_layout[(cname, "size")], cname
    for field, _ in py._fields_:
        assert getattr(py, field).offset == c_layout[(cname, field)], (cname, field)
