"""tpd_load_ply's binary decoder on files larger than one read block (two
blocks of vertices, each decoded by several host threads): the all-float32
fast path, the general path (float64 positions, an unused uint8 property
between the used ones) and the ASCII parser give bit-identical records for
the same values, and a truncated file raises. The records' meaning is pinned
against the reference's GaussianPoint::fromModel in test_golden_host.py."""
import numpy as np
import pytest

import torpedo_gb300 as T

N = 140_000  # more than one 131,072-vertex read block
USED = ["x", "y", "z", "f_dc_0", "f_dc_1", "f_dc_2", "opacity", "scale_0", "scale_1", "scale_2",
        "rot_0", "rot_1", "rot_2", "rot_3"]


def _values(n, seed=7):
    rng = np.random.default_rng(seed)
    v = rng.normal(size=(n, len(USED))).astype(np.float32)
    v[:, USED.index("rot_0")] += 2.0  # quaternions well away from zero
    return v


def _write_binary(path, vals, mixed):
    n = vals.shape[0]
    if mixed:
        fields = [("x", "<f8"), ("y", "<f8"), ("z", "<f8"), ("red", "u1")] + [(m, "<f4") for m in USED[3:]]
        ply_types = {"<f8": "double", "u1": "uchar", "<f4": "float"}
    else:
        fields = [(m, "<f4") for m in USED]
        ply_types = {"<f4": "float"}
    arr = np.zeros(n, dtype=np.dtype(fields))
    for j, m in enumerate(USED):
        arr[m] = vals[:, j]
    if mixed:
        arr["red"] = np.arange(n) % 251
    header = f"ply\nformat binary_little_endian 1.0\nelement vertex {n}\n"
    header += "".join(f"property {ply_types[t]} {m}\n" for m, t in fields) + "end_header\n"
    with open(path, "wb") as f:
        f.write(header.encode())
        f.write(arr.tobytes())


def _write_ascii(path, vals):
    n = vals.shape[0]
    header = f"ply\nformat ascii 1.0\nelement vertex {n}\n"
    header += "".join(f"property float {m}\n" for m in USED) + "end_header\n"
    lines = [" ".join(f"{x:.9g}" for x in row) for row in vals]  # %.9g round-trips a float32
    with open(path, "w") as f:
        f.write(header + "\n".join(lines) + "\n")


def test_binary_paths_and_ascii_agree(tmp_path):
    vals = _values(N)
    _write_binary(tmp_path / "f32.ply", vals, mixed=False)
    _write_binary(tmp_path / "mixed.ply", vals, mixed=True)
    a = T.load_ply(tmp_path / "f32.ply")
    b = T.load_ply(tmp_path / "mixed.ply")
    assert a.shape == (N, 60)
    np.testing.assert_array_equal(a.view(np.uint32), b.view(np.uint32))
    # the positions are the file's values; the SH beyond the three DC terms are zero
    np.testing.assert_array_equal(a[:, 0:3], vals[:, 0:3])
    np.testing.assert_array_equal(a[:, 12:15], vals[:, 3:6])
    assert not a[:, 15:].any()
    k = 2000
    _write_ascii(tmp_path / "a.ply", vals[:k])
    c = T.load_ply(tmp_path / "a.ply")
    np.testing.assert_array_equal(c.view(np.uint32), a[:k].view(np.uint32))


def test_truncated_binary_raises(tmp_path):
    vals = _values(N)
    _write_binary(tmp_path / "f32.ply", vals, mixed=False)
    data = (tmp_path / "f32.ply").read_bytes()
    (tmp_path / "cut.ply").write_bytes(data[:-100])
    with pytest.raises(T.TpdError):
        T.load_ply(tmp_path / "cut.ply")
