"""The blend's per-block cull never drops a pair the exact per-pixel rule
keeps: tests/cpp/cull_mask_check.c restates block_mask() and the per-pixel p2
of torpedo_gb300/csrc/blend.cu in C and checks them on random thin, rotated,
huge and near-threshold entries, for the forward's 8x8 and 8x4 blocks, with
the GPU's approximate square root and reciprocal stood in for by nudged
correctly rounded ones."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def test_block_mask_is_conservative(tmp_path):
    gcc = shutil.which("gcc")
    if not gcc:
        pytest.skip("gcc not found")
    exe = tmp_path / "cull_mask_check"
    r = subprocess.run([gcc, "-O2", "-ffp-contract=off", str(ROOT / "tests" / "cpp" / "cull_mask_check.c"), "-o",
                        str(exe), "-lm"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe), "100000", "7"], capture_output=True, text=True, timeout=120)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    viol, visits, truth = (int(v) for v in r.stdout.split()[1::2])
    assert viol == 0
    # the masks stay tight: within 10% of the blocks that hold a kept pixel
    assert truth <= visits <= 1.10 * truth
