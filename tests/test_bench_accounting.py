"""The bench line's launch count (gpu_launches) follows the frame's kernel list:
frame_begin, preprocess, the depth-sort passes (one per 8-bit digit of the
32 depth bits plus the view bits; a pass whose digit is uniform still
launches), the depth-order scan fused with keygen, per tile-id pass a counting
launch and a scatter (one onesweep launch per pass with the look-back form),
and the blend. The cfg1 frame (one view, 13-bit tile ids: 2 passes) is the 12
launches of its ncu launch list."""
import importlib.util
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.mark.parametrize("views,tile_passes,counted,launches", [
    (1, 2, True, 12),    # cfg1: 4 depth passes, 2 counted tile-id passes
    (1, 2, False, 10),   # the same frame with onesweep tile-id passes
    (64, 3, True, 15),   # cfg3: 6 view bits -> 5 depth passes, 3 tile-id passes
    (8, 3, True, 15),    # cfg4: 3 view bits -> 5 depth passes
    (2, 1, True, 11),    # 1 view bit -> 5 depth passes, 1 tile-id pass
])
def test_kernels_per_frame(bench, views, tile_passes, counted, launches):
    assert bench.kernels_per_frame(views, tile_passes, counted) == launches


def test_launch_list_profile_matches(bench):
    """The committed launch list of the cfg1 frame holds whole frames of as
    many kernels as the formula counts."""
    text = (ROOT / "profiles" / "launches_cfg1_frame.md").read_text()
    m = re.search(r"five whole frames of (\d+)\s+kernels", text)
    assert m, "the launch list states its kernels per frame"
    assert int(m.group(1)) == bench.kernels_per_frame(1, 2, True)
