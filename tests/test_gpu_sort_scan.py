"""The radix sort and the tile-count scan through their standalone C-ABI entry
points: bit-exact against a stable sort / a sequential scan on the same data,
over sizes around the 4096-key partition and the 2048-key histogram chunk,
several key widths, heavy ties, and empty input."""
import numpy as np
import pytest

import torpedo_gb300 as T
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _keys(rng, n, bits, ties=False):
    hi = max(0, bits - 32)
    k = rng.integers(0, 1 << min(bits, 32), size=n, dtype=np.uint64)
    if hi:
        k |= rng.integers(0, 1 << hi, size=n, dtype=np.uint64) << np.uint64(32)
    if ties and n:
        k[::3] = k[0]
        k[1::5] = k[min(1, n - 1)]
    return k


@pytest.mark.parametrize("n", [0, 1, 2, 31, 2047, 2048, 2049, 4095, 4096, 4097, 12289, 100_000, 1_000_003])
@pytest.mark.parametrize("bits", [13, 45])
def test_sort_matches_stable_sort(cuda, n, bits):
    torch = cuda
    rng = np.random.default_rng(n * 7 + bits)
    keys = _keys(rng, n, bits, ties=True)
    vals = np.arange(n, dtype=np.uint32)
    kt = torch.from_numpy(keys.view(np.int64)).cuda()
    vt = torch.from_numpy(vals.view(np.int32)).cuda()
    ko, vo = T.sort_pairs(kt, vt, bits)
    torch.cuda.synchronize()
    order = np.argsort(keys, kind="stable")
    np.testing.assert_array_equal(ko.cpu().numpy().view(np.uint64), keys[order])
    np.testing.assert_array_equal(vo.cpu().numpy().view(np.uint32), vals[order])


@pytest.mark.parametrize("bits", [1, 8, 9, 16, 33, 48, 64])
def test_sort_key_widths_low_bits_only(cuda, bits):
    """Only the low key_bits take part (the reference sorts the low 2P bits);
    higher bits ride along and ties keep input order."""
    torch = cuda
    rng = np.random.default_rng(bits)
    n = 50_000
    keys = rng.integers(0, np.iinfo(np.uint64).max, size=n, dtype=np.uint64, endpoint=True)
    vals = rng.integers(0, 1 << 32, size=n, dtype=np.uint64).astype(np.uint32)
    ko, vo = T.sort_pairs(torch.from_numpy(keys.view(np.int64)).cuda(), torch.from_numpy(vals.view(np.int32)).cuda(), bits)
    torch.cuda.synchronize()
    mask = np.uint64((1 << bits) - 1) if bits < 64 else np.uint64(0xFFFFFFFFFFFFFFFF)
    order = np.argsort(keys & mask, kind="stable")
    np.testing.assert_array_equal(ko.cpu().numpy().view(np.uint64), keys[order])
    np.testing.assert_array_equal(vo.cpu().numpy().view(np.uint32), vals[order])


def test_sort_matches_reference_radix4_on_pipeline_keys(cuda):
    """Keys of a real frame: the restated 4-way radix sort, std::stable_sort and the GPU agree."""
    torch = cuda
    from torpedo_gb300 import configs
    from tests import gpu_helpers as H

    recs = configs.scene("cfg2", 30_000).records
    cam = configs.cameras("cfg2")[0]
    o = H.oracle_frame(recs, cam, f64=False)
    bits = T.key_bits_for_tiles(((cam.width + 15) // 16) * ((cam.height + 15) // 16))
    k4, v4 = O.radix4_sort(o["keys_unsorted"], o["vals_unsorted"], (bits + 1) // 2)
    ko, vo = T.sort_pairs(torch.from_numpy(o["keys_unsorted"].view(np.int64)).cuda(),
                          torch.from_numpy(o["vals_unsorted"].view(np.int32)).cuda(), bits)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(ko.cpu().numpy().view(np.uint64), k4)
    np.testing.assert_array_equal(vo.cpu().numpy().view(np.uint32), v4)
    np.testing.assert_array_equal(k4, o["keys"])


@pytest.mark.parametrize("n", [0, 1, 1023, 1024, 1025, 300_000])
def test_scan_tiles_standalone(cuda, n):
    torch = cuda
    rng = np.random.default_rng(n)
    sp = np.zeros((n, 12), np.uint32)
    sp[:, 3] = rng.integers(0, 40, size=n)
    sp[::11, 3] = 0
    offs, tot = T.scan_tiles(torch.from_numpy(sp.view(np.int32)).cuda())
    torch.cuda.synchronize()
    exp, total = O.scan_tiles(sp)
    np.testing.assert_array_equal(offs.cpu().numpy().view(np.uint32), exp)
    assert int(tot.cpu().numpy().view(np.uint32)[0]) == total
