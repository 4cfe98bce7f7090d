"""The key sort's tile-id digit counts, taken row by row over tile rectangles
(count_tile_row in torpedo_gb300/csrc/preprocess.cu), restated in Python and
checked against counting every tile id: rows shorter and longer than 256 ids,
low digits that wrap round all 256 values, and tile ids of up to 4 digits."""
import numpy as np


def count_rows(rows, ndig):
    """The CUDA function's steps: digit 0 through a difference array over the
    256 values (+ a count added to every value), digits p >= 1 per value of
    t >> 8p, all in 32-bit unsigned arithmetic."""
    diff = np.zeros(257, np.uint64)
    every = 0
    hist = np.zeros((3, 256), np.uint64)
    m32 = (1 << 32) - 1
    for a0, w in rows:
        if w >= 256:
            every += w >> 8
        rem = w & 255
        if rem:
            st = a0 & 255
            e = st + rem
            diff[st] = (int(diff[st]) + 1) & m32
            if e <= 256:
                diff[e] = (int(diff[e]) + m32) & m32  # -1 (diff[256] is never read)
            else:
                diff[0] = (int(diff[0]) + 1) & m32
                diff[e - 256] = (int(diff[e - 256]) + m32) & m32
        last = a0 + w - 1
        for p in range(1, ndig):
            sh = 8 * p
            v0, v1 = a0 >> sh, last >> sh
            if v0 == v1:
                hist[p - 1][v0 & 255] += w
            else:
                hist[p - 1][v0 & 255] += ((v0 + 1) << sh) - a0
                for v in range(v0 + 1, v1):
                    hist[p - 1][v & 255] += 1 << sh
                hist[p - 1][v1 & 255] += last - (v1 << sh) + 1
    out = np.zeros((ndig, 256), np.uint64)
    out[0] = (np.cumsum(diff[:256]) + every) & m32
    out[1:ndig] = hist[:ndig - 1]
    return out


def brute(rows, ndig):
    out = np.zeros((ndig, 256), np.uint64)
    for a0, w in rows:
        t = np.arange(a0, a0 + w, dtype=np.uint64)
        for p in range(ndig):
            out[p] += np.bincount(((t >> np.uint64(8 * p)) & np.uint64(255)).astype(np.int64), minlength=256).astype(
                np.uint64)
    return out


def test_row_counts_match_every_tile_id():
    rng = np.random.default_rng(5)
    for tile_bits, wmax in ((9, 40), (13, 120), (19, 300), (26, 2000), (31, 70000)):
        ndig = (tile_bits + 7) // 8
        rows = []
        for _ in range(300):
            w = int(rng.integers(1, wmax + 1))
            a0 = int(rng.integers(0, (1 << tile_bits) - w + 1))
            rows.append((a0, w))
        rows += [(255, 2), (0, 256), (1, 256), (250, 263), (511, 1)]  # wraps and exact multiples
        rows = [(a0, w) for a0, w in rows if a0 + w <= (1 << tile_bits)]
        np.testing.assert_array_equal(count_rows(rows, ndig), brute(rows, ndig))
