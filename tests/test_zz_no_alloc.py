"""tpd_scan_tiles_static (scratch in the library's own device memory, no
workspace) through the C ABI: on two calls in a row on different inputs its
offsets and totals equal those of tpd_scan_tiles (caller workspace) and a
numpy exclusive prefix sum, bit for bit, with a clean device status; a
look-back that never completes (test hook) is reported in the status; sizes
above TPD_SCAN_STATIC_MAX_SPLATS are refused before any device work.
Collected last so it runs both after the other GPU tests and alone."""
import numpy as np
import pytest

from torpedo_gb300 import _lib as L

pytestmark = pytest.mark.gpu

MAX_SPLATS = 1 << 24  # TPD_SCAN_STATIC_MAX_SPLATS in include/tpdsplat.h


def _splats(torch, rng, n):
    s = np.zeros((n, 12), dtype=np.uint32)
    s[:, 3] = rng.integers(0, 65, size=n, dtype=np.uint32)
    s[rng.random(n) < 0.3, 3] = 0  # culled splats
    return torch.from_numpy(s.view(np.int32)).cuda()


def _numpy_scan(sp):
    counts = sp[:, 3].cpu().numpy().view(np.uint32).astype(np.uint64)
    excl = np.concatenate(([0], np.cumsum(counts)[:-1])).astype(np.uint64) if counts.size else counts
    return excl.astype(np.uint32), int(counts.sum())


def _scan_workspace(torch, lib, sp, stream):
    n = sp.shape[0]
    ws = torch.empty(max(1, int(lib.tpd_scan_workspace_size(n))), dtype=torch.uint8, device="cuda")
    offs = torch.full((max(1, n),), -1, dtype=torch.int32, device="cuda")
    tot = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    rc = lib.tpd_scan_tiles(sp.data_ptr(), n, offs.data_ptr(), tot.data_ptr(), ws.data_ptr(), ws.numel(), stream)
    assert rc == L.TPD_OK, L.status_string(rc)
    return offs, tot, ws


def _scan_static(torch, lib, sp, stream):
    n = sp.shape[0]
    offs = torch.full((max(1, n),), -1, dtype=torch.int32, device="cuda")
    tot = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    status = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    rc = lib.tpd_scan_tiles_static(sp.data_ptr(), n, offs.data_ptr(), tot.data_ptr(), status.data_ptr(), stream)
    assert rc == L.TPD_OK, L.status_string(rc)
    return offs, tot, status


def test_static_scan_matches_workspace_scan_twice(cuda):
    torch = cuda
    lib = L.load()
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(2024)
    for n in (1_000_003, 4097):  # two calls in a row, the second smaller than the first
        sp = _splats(torch, rng, n)
        o_ref, t_ref, ws = _scan_workspace(torch, lib, sp, stream)
        o_st, t_st, st = _scan_static(torch, lib, sp, stream)
        torch.cuda.synchronize()
        o_np, t_np = _numpy_scan(sp)
        assert int(st.item()) == 0
        assert int(ws[:4].view(torch.int32).item()) == 0
        assert int(t_st.item()) == int(t_ref.item()) == t_np
        np.testing.assert_array_equal(o_st.cpu().numpy().view(np.uint32), o_np)
        np.testing.assert_array_equal(o_st.cpu().numpy(), o_ref.cpu().numpy())


def test_static_scan_edge_sizes(cuda):
    torch = cuda
    lib = L.load()
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(7)
    for n in (0, 1, 1023, 1024, 1025):
        sp = _splats(torch, rng, n) if n else torch.zeros((0, 12), dtype=torch.int32, device="cuda")
        o_ref, t_ref, _ = _scan_workspace(torch, lib, sp, stream)
        o_st, t_st, st = _scan_static(torch, lib, sp, stream)
        torch.cuda.synchronize()
        o_np, t_np = _numpy_scan(sp)
        assert int(st.item()) == 0
        assert int(t_st.item()) == int(t_ref.item()) == t_np
        if n:
            np.testing.assert_array_equal(o_st.cpu().numpy()[:n].view(np.uint32), o_np)
            np.testing.assert_array_equal(o_st.cpu().numpy(), o_ref.cpu().numpy())


def test_static_scan_reports_a_lookback_that_runs_out(cuda):
    """Partition 0 never publishes (test hook, a flag nothing sets): partition
    1's bounded wait runs out and both scans report it; the context stays
    usable and the next call is clean again."""
    torch = cuda
    lib = L.load()
    stream = torch.cuda.current_stream().cuda_stream
    sp = _splats(torch, np.random.default_rng(3), 5000)  # 5 partitions of 1024 splats
    lib.tpd_test_set_never_publish(1)
    try:
        _, _, ws = _scan_workspace(torch, lib, sp, stream)
        _, _, st = _scan_static(torch, lib, sp, stream)
        torch.cuda.synchronize()
    finally:
        lib.tpd_test_set_never_publish(0)
    assert int(st.item()) & L.DEVSTAT_LOOKBACK_TIMEOUT
    assert int(ws[:4].view(torch.int32).item()) & L.DEVSTAT_LOOKBACK_TIMEOUT
    o_st, t_st, st = _scan_static(torch, lib, sp, stream)
    torch.cuda.synchronize()
    o_np, t_np = _numpy_scan(sp)
    assert int(st.item()) == 0 and int(t_st.item()) == t_np
    np.testing.assert_array_equal(o_st.cpu().numpy().view(np.uint32), o_np)


def test_static_scan_refuses_oversize(cuda):
    torch = cuda
    lib = L.load()
    buf = torch.zeros(16, dtype=torch.int32, device="cuda")  # never read: the size check comes first
    rc = lib.tpd_scan_tiles_static(buf.data_ptr(), MAX_SPLATS + 1, buf.data_ptr(), buf.data_ptr(), None, None)
    assert rc == L.TPD_ERR_CAPACITY
