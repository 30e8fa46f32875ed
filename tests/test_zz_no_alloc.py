"""The scan entry point that allocates nothing (vkvg_gb300_exclusive_scan_noalloc).

Collected last, so it runs both alone and after every other test in one
process.  Each check makes two calls in a row through the C ABI: the second
reuses the fixed scratch the first one left behind.  The reference for its
results is the library's own pipeline scan, read back through the existing
vkvg_gb300_debug_subpaths entry point (subpath first-point offsets are the
pipeline's exclusive scan of the flattened point counts), plus the definition
(numpy cumsum, uint32 arithmetic) on sizes from one item to the limit."""
import numpy as np
import pytest

import parity_util as pu
from vkvg_gb300 import scenes

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _dev_u32(a):
    return torch.from_numpy(np.ascontiguousarray(a, np.uint32).view(np.int32)).cuda()


def _scan_twice(gb, counts):
    """two consecutive no-alloc scans of counts; returns both results (uint32, n + 1)"""
    n = int(counts.size)
    d_in = _dev_u32(counts) if n else torch.zeros(1, dtype=torch.int32, device="cuda")
    d_out = torch.empty(n + 1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    got = []
    for _ in range(2):
        d_out.fill_(-1)
        st = gb.exclusive_scan_noalloc(d_in.data_ptr(), n, d_out.data_ptr(), stream)
        torch.cuda.synchronize()
        assert st == 0
        got.append(d_out.cpu().numpy().view(np.uint32).copy())
    return got


def _excl(counts):
    c = np.ascontiguousarray(counts, np.uint64)
    out = np.zeros(c.size + 1, np.uint64)
    np.cumsum(c, out=out[1:])
    return (out & 0xFFFFFFFF).astype(np.uint32)


def test_noalloc_scan_matches_pipeline_scan(gb):
    sc = scenes.curve_heavy(n_paths=48, size=256, seed=7, n_min=2, n_max=12)
    dev, surf, ctx = pu.run_gpu(gb, sc)
    first, count, _ = ctx.debug_subpaths()
    assert count.size > 40
    # the existing path's offsets are its exclusive scan of the point counts
    assert first[0] == 0 and np.array_equal(first[1:], (np.cumsum(count.astype(np.uint64))[:-1]).astype(np.uint32))
    for got in _scan_twice(gb, count):
        assert np.array_equal(got[:-1], first)
        assert got[-1] == int(first[-1]) + int(count[-1])
    ctx.destroy()
    surf.destroy()
    dev.destroy()


@pytest.mark.parametrize("n", [0, 1, 4095, 4096, 4097, 1_000_003, 1 << 26])
def test_noalloc_scan_sizes(gb, n):
    rng = np.random.default_rng(n)
    counts = rng.integers(0, 1 << 12, n, dtype=np.uint32)
    if n == 1 << 26:
        counts[::4096] = 0xFFFFFFFF  # totals wrap modulo 2^32
    want = _excl(counts)
    for got in _scan_twice(gb, counts):
        assert np.array_equal(got, want)


def test_noalloc_scan_rejects_oversize(gb):
    n = gb.SCAN_NOALLOC_MAX + 1
    d_out = torch.full((2,), -1, dtype=torch.int32, device="cuda")
    d_in = torch.zeros(1, dtype=torch.int32, device="cuda")
    for _ in range(2):
        st = gb.exclusive_scan_noalloc(d_in.data_ptr(), n, d_out.data_ptr(), 0)
        assert st == 1  # VKVG_STATUS_NO_MEMORY, nothing launched
    torch.cuda.synchronize()
    assert d_out.cpu().tolist() == [-1, -1]
