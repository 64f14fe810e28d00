"""The allocation-free merge entry point (capssa_merge_noalloc_u8_u32).

It serves callers that cannot call cudaMalloc where they merge (their own
pool allocator owns the device memory, or an allocation's synchronisation is
not acceptable on that stream): every buffer is theirs and the merge-path
scratch is a static device array.  This test calls it through the C ABI
twice in a row and checks both results against the allocating entry point
(capssa_merge_u8_u32) — bit-exact, the tolerance of every integer test here.
The file sorts last so a stop-at-first-failure run has run everything else.
"""
import ctypes as C

import numpy as np
import pytest

import oracle as orc

pytestmark = pytest.mark.gpu

capssa = pytest.importorskip("capssa")
torch = pytest.importorskip("torch")


def _fn():
    f = capssa.lib.capssa_merge_noalloc_u8_u32
    vp, u64 = C.c_void_p, C.c_uint64
    f.argtypes = [vp, vp, u64, vp, u64, C.c_int32, vp, vp, u64, vp, vp, u64, u64, vp, vp]
    f.restype = C.c_int
    return f


def _case(seed, n, segmented):
    rng = np.random.default_rng(seed)
    t = rng.integers(0, 3, n).astype(np.uint8)
    ends = None
    if segmented:
        e = np.cumsum(rng.integers(2, 40, n))
        ends = np.array(e[e < n].tolist() + [n], dtype=np.uint64)
    lo = orc.Limits(n, ends)
    perm = rng.permutation(n).astype(np.uint32)
    h = n // 3
    x, lx = orc.build_in_memory(t, perm[:h], lo, with_lcp=True)
    y, ly = orc.build_in_memory(t, perm[h:], lo, with_lcp=True)
    return t, ends, x, lx, y, ly


def _dev(a, dtype):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda").view(dtype)


def _noalloc(f, t, ends, x, lx, y, ly):
    n = len(t)
    text = torch.zeros(n + 64, dtype=torch.uint8, device="cuda")  # 64 readable bytes past the end
    text[:n] = torch.from_numpy(t).to("cuda")
    d_ends = _dev(ends.view(np.int64), torch.int64) if ends is not None else None
    dx, dlx = _dev(x.view(np.int32), torch.int32), _dev(lx.view(np.int32), torch.int32)
    dy, dly = _dev(y.view(np.int32), torch.int32), _dev(ly.view(np.int32), torch.int32)
    z = torch.empty(len(x) + len(y), dtype=torch.int32, device="cuda")
    lz = torch.empty_like(z)
    stream = torch.cuda.current_stream().cuda_stream
    st = f(stream, text.data_ptr(), n, d_ends.data_ptr() if d_ends is not None else None,
           len(ends) if ends is not None else 0, 0, dx.data_ptr(), dlx.data_ptr(), len(x),
           dy.data_ptr(), dly.data_ptr(), len(y), (1 << 64) - 1, z.data_ptr(), lz.data_ptr())
    return st, z.cpu().numpy().view(np.uint32), lz.cpu().numpy().view(np.uint32)


def test_noalloc_merge_matches_allocating_merge_twice():
    torch.cuda.init()
    f = _fn()
    with capssa.Context(0) as ctx:
        for seed, n, seg in ((11, 20000, False), (12, 9000, True)):  # two calls in a row
            t, ends, x, lx, y, ly = _case(seed, n, seg)
            st, z, lz = _noalloc(f, t, ends, x, lx, y, ly)
            assert st == 0
            lp = capssa.SegmentedText(n, ends) if seg else capssa.PlainText(n)
            wz, wlz = ctx.merge(t, x, lx, y, ly, lp)
            assert np.array_equal(z, wz)
            assert np.array_equal(lz, wlz)


def test_noalloc_merge_rejects_contract_violations():
    f = _fn()
    t, ends, x, lx, y, ly = _case(13, 500, False)
    x = x.copy()
    x[0] = 10_000  # position beyond the text
    st, _, _ = _noalloc(f, t, ends, x, lx, y, ly)
    assert st == 1  # CAPSSA_EINVAL
    # oversize merges are refused before any work (no device buffers read)
    st = f(None, None, 0, None, 0, 0, None, None, (1 << 24), None, None, 1, 0, None, None)
    assert st == 1
