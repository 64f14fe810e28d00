"""The allocation-free merge entry point (capssa_merge_noalloc_u8_u32).

It serves callers that cannot call cudaMalloc where they merge (their own
pool allocator owns the device memory, or an allocation's synchronisation is
not acceptable on that stream): every buffer is theirs and the merge-path
scratch is a static device array.  This test calls it through the C ABI
several times in a row and checks every result against the allocating entry
point (capssa_merge_u8_u32) and against the oracle's merge — bit-exact, the
tolerance of every integer test here — under both boundary orders, plus the
one-sided merges and the contract checks.
The file sorts last so a stop-at-first-failure run has run everything else.
"""
import ctypes as C

import numpy as np
import pytest

import oracle as orc

pytestmark = pytest.mark.gpu

capssa = pytest.importorskip("capssa")
torch = pytest.importorskip("torch")

SHORTER, LONGER = 0, 1


def _fn():
    f = capssa.lib.capssa_merge_noalloc_u8_u32
    vp, u64 = C.c_void_p, C.c_uint64
    f.argtypes = [vp, vp, u64, vp, u64, C.c_int32, vp, vp, u64, vp, vp, u64, u64, vp, vp]
    f.restype = C.c_int
    return f


def _case(seed, n, segmented, boundary=SHORTER, split=3):
    rng = np.random.default_rng(seed)
    t = rng.integers(0, 3, n).astype(np.uint8)
    ends = None
    if segmented:
        e = np.cumsum(rng.integers(2, 40, n))
        ends = np.array(e[e < n].tolist() + [n], dtype=np.uint64)
    lo = orc.Limits(n, ends, longer_first=boundary == LONGER)
    perm = rng.permutation(n).astype(np.uint32)
    h = n // split if split else 0
    x, lx = orc.build_in_memory(t, perm[:h], lo, with_lcp=True)
    y, ly = orc.build_in_memory(t, perm[h:], lo, with_lcp=True)
    return t, ends, lo, x, lx, y, ly


def _dev(a, dtype):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda").view(dtype)


def _noalloc(f, t, ends, x, lx, y, ly, boundary=SHORTER):
    n = len(t)
    text = torch.zeros(n + 64, dtype=torch.uint8, device="cuda")  # 64 readable bytes past the end
    text[:n] = torch.from_numpy(t).to("cuda")
    d_ends = _dev(ends.view(np.int64), torch.int64) if ends is not None else None

    def buf(a):
        if len(a) == 0:
            return None, 0
        d = _dev(a.view(np.int32), torch.int32)
        return d, d.data_ptr()

    dx, px = buf(x)
    dlx, plx = buf(lx)
    dy, py = buf(y)
    dly, ply = buf(ly)
    z = torch.empty(len(x) + len(y), dtype=torch.int32, device="cuda")
    lz = torch.empty_like(z)
    stream = torch.cuda.current_stream().cuda_stream
    st = f(stream, text.data_ptr(), n, d_ends.data_ptr() if d_ends is not None else None,
           len(ends) if ends is not None else 0, boundary, px, plx, len(x), py, ply, len(y),
           (1 << 64) - 1, z.data_ptr(), lz.data_ptr())
    return st, z.cpu().numpy().view(np.uint32), lz.cpu().numpy().view(np.uint32)


def _lp(n, ends, boundary):
    b = capssa.BoundaryRank.LONGER_FIRST if boundary == LONGER else capssa.BoundaryRank.SHORTER_FIRST
    return capssa.SegmentedText(n, ends, b) if ends is not None else capssa.PlainText(n, b)


def test_noalloc_merge_matches_allocating_merge_and_oracle():
    torch.cuda.init()
    f = _fn()
    cases = (  # several calls in a row: both boundary orders, plain and segmented
        (11, 20000, False, SHORTER), (12, 9000, True, SHORTER),
        (14, 12000, False, LONGER), (15, 7000, True, LONGER),
    )
    with capssa.Context(0) as ctx:
        for seed, n, seg, bd in cases:
            t, ends, lo, x, lx, y, ly = _case(seed, n, seg, bd)
            st, z, lz = _noalloc(f, t, ends, x, lx, y, ly, bd)
            assert st == 0
            wz, wlz = ctx.merge(t, x, lx, y, ly, _lp(n, ends, bd))
            assert np.array_equal(z, wz)
            assert np.array_equal(lz, wlz)
            oz, olz = orc.merge(t, x, lx, y, ly, lo)
            assert np.array_equal(z, oz)
            assert np.array_equal(lz, olz)


def test_noalloc_merge_one_sided_runs_copy():
    f = _fn()
    for split in (0, 1):  # x empty, then y empty
        t, ends, lo, x, lx, y, ly = _case(16, 3000, True, SHORTER, split=split)
        st, z, lz = _noalloc(f, t, ends, x, lx, y, ly)
        assert st == 0
        oz, olz = orc.merge(t, x, lx, y, ly, lo)
        assert np.array_equal(z, oz)
        assert np.array_equal(lz, olz)


def test_noalloc_merge_rejects_contract_violations():
    f = _fn()
    t, ends, lo, x, lx, y, ly = _case(13, 500, False)
    bad = x.copy()
    bad[0] = 10_000  # position beyond the text
    st, _, _ = _noalloc(f, t, ends, bad, lx, y, ly)
    assert st == 1  # CAPSSA_EINVAL
    t, ends, lo, x, lx, y, ly = _case(17, 600, True)
    for broken in (ends[::-1].copy(), np.append(ends[:-1], ends[-1] - 1).astype(np.uint64)):
        st, _, _ = _noalloc(f, t, broken, x, lx, y, ly)  # non-increasing ends / last end != n
        assert st == 1
    st, _, _ = _noalloc(f, t, ends, x, lx, y, ly, boundary=7)  # unknown boundary order
    assert st == 1
    # oversize merges are refused before any work (no device buffers read),
    # including lengths whose sum would wrap around
    st = f(None, None, 0, None, 0, 0, None, None, (1 << 24), None, None, 1, 0, None, None)
    assert st == 1
    st = f(None, None, 0, None, 0, 0, None, None, 2, None, None, (1 << 64) - 1, 0, None, None)
    assert st == 1
    # the scratch still serves a valid merge after the refusals
    t, ends, lo, x, lx, y, ly = _case(18, 4000, False)
    st, z, lz = _noalloc(f, t, ends, x, lx, y, ly)
    assert st == 0
    oz, olz = orc.merge(t, x, lx, y, ly, lo)
    assert np.array_equal(z, oz) and np.array_equal(lz, olz)
