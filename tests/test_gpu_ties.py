"""The reference's order inside tie classes (capssa_opts.tie_order =
CAPSSA_TIES_REFERENCE), against the oracle's merge sort without any
canonicalisation.

Under SegmentedText with ShorterFirst, suffixes with equal symbols up to equal
limits compare Equal and the reference emits them in its merge sort's order
(src/sample_sort.rs:221-266, 430-497).  The oracle restates that merge sort,
so its output order is the reference's: every case here is np.array_equal.
The default order (ascending input order) is checked to stay as it was.
"""
import numpy as np
import pytest

import oracle as orc

pytestmark = pytest.mark.gpu

capssa = pytest.importorskip("capssa")

REF = capssa.TieOrder.REFERENCE


@pytest.fixture(scope="module")
def ctx():
    c = capssa.Context(0)
    yield c
    c.close()


def _seg(rng, n_seg, lmin, lmax, sigma):
    lengths = rng.integers(lmin, lmax + 1, n_seg)
    ends = np.cumsum(lengths).astype(np.uint64)
    t = rng.integers(0, sigma, int(ends[-1])).astype(np.uint8)
    return t, ends


def _check(ctx, t, ends, positions=None, max_ctx=orc.UNBOUNDED, index=np.uint32):
    n = len(t)
    lp = capssa.SegmentedText(n, ends)
    lo = orc.Limits(n, ends)
    opts = capssa.Opts(max_context=max_ctx, tie_order=REF)
    if positions is None:
        got = ctx.build_in_memory(t, lp, opts, index=index)
        want = orc.build_in_memory(t, None, lo, max_ctx, index=index)
    else:
        pos = np.asarray(positions, dtype=index)
        got = ctx.build_in_memory_for_positions(t, pos, lp, opts)
        want = orc.build_in_memory(t, pos, lo, max_ctx, index=index)
    assert got.dtype == want.dtype
    assert np.array_equal(got, want)
    return ctx.stats()


@pytest.mark.parametrize("index", [np.uint32, np.uint64])
def test_reference_tie_order_random_segmented(ctx, index):
    rng = np.random.default_rng(0x71E5)
    classes = 0
    for trial in range(60):
        t, ends = _seg(rng, int(rng.integers(1, 80)), 1, 12, int(rng.integers(1, 4)))
        st = _check(ctx, t, ends, index=index)
        classes += st["tie_classes"]
    assert classes > 500  # the cases do have ties


def test_reference_tie_order_subsets_repeats_and_empty_suffix(ctx):
    rng = np.random.default_rng(0x5B5E7)
    for trial in range(60):
        t, ends = _seg(rng, int(rng.integers(1, 60)), 1, 10, int(rng.integers(1, 4)))
        n = len(t)
        kind = trial % 3
        if kind == 0:  # distinct, unsorted
            pos = rng.permutation(n)[: max(1, (2 * n) // 3)]
        elif kind == 1:  # repeats and the empty suffix n
            pos = rng.integers(0, n + 1, max(1, n // 2))
        else:  # distinct, ascending (the filter shape)
            pos = np.sort(rng.permutation(n)[: max(1, n // 2)])
        _check(ctx, t, ends, positions=pos, index=np.uint32 if trial % 2 else np.uint64)


@pytest.mark.parametrize("max_ctx", [0, 1, 3, 7])
def test_reference_tie_order_finite_context(ctx, max_ctx):
    rng = np.random.default_rng(0xC7 + max_ctx)
    for trial in range(20):
        t, ends = _seg(rng, int(rng.integers(1, 60)), 1, 15, int(rng.integers(1, 4)))
        _check(ctx, t, ends, max_ctx=max_ctx)
        pos = rng.integers(0, len(t) + 1, max(1, len(t) // 2))
        _check(ctx, t, ends, positions=pos, max_ctx=max_ctx)


def test_reference_tie_order_lcp_unchanged(ctx):
    rng = np.random.default_rng(0x1C9)
    t, ends = _seg(rng, 400, 1, 9, 2)
    n = len(t)
    lp = capssa.SegmentedText(n, ends)
    lo = orc.Limits(n, ends)
    sa, lcp = ctx.build_in_memory_lcp(t, None, lp, capssa.Opts(tie_order=REF))
    wsa, wlcp = orc.build_in_memory(t, None, lo, with_lcp=True)
    assert np.array_equal(sa, wsa)
    assert np.array_equal(lcp, wlcp)


def test_default_tie_order_is_ascending_input_order(ctx):
    rng = np.random.default_rng(0xD3F)
    t, ends = _seg(rng, 300, 1, 8, 2)
    n = len(t)
    lo = orc.Limits(n, ends)
    got = ctx.build_in_memory(t, capssa.SegmentedText(n, ends))
    assert ctx.stats()["tie_classes"] == 0  # the pass did not run
    want = orc.build_in_memory(t, None, lo)
    cmp = orc.adjacent_cmp(t, want, lo)
    assert np.array_equal(got, orc.canonical_ties(want, cmp))


def test_reference_tie_order_large_classes(ctx):
    """2^21 symbols in segments of 1-6 over two letters: classes of tens of
    thousands of members, split at every merge-tree level, and walks that run
    out of budget (the scan fallback)."""
    rng = np.random.default_rng(0xB16)
    t, ends = _seg(rng, 600_000, 1, 6, 2)
    t = t[: 1 << 21].copy()
    ends = ends[ends < len(t)]
    ends = np.append(ends, len(t)).astype(np.uint64)
    st = _check(ctx, t, ends)
    assert st["tie_classes"] > 50
    pos = rng.permutation(len(t))[: len(t) // 2]
    _check(ctx, t, ends, positions=pos, index=np.uint64)
