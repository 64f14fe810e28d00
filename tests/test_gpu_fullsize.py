"""Full-size properties: the bench workloads at their real sizes, checked by
size-independent properties instead of the oracle (which would take hours).
Each suffix array must be a permutation of the requested positions, and every
adjacent pair must be ordered under suffix_cmp_with (src/lcp.rs:184-201).
The pair check runs through the library's warp-LCP comparison kernels, which
share no code with the sort."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

capssa = pytest.importorskip("capssa")


@pytest.fixture(scope="module")
def ctx():
    c = capssa.Context(0)
    yield c
    c.close()


def test_bench_workload_2p28_plain(ctx):
    """n = 2^28 DNA with 30% planted repeats, PlainText, u32: a permutation of
    0..n-1 in strictly increasing suffix order (PlainText suffixes never tie)."""
    from capssa import workloads
    n = 1 << 28
    t = workloads.dna_with_repeats(n, seed=2)
    sa = ctx.build_in_memory(t)
    assert sa.dtype == np.uint32 and len(sa) == n
    seen = np.zeros(n, dtype=bool)
    seen[sa] = True
    assert seen.all()
    cmp = ctx.suffix_cmp(t, sa[:-1].astype(np.uint64), sa[1:].astype(np.uint64))
    assert (cmp == -1).all()


def test_segmented_filtered_2p29(ctx):
    """n = 2^29 segmented text (lognormal segments, long runs), the positions
    with text[p] < 4 through the GPU filter source, u64: exactly the kept
    positions, non-decreasing under the segmented comparator (ties allowed,
    src/sample_sort.rs:908-934)."""
    from capssa import workloads
    text, ends, pos = workloads.segmented_filtered(1 << 29)
    n = len(text)
    lp = capssa.SegmentedText(n, ends)
    got = ctx.build_in_memory_for_filter(text, 0, 4, lp=lp, index=np.uint64)
    assert len(got) == len(pos)
    mark = np.zeros(n, dtype=bool)
    mark[got] = True
    assert mark.sum() == len(pos) and mark[pos].all()
    cmp = ctx.suffix_cmp(text, got[:-1], got[1:], lp)
    assert (cmp <= 0).all()
