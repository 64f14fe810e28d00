"""The benchmark workloads at their real sizes, checked against the oracle.

  C2  n = 2^28 DNA with 30% planted repeats, PlainText, u32: bit-exact.
  C4  the sample sort of the C2 text with p = 4096 learned partitions,
      bucketed before the sort: the emitted order bit-exact, the pivots the
      oracle's sorted sample and every bucket's size counted on the oracle's
      suffix array; the reference-rule plan (pivots, sizes) equal to the
      oracle's sample sort.
  C3  n = 2^29 segmented text, the positions with text[p] < 4, u64:
      ShorterFirst equal after canonicalising each tie class (the reference
      leaves the order inside a class unpinned, src/sample_sort.rs:908-934),
      with the GPU's classes in ascending position; with the reference tie
      order requested, bit-exact; the same positions under the STAR
      LongerFirst order (a total order): bit-exact.
  C5  8,192 texts sorted in one batched call: every 8th text and the longest
      one bit-exact against the oracle, text by text.

The oracle is the C restatement (all host cores); each text is generated
once per module.  On top of the oracle comparison every output is checked
for the reference's own validity property (a permutation of the requested
positions in non-decreasing suffix order, src/sample_sort.rs:895-934).
"""
import numpy as np
import pytest

import oracle as orc

pytestmark = pytest.mark.gpu

capssa = pytest.importorskip("capssa")


@pytest.fixture(scope="module")
def ctx():
    c = capssa.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def c2():
    from capssa import workloads
    t = workloads.dna_with_repeats(1 << 28, seed=2)
    return t, orc.build_in_memory(t)


@pytest.fixture(scope="module")
def c3():
    from capssa import workloads
    return workloads.segmented_filtered(1 << 29)


@pytest.fixture(scope="module")
def c3_want(c3):
    """The oracle's ShorterFirst order of C3 (the reference's, ties included)."""
    text, ends, pos = c3
    return orc.build_in_memory(text, pos, orc.Limits(len(text), ends), index=np.uint64)


def test_c2_bench_text_2p28_bit_exact(ctx, c2):
    t, want = c2
    got = ctx.build_in_memory(t)
    assert got.dtype == np.uint32 and len(got) == len(t)
    assert np.array_equal(got, want)


def test_c4_learned_sample_sort_2p28_bit_exact(ctx, c2):
    from test_gpu_partition import pf_expected_plan, sizes_between
    t, want = c2
    opts = capssa.ExtMemOpts(subproblem_count=4096, partition=capssa.Partition.LEARNED)
    got = ctx.build_in_memory_sample_sort(t, opts)
    assert got.dtype == np.uint64
    assert np.array_equal(got, want.astype(np.uint64))
    del got
    cmp = orc.adjacent_cmp(t, want, orc.Limits(len(t)))
    ends, sizes = pf_expected_plan(t, orc.Limits(len(t)), 4096, want)
    k, pv, sz = ctx.sample_sort_plan(t, capssa.ExtMemOpts(subproblem_count=4096))
    assert k == 4096
    assert np.array_equal(sz.astype(np.int64), sizes)
    assert np.array_equal(sizes_between(want, cmp, pv)[1], ends)  # the same pivots
    k, pv, sz = ctx.sample_sort_plan(t, opts)  # learned: pivots where the model steps
    st = ctx.stats()
    assert k == 4096
    assert np.array_equal(sz.astype(np.int64), sizes_between(want, cmp, pv)[0])
    assert st["mispredicted"] < 0.1 * len(t)
    del cmp
    _, kp, opv, osz = orc.sample_sort(t, subproblem_count=4096)
    for part in (capssa.Partition.LEARNED, capssa.Partition.SPLITTERS):
        k, pv, sz = ctx.sample_sort_plan(t, capssa.ExtMemOpts(
            subproblem_count=4096, partition=part, sampling=capssa.Sampling.REFERENCE))
        assert k == kp == 4096
        assert np.array_equal(pv, opv[:k - 1])
        assert np.array_equal(sz, osz[:k])


def test_c2_small_subset_2p28_sorted_alone(ctx, c2):
    """2^16 positions of the 2^28-symbol text: sorted on their own, bit-exact,
    in a small fraction of the whole-text build's device time."""
    import torch
    t, _ = c2
    rng = np.random.default_rng(65)
    pos = np.sort(rng.choice(len(t), size=1 << 16, replace=False)).astype(np.uint32)
    want = orc.build_in_memory(t, pos)
    got = ctx.build_in_memory_for_positions(t, pos)
    assert ctx.stats()["sparse_subset"] == 1
    assert np.array_equal(got, want)
    td = torch.from_numpy(t).cuda()
    pd = torch.from_numpy(pos.view(np.int32)).cuda()
    out = torch.empty(len(pos), dtype=torch.int32, device="cuda")
    full = torch.empty(len(t), dtype=torch.int32, device="cuda")
    ctx.build_in_memory_for_positions(td, pd, out=out)
    ctx.build_in_memory(td, out=full)
    ctx.build_in_memory_for_positions(td, pd, out=out)
    sub_ms = ctx.stats()["device_ms"]
    ctx.build_in_memory(td, out=full)
    full_ms = ctx.stats()["device_ms"]
    print("subset of 2^16: %.2f ms, whole text: %.2f ms" % (sub_ms, full_ms))
    assert sub_ms < full_ms / 4


def test_c3_segmented_filtered_2p29(ctx, c3, c3_want):
    text, ends, pos = c3
    n = len(text)
    lp = capssa.SegmentedText(n, ends)
    lo = orc.Limits(n, ends)
    got = ctx.build_in_memory_for_positions(text, pos, lp)
    assert got.dtype == np.uint64 and len(got) == len(pos)
    want = c3_want
    cw = orc.adjacent_cmp(text, want, lo)
    assert (cw <= 0).all()
    canon = orc.canonical_ties(want, cw)
    assert np.array_equal(orc.canonical_ties(got, cw), canon)
    assert np.array_equal(got, canon)  # GPU tie classes in ascending position
    del canon
    # the filter source gives the same order
    f = ctx.build_in_memory_for_filter(text, 0, 4, lp=lp, index=np.uint64)
    assert np.array_equal(f, got)


def test_c3_reference_tie_order_2p29_bit_exact(ctx, c3, c3_want):
    """The same positions in the reference's own tie order: the output equals
    the oracle's merge sort element for element."""
    text, ends, pos = c3
    lp = capssa.SegmentedText(len(text), ends)
    opts = capssa.Opts(tie_order=capssa.TieOrder.REFERENCE)
    got = ctx.build_in_memory_for_positions(text, pos, lp, opts)
    st = ctx.stats()
    print("C3 tie classes %d, reference tie order %.2f ms of %.2f ms" %
          (st["tie_classes"], st["tie_order_ms"], st["device_ms"]))
    assert st["tie_classes"] > 0
    assert np.array_equal(got, c3_want)


def test_c3_star_order_2p29_bit_exact(ctx, c3):
    text, ends, pos = c3
    n = len(text)
    lp = capssa.SegmentedText(n, ends, capssa.BoundaryRank.LONGER_FIRST)
    got = ctx.build_in_memory_for_positions(text, pos, lp)
    want = orc.build_in_memory(text, pos, orc.Limits(n, ends, longer_first=True),
                               index=np.uint64)
    assert np.array_equal(got, want)


def test_c5_batched_8192_texts(ctx):
    from capssa import workloads
    cat, offs = workloads.batched_texts()
    got = ctx.build_batched(cat, offs)
    lens = np.diff(offs.astype(np.int64))
    sample = sorted(set(range(0, len(lens), 8)) | {int(np.argmax(lens))})
    assert len(sample) >= 1024
    for i in sample:
        a, b = int(offs[i]), int(offs[i + 1])
        want = orc.build_in_memory(np.ascontiguousarray(cat[a:b]))
        assert np.array_equal(got[a:b], want), i
