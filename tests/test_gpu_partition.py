"""GPU tests of the sample sort's partition plan and the learned CDF model.

The plan (p, pivots, partition sizes) is compared with the oracle's
restatement of build_in_memory_sample_sort (src/ext_mem.rs:1191-1428); the
learned partition must reproduce the splitter partition exactly; the model's
GPU gradients are checked against the oracle's (relative 1e-4 of the largest
component, FP32 against double accumulation)."""
import math

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


def _dna(n, seed):
    from capssa import workloads
    return workloads.dna_with_repeats(n, seed=seed)


# ---------------------------------------------------------------- model

def test_cdf_grad_matches_oracle(ctx):
    rng = np.random.default_rng(11)
    for n in (1, 31, 1000, 70000):
        params = rng.normal(0, 0.4, capssa.CDF_PARAMS).astype(np.float32)
        x = rng.integers(0, 2 ** 64 - 1, n, dtype=np.uint64)
        t = rng.random(n).astype(np.float32)
        loss, g = ctx.cdf_grad(params, x, t)
        want_loss, want = orc.cdf_loss_grad(params, x, t)
        scale = max(1e-12, float(np.max(np.abs(want))))
        assert np.max(np.abs(g - want)) <= 1e-4 * scale, (n, np.max(np.abs(g - want)), scale)
        assert abs(loss - want_loss) <= 1e-4 * max(1.0, want_loss)


def _bf16(a):
    """float32 values rounded to the nearest BF16 (ties to even)."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def test_cdf_tensor_core_inference_matches_oracle(ctx):
    """The learned partition's inference (BF16 weights, layer 1 on the
    tensor cores with every input split into two BF16 parts, fp32 layer 2)
    against the oracle's double-precision forward pass of the same
    BF16-rounded weights: within 1e-4 of the output scale, on prefixes
    spread over the whole key range and on a trained CDF."""
    rng = np.random.default_rng(14)
    for scale in (0.3, 2.0):
        params = _bf16(rng.normal(0, scale, capssa.CDF_PARAMS))
        x = rng.integers(0, 2 ** 64 - 1, 5000, dtype=np.uint64)
        got = ctx.cdf_infer(params, x)
        want = orc.cdf_forward(params, x)
        tol = 1e-4 * max(1.0, float(np.max(np.abs(want))))
        assert np.max(np.abs(got - want)) <= tol, (scale, np.max(np.abs(got - want)))
    xs = np.sort(rng.integers(0, 2 ** 64 - 1, 65536, dtype=np.uint64))
    ts = ((np.arange(len(xs)) + 0.5) / len(xs)).astype(np.float32)
    params, _ = ctx.cdf_train(xs, ts, steps=100)
    params = _bf16(params)
    got = ctx.cdf_infer(params, xs[::7])
    want = orc.cdf_forward(params, xs[::7])
    assert np.max(np.abs(got - want)) <= 1e-4


def test_cdf_train_learns_a_cdf(ctx):
    """Trained on sorted prefixes with rank-fraction targets, the model's
    (oracle-evaluated) predictions land within a few buckets of 4096."""
    rng = np.random.default_rng(12)
    x = np.sort(rng.integers(0, 2 ** 64 - 1, 65536, dtype=np.uint64))
    t = ((np.arange(len(x)) + 0.5) / len(x)).astype(np.float32)
    params, loss = ctx.cdf_train(x, t, steps=300)
    assert loss < 1e-4
    y = orc.cdf_forward(params, x[::64])
    err = np.abs(y - t[::64].astype(np.float64))
    assert np.mean(err) * 4096 < 4.0


# ---------------------------------------------------------------- plan

def _orc_limits(n, ends=None, longer_first=False):
    return orc.Limits(n, ends, longer_first)


REF = capssa.Sampling.REFERENCE


@pytest.mark.parametrize("p", [2, 16, 100])
def test_plan_matches_oracle_plain(ctx, p):
    t = _dna(60000, seed=3)
    k, pv, sz = ctx.sample_sort_plan(t, capssa.ExtMemOpts(subproblem_count=p, sampling=REF))
    _, kp, opv, osz = orc.sample_sort(t, subproblem_count=p)
    assert k == kp == p
    assert pv.tolist() == opv.tolist()
    assert sz.tolist() == osz.tolist()
    assert int(sz.sum()) == len(t)


def test_plan_matches_oracle_star_and_segmented(ctx):
    rng = np.random.default_rng(4)
    t = rng.integers(0, 4, 30000).astype(np.uint8)
    ends = sorted(set(rng.integers(1, 30000, 40).tolist()) | {30000})
    # STAR (total order): pivots and sizes equal
    lp = capssa.SegmentedText(len(t), ends, capssa.BoundaryRank.LONGER_FIRST)
    k, pv, sz = ctx.sample_sort_plan(t, capssa.ExtMemOpts(subproblem_count=24, sampling=REF),
                                     lp=lp)
    _, kp, opv, osz = orc.sample_sort(t, limits=_orc_limits(len(t), ends, True),
                                      subproblem_count=24)
    assert pv.tolist() == opv.tolist() and sz.tolist() == osz.tolist()
    # ShorterFirst: tied pivots may differ, the partition sizes may not
    lp = capssa.SegmentedText(len(t), ends)
    k, pv, sz = ctx.sample_sort_plan(t, capssa.ExtMemOpts(subproblem_count=24, sampling=REF),
                                     lp=lp)
    _, kp, opv, osz = orc.sample_sort(t, limits=_orc_limits(len(t), ends), subproblem_count=24)
    assert sz.tolist() == osz.tolist()


def test_plan_matches_oracle_subset(ctx):
    rng = np.random.default_rng(5)
    t = rng.integers(0, 6, 20000).astype(np.uint8)
    pos = np.nonzero(t < 4)[0].astype(np.uint64)
    pos = np.concatenate([pos, pos[:50], [len(t)]]).astype(np.uint64)  # duplicates, empty suffix
    k, pv, sz = ctx.sample_sort_plan(t, capssa.ExtMemOpts(subproblem_count=12), positions=pos)
    _, kp, opv, osz = orc.sample_sort(t, pos, subproblem_count=12)
    assert k == kp and sz.tolist() == osz.tolist()


def test_plan_with_finite_context(ctx):
    t = _dna(20000, seed=6)
    opts = capssa.ExtMemOpts(subproblem_count=10, max_context=8)
    k, pv, sz = ctx.sample_sort_plan(t, opts)
    _, kp, opv, osz = orc.sample_sort(t, max_ctx=8, subproblem_count=10)
    assert sz.tolist() == osz.tolist()


# ---------------------------------------------------------------- partition first

def pf_sample_count(n, p):
    """The splitter sample's size: the reference sampler's count
    (src/ext_mem.rs:1282-1287), capped at n."""
    total = min(max(p * math.ceil(4 * max(math.log(n), 1.0)), p), n)
    return min(-(-total // p) * p, n)


def pf_expected_plan(t, lo, p, want_sa):
    """The partition-first plan restated with the oracle: the sample (ns
    evenly spaced midpoints of the text) in exact suffix order, pivots
    sample[(j + 1) * ns / p], and every bucket's size counted on the oracle's
    suffix array (bucket j: pivot[j-1] < s <= pivot[j], so it ends at the
    last suffix of pivot j's tie class).  Returns (pivot tie-class ends,
    sizes)."""
    n = len(t)
    ns = pf_sample_count(n, p)
    samples = ((2 * np.arange(ns, dtype=np.uint64) + 1) * n) // (2 * ns)
    ss = orc.build_in_memory(t, samples.astype(np.uint32), lo)
    piv = ss[(np.arange(1, p, dtype=np.int64) * ns) // p]
    cmp = orc.adjacent_cmp(t, want_sa, lo)
    # last SA index of every suffix's tie class
    last = np.arange(n, dtype=np.int64)
    tie = np.nonzero(cmp == 0)[0]
    for i in tie[::-1]:
        last[i] = last[i + 1]
    isa = np.empty(n, dtype=np.int64)
    isa[want_sa] = np.arange(n)
    ends = last[isa[piv.astype(np.int64)]]
    sizes = np.diff(np.concatenate([[-1], ends, [n - 1]]))
    return ends, sizes


def sizes_between(want_sa, cmp, pv):
    """Bucket sizes of the partition by pivots pv (bucket j: pivot[j-1] < s <=
    pivot[j]) counted on the oracle's suffix array (cmp: its adjacent_cmp);
    also returns each pivot's tie-class end."""
    n = len(want_sa)
    last = np.arange(n, dtype=np.int64)
    for i in np.nonzero(cmp == 0)[0][::-1]:
        last[i] = last[i + 1]
    isa = np.empty(n, dtype=np.int64)
    isa[want_sa] = np.arange(n)
    ends = last[isa[np.asarray(pv, dtype=np.int64)]]
    return np.diff(np.concatenate([[-1], ends, [n - 1]])), ends


def check_learned_pf(ctx, t, p, lp=None, lo=None):
    """The learned partition: its pivots are samples of the splitter sample
    (where the model's predicted bucket steps), in order; the emitted order is
    the oracle's; every bucket holds exactly the suffixes between its pivots;
    nearly every prediction is right at the first check."""
    n = len(t)
    lo = lo or orc.Limits(n)
    want = orc.build_in_memory(t, None, lo)
    opts = capssa.ExtMemOpts(subproblem_count=p, partition=capssa.Partition.LEARNED)
    got = ctx.build_in_memory_sample_sort(t, opts, lp=lp)
    assert np.array_equal(got, want.astype(np.uint64))
    k, pv, sz = ctx.sample_sort_plan(t, opts, lp=lp)
    st = ctx.stats()
    assert k == p
    ns = pf_sample_count(n, p)
    samples = set((((2 * np.arange(ns, dtype=np.uint64) + 1) * n) // (2 * ns)).tolist())
    assert all(int(x) in samples for x in pv)
    cmp = orc.adjacent_cmp(t, want, lo)
    sizes, ends = sizes_between(want, cmp, pv)
    assert (np.diff(ends) >= 0).all()
    assert np.array_equal(sz.astype(np.int64), sizes)
    assert st["mispredicted"] < 0.1 * n, st["mispredicted"] / n
    return st


def check_pf(ctx, t, p, lp=None, lo=None, partition=capssa.Partition.SPLITTERS, ties=False):
    n = len(t)
    lo = lo or orc.Limits(n)
    want = orc.build_in_memory(t, None, lo)
    opts = capssa.ExtMemOpts(subproblem_count=p, partition=partition)
    got = ctx.build_in_memory_sample_sort(t, opts, lp=lp)
    if ties:
        cw = orc.adjacent_cmp(t, want, lo)
        assert np.array_equal(got, orc.canonical_ties(want, cw).astype(np.uint64))
    else:
        assert np.array_equal(got, want.astype(np.uint64))
    k, pv, sz = ctx.sample_sort_plan(t, opts, lp=lp)
    st = ctx.stats()
    ends, sizes = pf_expected_plan(t, lo, p, want)
    isa = np.empty(n, dtype=np.int64)
    isa[want] = np.arange(n)
    assert k == p
    # pivots: the same suffixes, or (ShorterFirst ties) members of the same class
    last = np.arange(n, dtype=np.int64)
    cmp = orc.adjacent_cmp(t, want, lo)
    for i in np.nonzero(cmp == 0)[0][::-1]:
        last[i] = last[i + 1]
    assert np.array_equal(last[isa[pv.astype(np.int64)]], ends)
    assert np.array_equal(sz.astype(np.int64), sizes)
    return st


@pytest.mark.parametrize("p", [2, 64, 1024])
def test_partition_first_plain_bit_exact(ctx, p):
    """Buckets found before the sort by comparing every suffix with the
    pivots: the emitted order is the oracle's, the pivots are the oracle's
    sorted sample, and each bucket holds exactly the suffixes between its
    pivots."""
    st = check_pf(ctx, _dna(1 << 20, seed=30 + p), p)
    assert st["partitions"] == p and st["partition_probes"] > 0


def test_partition_first_bisection(ctx):
    """The plain binary search over all pivots (no index of their leading
    key bits) finds the same buckets with log2(p) probes per suffix."""
    t = _dna(1 << 20, seed=41)
    st = check_pf(ctx, t, 1024, partition=capssa.Partition.BISECT)
    assert st["partition_probes"] >= 9 * len(t)
    st2 = check_pf(ctx, t, 1024)
    assert st2["partition_probes"] < st["partition_probes"] / 4


def test_partition_first_learned(ctx):
    t = _dna(1 << 20, seed=40)
    st = check_learned_pf(ctx, t, 1024)
    assert st["train_samples"] > 0


def test_partition_first_learned_star_segments(ctx):
    t = _dna(300000, seed=45)
    rng = np.random.default_rng(46)
    ends = np.unique(np.concatenate([rng.integers(1, len(t), 400), [len(t)]])).astype(np.uint64)
    lp = capssa.SegmentedText(len(t), ends, capssa.BoundaryRank.LONGER_FIRST)
    check_learned_pf(ctx, t, 200, lp, orc.Limits(len(t), ends, longer_first=True))


@pytest.mark.parametrize("dtype", [np.uint16, np.uint32])
def test_partition_first_wide_symbols(ctx, dtype):
    rng = np.random.default_rng(41)
    t = rng.integers(0, 300 if dtype == np.uint16 else 70000, 200000).astype(dtype)
    t[5000:9000] = t[100:4100]  # a long repeat
    check_pf(ctx, t, 128)


def test_partition_first_star_segments(ctx):
    t = _dna(300000, seed=42)
    rng = np.random.default_rng(43)
    ends = np.unique(np.concatenate([rng.integers(1, len(t), 400), [len(t)]])).astype(np.uint64)
    lp = capssa.SegmentedText(len(t), ends, capssa.BoundaryRank.LONGER_FIRST)
    check_pf(ctx, t, 200, lp, orc.Limits(len(t), ends, longer_first=True))


def test_partition_first_shorter_first_segments(ctx):
    """ShorterFirst segments tie: the emitted order equals the oracle's after
    canonicalising each tie class (GPU classes in ascending position)."""
    rng = np.random.default_rng(44)
    t = rng.integers(0, 4, 200000).astype(np.uint8)
    ends = np.unique(np.concatenate([rng.integers(1, len(t), 3000), [len(t)]])).astype(np.uint64)
    lp = capssa.SegmentedText(len(t), ends)
    check_pf(ctx, t, 100, lp, orc.Limits(len(t), ends), ties=True)


def test_partition_first_falls_back_on_deep_ties(ctx):
    """A single-symbol text: the sample's keys all tie and its comparisons run
    past 2^16 symbols, so the sort runs first and the plan is the reference
    rule's (equal to the oracle's sample sort); the output is the same."""
    t = np.zeros(1 << 17, dtype=np.uint8)
    want = orc.build_in_memory(t).astype(np.uint64)
    opts = capssa.ExtMemOpts(subproblem_count=16)
    assert np.array_equal(ctx.build_in_memory_sample_sort(t, opts), want)
    k, pv, sz = ctx.sample_sort_plan(t, opts)
    _, kp, opv, osz = orc.sample_sort(t, subproblem_count=16)
    assert pv.tolist() == opv.tolist() and sz.tolist() == osz.tolist()


# ---------------------------------------------------------------- learned partition

def test_learned_partition_against_splitters(ctx):
    """Learned and splitter partitions of one text: both exact (bucket sizes
    counted on the oracle), the learned model's guesses almost all right at
    the first check (its pivots sit where its predicted bucket steps), the
    splitter search starting from a top-bits index of the pivot keys.
    Comparisons per suffix, misprediction rate, bucket imbalance and the
    model's training are reported."""
    t = _dna(1 << 20, seed=7)
    p = 1024
    k, pv, sz = ctx.sample_sort_plan(t, capssa.ExtMemOpts(subproblem_count=p))
    st_s = ctx.stats()
    k2, pv2, sz2 = ctx.sample_sort_plan(
        t, capssa.ExtMemOpts(subproblem_count=p, partition=capssa.Partition.LEARNED))
    st_l = ctx.stats()
    want = orc.build_in_memory(t)
    cmp = orc.adjacent_cmp(t, want, orc.Limits(len(t)))
    assert np.array_equal(sz.astype(np.int64), sizes_between(want, cmp, pv)[0])
    assert np.array_equal(sz2.astype(np.int64), sizes_between(want, cmp, pv2)[0])
    m = len(t)
    probes_s = st_s["partition_probes"] / m
    probes_l = st_l["partition_probes"] / m
    mis_rate = st_l["mispredicted"] / m
    imbalance = st_l["max_partition"] / (m / p)
    print("splitter probes/suffix %.2f, learned %.2f, mispredicted %.3f, imbalance %.2f, "
          "train %d samples in %.2f ms, loss %.2e, partition %.2f ms vs %.2f ms"
          % (probes_s, probes_l, mis_rate, imbalance, st_l["train_samples"], st_l["train_ms"],
             st_l["model_loss"], st_l["partition_ms"], st_s["partition_ms"]))
    assert probes_l < 3.0
    assert mis_rate < 0.1
    assert probes_s < 2.0
    assert st_l["train_samples"] > 0 and st_l["model_loss"] < 1e-5
    assert imbalance < 2.0


def test_learned_sample_sort_output_is_bit_exact(ctx):
    t = _dna(1 << 18, seed=8)
    want = orc.build_in_memory(t).astype(np.uint64)
    got = ctx.build_in_memory_sample_sort(
        t, capssa.ExtMemOpts(subproblem_count=64, partition=capssa.Partition.LEARNED))
    assert np.array_equal(got, want)
    st = ctx.stats()
    assert st["partitions"] == 64 and st["max_partition"] > 0
