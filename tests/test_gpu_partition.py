"""GPU tests of the sample sort's partition plan and the learned CDF model.

The plan (p, pivots, partition sizes) is compared with the oracle's
restatement of build_in_memory_sample_sort (src/ext_mem.rs:1191-1428); the
learned partition must reproduce the splitter partition exactly; the model's
GPU gradients are checked against the oracle's (relative 1e-4 of the largest
component, FP32 against double accumulation)."""
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


@pytest.mark.parametrize("p", [2, 16, 100])
def test_plan_matches_oracle_plain(ctx, p):
    t = _dna(60000, seed=3)
    k, pv, sz = ctx.sample_sort_plan(t, capssa.ExtMemOpts(subproblem_count=p))
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
    k, pv, sz = ctx.sample_sort_plan(t, capssa.ExtMemOpts(subproblem_count=24), lp=lp)
    _, kp, opv, osz = orc.sample_sort(t, limits=_orc_limits(len(t), ends, True),
                                      subproblem_count=24)
    assert pv.tolist() == opv.tolist() and sz.tolist() == osz.tolist()
    # ShorterFirst: tied pivots may differ, the partition sizes may not
    lp = capssa.SegmentedText(len(t), ends)
    k, pv, sz = ctx.sample_sort_plan(t, capssa.ExtMemOpts(subproblem_count=24), lp=lp)
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


# ---------------------------------------------------------------- learned partition

def test_learned_partition_equals_splitters_and_gains(ctx):
    """The learned partition gives the splitter partition exactly, and needs
    far fewer suffix-vs-pivot comparisons than the binary search (the gain
    the model buys); misprediction rate and bucket imbalance are reported."""
    t = _dna(1 << 20, seed=7)
    p = 1024
    k, pv, sz = ctx.sample_sort_plan(t, capssa.ExtMemOpts(subproblem_count=p))
    st_s = ctx.stats()
    k2, pv2, sz2 = ctx.sample_sort_plan(
        t, capssa.ExtMemOpts(subproblem_count=p, partition=capssa.Partition.LEARNED))
    st_l = ctx.stats()
    assert pv2.tolist() == pv.tolist() and sz2.tolist() == sz.tolist()
    m = len(t)
    probes_s = st_s["partition_probes"] / m
    probes_l = st_l["partition_probes"] / m
    mis_rate = st_l["mispredicted"] / m
    imbalance = st_l["max_partition"] / (m / p)
    print("splitter probes/suffix %.2f, learned %.2f, mispredicted %.3f, imbalance %.2f, "
          "train %d samples in %.2f ms, loss %.2e, partition %.2f ms vs %.2f ms"
          % (probes_s, probes_l, mis_rate, imbalance, st_l["train_samples"], st_l["train_ms"],
             st_l["model_loss"], st_l["partition_ms"], st_s["partition_ms"]))
    # the sample's empirical CDF has noise at the scale of one bucket, so a
    # smooth model lands next to the right bucket about as often as in it:
    # the fixup is one step, against ~log2(p) steps of binary search
    assert probes_s >= 9.0
    assert probes_l < probes_s / 2
    assert mis_rate < 0.95
    assert st_l["train_samples"] > 0 and st_l["model_loss"] < 1e-5


def test_learned_sample_sort_output_is_bit_exact(ctx):
    t = _dna(1 << 18, seed=8)
    want = orc.build_in_memory(t).astype(np.uint64)
    got = ctx.build_in_memory_sample_sort(
        t, capssa.ExtMemOpts(subproblem_count=64, partition=capssa.Partition.LEARNED))
    assert np.array_equal(got, want)
    st = ctx.stats()
    assert st["partitions"] == 64 and st["max_partition"] > 0
