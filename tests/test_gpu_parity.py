"""GPU parity: every builder and primitive of the C ABI against the CPU oracle
(the restated reference algorithm) and the reference's own fixtures.

Bar: bit-exact.  Where the reference's comparator returns Equal
(SegmentedText's default boundary order) the reference leaves the relative
order unpinned (src/sample_sort.rs:908-913); there the GPU order is
ascending position and the check is equality after canonicalising each tie
class, plus the reference's validity property."""
import numpy as np
import pytest

import oracle as orc
from golden.make_golden import brute as py_brute, lcg_stream, spacer_ends

pytestmark = pytest.mark.gpu

capssa = pytest.importorskip("capssa")


@pytest.fixture(scope="module")
def ctx():
    c = capssa.Context(0)
    yield c
    c.close()


def tie_runs(text, sa, lp_orc, max_ctx=orc.UNBOUNDED):
    runs, cur = [], 1
    for i in range(1, len(sa)):
        if orc.suffix_cmp(text, int(sa[i - 1]), int(sa[i]), lp_orc, max_ctx) == 0:
            cur += 1
        else:
            runs.append(cur)
            cur = 1
    if len(sa):
        runs.append(cur)
    return runs


def canon(sa, runs):
    out, i = [], 0
    for r in runs:
        out.extend(sorted(int(x) for x in sa[i:i + r]))
        i += r
    return out


def limits_pair(n, ends=None, longer_first=False):
    b = capssa.BoundaryRank.LONGER_FIRST if longer_first else capssa.BoundaryRank.SHORTER_FIRST
    if ends is None:
        return capssa.PlainText(n, b), orc.Limits(n, None, longer_first)
    return capssa.SegmentedText(n, ends, b), orc.Limits(n, ends, longer_first)


def check_against_oracle(ctx, text, positions=None, ends=None, longer_first=False,
                         max_ctx=orc.UNBOUNDED, index=np.uint32, partition=None):
    n = len(text)
    lp, lo = limits_pair(n, ends, longer_first)
    if partition is None:
        opts = capssa.Opts(max_context=max_ctx)
    else:
        opts = capssa.ExtMemOpts(max_context=max_ctx, partition=partition)
    if positions is None:
        got = ctx.build_in_memory(text, lp, opts, index=index)
        want = orc.build_in_memory(text, None, lo, max_ctx, index=index)
    else:
        pos = np.asarray(positions, dtype=index)
        got = ctx.build_in_memory_for_positions(text, pos, lp, opts)
        want = orc.build_in_memory(text, pos, lo, max_ctx, index=index)
    assert got.dtype == np.dtype(index)
    if ends is not None and not longer_first:
        runs = tie_runs(text, want, lo, max_ctx)
        assert canon(got, runs) == canon(want, runs)
        # GPU tie classes come out in ascending position
        assert got.tolist() == canon(got, runs)
    else:
        assert got.tolist() == want.tolist()
    return got


# ---------------------------------------------------------------- fixtures

@pytest.mark.parametrize("index", [np.uint32, np.uint64])
def test_reference_fixtures(ctx, golden, index):
    for c in golden["sa"]:
        t = np.array(c["text"], dtype=np.uint8)
        lp, _ = limits_pair(len(t), c["ends"], c["longer_first"])
        mx = orc.UNBOUNDED if c["max_ctx"] is None else c["max_ctx"]
        opts = capssa.Opts(max_context=mx)
        if c["positions"] is None:
            got = ctx.build_in_memory(t, lp, opts, index=index)
        else:
            got = ctx.build_in_memory_for_positions(t, np.array(c["positions"], dtype=index), lp,
                                                    opts)
        if c["ends"] is not None and not c["longer_first"]:
            assert canon(got, c["ties"]) == c["sa"], c["name"]
        else:
            assert got.tolist() == c["sa"], c["name"]
        if "lcp" in c:
            sa, lcp = ctx.build_in_memory_lcp(t, None, lp, opts, index=index)
            assert lcp.tolist() == c["lcp"], c["name"]


def test_star_literal(ctx):
    lp = capssa.SegmentedText(4, [4], capssa.BoundaryRank.LONGER_FIRST)
    assert ctx.build_in_memory(b"AAAA", lp).tolist() == [0, 1, 2, 3]  # src/sample_sort.rs:1059-1070


def test_empty_and_single(ctx):
    assert ctx.build_in_memory(np.zeros(0, dtype=np.uint8)).tolist() == []
    assert ctx.build_in_memory(np.array([7], dtype=np.uint8)).tolist() == [0]
    assert ctx.build_in_memory_for_positions(b"banana", np.zeros(0, np.uint32)).tolist() == []


# ---------------------------------------------------------------- random vs oracle

@pytest.mark.parametrize("dtype,sigma", [(np.uint8, 2), (np.uint8, 4), (np.uint8, 6),
                                         (np.uint8, 16), (np.uint8, 100), (np.uint8, 255),
                                         (np.uint16, 16), (np.uint16, 4000),
                                         (np.uint32, 32), (np.uint32, 1 << 31)])
def test_random_plain(ctx, dtype, sigma):
    rng = np.random.default_rng(0xC0FFEE + sigma)
    for n in (1, 2, 3, 7, 16, 17, 63, 64, 65, 200, 1000, 5000):
        t = rng.integers(0, sigma, n, dtype=np.uint64).astype(dtype)
        check_against_oracle(ctx, t)


@pytest.mark.parametrize("sigma,geometry", [(2, (24, 1, 8)), (16, (8, 4, 8)), (200, (6, 8, 12))])
def test_flagless_keys_other_symbol_widths(ctx, sigma, geometry):
    """Plain texts of 2^21 + 37 symbols over 2, 16 and 200 symbols.  Codes of
    1 and 4 bits take the flagless geometry with whole radix digits (24 and 8
    symbols, 8-byte records), so the key kernel that counts one digit
    histogram and shifts it for the other passes runs for widths other than
    DNA's; 8-bit codes take 6 symbols and a length field (12-byte records).
    A long run and a periodic stretch give deep groups.  Bit-exact with the
    oracle."""
    rng = np.random.default_rng(0xF1A6 + sigma)
    t = rng.integers(0, sigma, (1 << 21) + 37).astype(np.uint8)
    t[5000:25000] = 1
    t[100000:130000] = np.tile(np.array([0, sigma - 1], dtype=np.uint8), 15000)
    got = ctx.build_in_memory(t)
    st = ctx.stats()
    assert (st["key_symbols"], st["key_bits_per_symbol"], st["sort_item_bytes"]) == geometry
    assert np.array_equal(got, orc.build_in_memory(t))


def test_long_runs_and_periodic(ctx):
    check_against_oracle(ctx, np.full(20000, 7, dtype=np.uint8))
    check_against_oracle(ctx, (np.arange(30000) % 3).astype(np.uint8))
    mixed = np.concatenate([np.arange(500) % 4, np.full(15000, 4), np.arange(500) % 4])
    check_against_oracle(ctx, mixed.astype(np.uint8))
    # repeat with a unique terminator, many copies of one unit
    unit = np.frombuffer(b"ACGTACGTACGTACGTACGTACGTACGT", dtype=np.uint8)
    check_against_oracle(ctx, np.concatenate([np.tile(unit, 500), [200]]).astype(np.uint8))


@pytest.mark.parametrize("copies,unit", [(3, 9000), (40, 3000), (2500, 40), (5000, 3)])
def test_repeat_structures(ctx, copies, unit):
    """Tied groups of every kind: few members with LCPs past the direct
    comparison depth (rank doubling), medium groups (block sort), and
    groups of thousands (radix path)."""
    rng = np.random.default_rng(copies)
    u = rng.integers(0, 4, unit).astype(np.uint8)
    parts = []
    for _ in range(copies):
        parts.append(u)
        parts.append(rng.integers(0, 4, int(rng.integers(1, 50))).astype(np.uint8))
    t = np.concatenate(parts)
    check_against_oracle(ctx, t)
    ends = np.cumsum([len(x) for x in parts])
    check_against_oracle(ctx, t, ends=ends)
    check_against_oracle(ctx, t, ends=ends, longer_first=True)


@pytest.mark.parametrize("index", [np.uint32, np.uint64])
def test_random_segmented_and_star(ctx, index):
    rng = np.random.default_rng(0x5E6)
    for trial in range(30):
        lengths = rng.integers(1 if trial % 3 == 0 else 5, 50, rng.integers(1, 40))
        ends = np.cumsum(lengths)
        n = int(ends[-1])
        t = rng.integers(0, 3, n).astype(np.uint8)
        check_against_oracle(ctx, t, ends=ends, index=index)
        check_against_oracle(ctx, t, ends=ends, longer_first=True, index=index)
        keep = np.nonzero(rng.random(n) < 0.7)[0]
        check_against_oracle(ctx, t, positions=keep, ends=ends, index=index)
        check_against_oracle(ctx, t, positions=keep, ends=ends, longer_first=True, index=index)


def test_segmented_many_segments_uses_directory(ctx):
    rng = np.random.default_rng(77)
    lengths = 1 + (np.arange(3000) % 97)  # >= 256 segments: boundary directory
    ends = np.cumsum(lengths)
    n = int(ends[-1])
    t = rng.integers(0, 4, n).astype(np.uint8)
    check_against_oracle(ctx, t, ends=ends)
    check_against_oracle(ctx, t, ends=ends, longer_first=True)


@pytest.mark.parametrize("max_ctx", [0, 1, 2, 4, 16, 100])
def test_finite_context(ctx, max_ctx):
    rng = np.random.default_rng(0x0F117EC7)
    for n in (2, 3, 7, 64, 500, 3000):
        t = rng.integers(0, 3, n).astype(np.uint8)
        check_against_oracle(ctx, t, max_ctx=max_ctx)
        lengths = rng.integers(3, 40, 200)
        ends = np.cumsum(lengths)
        ends = ends[ends < n].tolist() + [n]
        check_against_oracle(ctx, t, ends=ends, max_ctx=max_ctx)
        check_against_oracle(ctx, t, ends=ends, longer_first=True, max_ctx=max_ctx)


def test_for_positions_subsets_duplicates_and_end(ctx):
    rng = np.random.default_rng(0xFEED)
    for n in (33, 200, 1000):
        t = rng.integers(0, 6, n).astype(np.uint8)
        keep = np.nonzero(rng.integers(0, 10, n) < 7)[0]
        check_against_oracle(ctx, t, positions=rng.permutation(keep))
        # duplicates and the empty suffix at n
        pos = np.concatenate([keep[:10], keep[:10], [n, n]]).astype(np.uint64)
        got = ctx.build_in_memory_for_positions(t, pos)
        want = orc.build_in_memory(t, pos, index=np.uint64)
        assert sorted(got.tolist()) == sorted(want.tolist())
        runs = tie_runs(t, want, orc.Limits(n))
        assert canon(got, runs) == canon(want, runs)
        # distinct positions with the empty suffix once (bitmap path), both
        # boundary orders, u32 and u64
        pos1 = rng.permutation(np.concatenate([keep, [n]]))
        for lf in (False, True):
            for index in (np.uint32, np.uint64):
                check_against_oracle(ctx, t, positions=pos1, longer_first=lf, index=index)
    with pytest.raises(ValueError):
        ctx.build_in_memory_for_positions(b"banana", np.array([0, 7], dtype=np.uint32))
    with pytest.raises(ValueError):  # beyond the end, among distinct positions
        ctx.build_in_memory_for_positions(np.zeros(5000, np.uint8) + 1,
                                          np.arange(0, 5002, dtype=np.uint64))


def test_invalid_segments_rejected(ctx):
    with pytest.raises(ValueError):
        capssa.SegmentedText.from_lengths(20, [3, 5, 7])
    bad = capssa.SegmentedText.__new__(capssa.SegmentedText)
    bad.n, bad.ends, bad.boundary = 15, np.array([3, 3, 15], np.uint64), 0
    with pytest.raises(ValueError):
        ctx.build_in_memory(np.zeros(15, np.uint8), bad)


# ---------------------------------------------------------------- primitives

def test_lcp_known_answers(ctx, golden):
    for c in golden["lcp_u8"]:
        t = np.array(c["text"], dtype=np.uint8)
        mx = orc.UNBOUNDED if c["max"] is None else c["max"]
        assert int(ctx.lcp(t, c["p"], c["q"], mx)[0]) == c["want"], c["ref"]
    for c in golden["lcp_u16"]:
        t = np.array(c["text"], dtype=np.uint16)
        assert int(ctx.lcp(t, c["p"], c["q"])[0]) == c["want"], c["ref"]


@pytest.mark.parametrize("dtype,sigma", [(np.uint8, 4), (np.uint16, 16), (np.uint32, 32)])
def test_lcp_and_cmp_random_pairs(ctx, dtype, sigma):
    rng = np.random.default_rng(0x2468)
    for n in (1, 8, 9, 100, 2000):
        t = rng.integers(0, sigma, n).astype(dtype)
        # long equal stretches make multi-step warp compares happen
        if n > 100:
            t[n // 2: n // 2 + 900] = t[: min(900, n - n // 2)][: len(t[n // 2: n // 2 + 900])]
        p = rng.integers(0, n + 1, 300)
        q = rng.integers(0, n + 1, 300)
        for mx in (orc.UNBOUNDED, 5):
            got = ctx.lcp(t, p, q, mx)
            want = [orc.lcp(t, a, b, mx) for a, b in zip(p, q)]
            assert got.tolist() == want
        ends = np.unique(np.concatenate([rng.integers(1, n + 1, 5), [n]]))
        lp, lo = limits_pair(n, ends)
        pp, qq = p[p < n], q[: len(p[p < n])]
        qq = np.minimum(qq, n - 1)
        got = ctx.suffix_cmp(t, pp, qq, lp)
        want = [orc.suffix_cmp(t, a, b, lo) for a, b in zip(pp, qq)]
        assert got.tolist() == want


def _runs_with_lcp(t, pos, lo, index):
    sa, lcp = orc.build_in_memory(t, np.asarray(pos, dtype=index), lo, with_lcp=True, index=index)
    return sa, lcp


@pytest.mark.parametrize("index", [np.uint32, np.uint64])
def test_merge_matches_reference_merge(ctx, index):
    """The merge-path kernel reproduces sample_sort::merge exactly, including
    the reference's alternating order on comparator ties."""
    rng = np.random.default_rng(0x1CB0)
    for trial in range(12):
        n = int(rng.integers(2, 3000))
        t = rng.integers(0, 3, n).astype(np.uint8)
        if trial % 2:
            lengths = rng.integers(2, 12, n)
            ends = np.cumsum(lengths)
            ends = ends[ends < n].tolist() + [n]
        else:
            ends = None
        lp, lo = limits_pair(n, ends, longer_first=(trial % 4 == 3))
        perm = rng.permutation(n)
        h = int(rng.integers(0, n + 1))
        x, lx = _runs_with_lcp(t, perm[:h], lo, index)
        y, ly = _runs_with_lcp(t, perm[h:], lo, index)
        z, lz = ctx.merge(t, x, lx, y, ly, lp)
        wz, wlz = orc.merge(t, x, lx, y, ly, lo)
        assert z.tolist() == wz.tolist(), trial
        assert lz.tolist() == wlz.tolist(), trial


# ---------------------------------------------------------------- sample sort

def test_sample_sort_matches_build_in_memory(ctx):
    rng = np.random.default_rng(0xC0DEC0DE)
    for n in (16, 200, 2000, 100000):
        t = rng.integers(0, 6, n).astype(np.uint8)
        for p in (0, 1, 4, 16):
            got = ctx.build_in_memory_sample_sort(t, capssa.ExtMemOpts(subproblem_count=p))
            assert got.dtype == np.uint64
            assert got.tolist() == orc.build_in_memory(t).tolist()
    for name in (b"banana", b"mississippi", b"abracadabra"):
        got = ctx.build_in_memory_sample_sort(np.frombuffer(name, np.uint8))
        assert got.tolist() == py_brute(name)


def test_sample_sort_for_positions_subset(ctx):
    rng = np.random.default_rng(0xCA755A)
    for n in (50, 500, 2000):
        t = rng.integers(0, 6, n).astype(np.uint8)
        pos = np.nonzero(t < 4)[0].astype(np.uint64)
        got = ctx.build_in_memory_sample_sort(t, capssa.ExtMemOpts(subproblem_count=3),
                                              positions=pos)
        want, *_ = orc.sample_sort(t, pos, subproblem_count=3)
        assert got.tolist() == want.tolist()


def test_sample_sort_emit_abort(ctx):
    """try_build_ext_mem_returns_typed_emit_error shape (src/ext_mem.rs:2894-2915)."""
    class Stop(Exception):
        pass

    seen = []

    def emit(batch):
        seen.append(len(batch))
        raise Stop()

    with pytest.raises(capssa.BuildError) as ei:
        ctx.try_build_in_memory_sample_sort(np.frombuffer(b"banana", np.uint8),
                                            capssa.ExtMemOpts(subproblem_count=2), emit)
    assert isinstance(ei.value.inner, Stop)
    assert seen == [6]
    # the context stays usable
    assert ctx.build_in_memory(b"banana").tolist() == py_brute(b"banana")


# ---------------------------------------------------------------- batched

@pytest.mark.parametrize("index", [np.uint32, np.uint64])
def test_batched_matches_per_text(ctx, index):
    rng = np.random.default_rng(5)
    lens = rng.integers(0, 3000, 40)
    lens[3] = 0
    texts = [rng.integers(0, 4, L).astype(np.uint8) for L in lens]
    for i in range(0, 40, 7):  # plant repeats across texts
        if lens[i] > 100 and lens[i + 1] > 100:
            texts[i + 1][:100] = texts[i][:100]
    cat = np.concatenate(texts)
    offs = np.concatenate([[0], np.cumsum(lens)]).astype(np.uint64)
    got = ctx.build_batched(cat, offs, index=index)
    for i, tx in enumerate(texts):
        assert got[offs[i]:offs[i + 1]].tolist() == orc.build_in_memory(tx).tolist(), i


@pytest.mark.parametrize("dtype,span", [(np.uint8, 256), (np.uint16, 40000),
                                        (np.uint32, 1 << 31)])
def test_batched_many_small_texts(ctx, dtype, span):
    # thousands of texts of 0..6 symbols (empty and one-symbol texts among
    # them), equal texts repeated, wide alphabets
    rng = np.random.default_rng(11)
    lens = rng.integers(0, 7, 3000)
    texts = [rng.integers(0, 3, L).astype(dtype) * (span // 3) for L in lens]
    for i in range(0, 3000, 5):
        texts[i] = texts[0].copy()
        lens[i] = len(texts[0])
    cat = np.concatenate(texts).astype(dtype)
    offs = np.concatenate([[0], np.cumsum(lens)]).astype(np.uint64)
    got = ctx.build_batched(cat, offs, index=np.uint64)
    for i, tx in enumerate(texts):
        assert got[offs[i]:offs[i + 1]].tolist() == orc.build_in_memory(tx).tolist(), i


def test_batched_device_output_and_long_texts(ctx):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(12)
    lens = np.array([70000, 1, 0, 120000, 3, 90000])
    texts = [rng.integers(0, 2, L).astype(np.uint8) for L in lens]
    texts[3][50000:90000] = texts[0][10000:50000]  # a long repeat across texts
    cat = np.concatenate(texts)
    offs = np.concatenate([[0], np.cumsum(lens)]).astype(np.uint64)
    out = torch.empty(int(offs[-1]), dtype=torch.int32, device="cuda")
    ctx.build_batched(cat, offs, index=np.uint32, out=out)
    got = out.cpu().numpy().view(np.uint32)
    for i, tx in enumerate(texts):
        assert np.array_equal(got[offs[i]:offs[i + 1]], orc.build_in_memory(tx)), i


# ---------------------------------------------------------------- packed keys

def test_pack_params_and_keys(ctx, golden):
    P = golden["pack"]
    t = np.array(P["policy_text"], dtype=np.uint8)
    assert ctx.pack_params(t, 0) is None
    assert ctx.pack_params(t, 1) is None
    assert ctx.pack_params(t, 2, len(t) - 1) is None
    assert ctx.pack_params(t, 2, len(t)) is not None
    pk = ctx.pack_params(np.arange(255, dtype=np.uint8), 1)
    assert (pk["bits"], pk["k"]) == (8, 8)
    assert ctx.pack_params(np.arange(256, dtype=np.uint8), 1) is None
    for key, mod, run, lf in (("lcg_segmented", 617, 9, False), ("lcg_star", 411, 7, True)):
        st = lcg_stream(P[key]["seed"])
        tx = np.array([5 if i % mod < run else next(st) % 5 for i in range(P[key]["n"])],
                      dtype=np.uint8)
        ends = spacer_ends(tx.tolist())
        lp, lo = limits_pair(len(tx), ends, lf)
        gp = ctx.pack_params(tx, 1)
        op = orc.pack_params(tx, 1)
        assert (gp["bits"], gp["k"], gp["alphabet"]) == (op["bits"], op["k"], op["alphabet"])
        pos = np.nonzero(tx < 4)[0]
        assert ctx.pack_keys(tx, gp, pos, lp).tolist() == orc.pack_keys(tx, op, pos, lo).tolist()
        sa, lcp = ctx.seed_subarray(tx, gp, pos, lp)
        osa, olcp = orc.seed_subarray(tx, op, pos, lo)
        if lf:
            assert sa.tolist() == osa.tolist()
        else:
            runs = tie_runs(tx, osa, lo)
            assert canon(sa, runs) == canon(osa, runs)
        assert lcp.tolist() == olcp.tolist() or not lf and lcp[0] == 0


# ---------------------------------------------------------------- workload-shaped

def test_config1_uniform_dna_bit_exact(ctx):
    """n = 2^20 i.i.d. uniform {0,1,2,3}, u32: bit-exact against the oracle."""
    from capssa import workloads
    t = workloads.uniform_dna(1 << 20, seed=1)
    got = ctx.build_in_memory(t)
    want = orc.build_in_memory(t)
    assert np.array_equal(got, want)


def test_repeat_text_bit_exact(ctx):
    from capssa import workloads
    t = workloads.dna_with_repeats(1 << 19, seed=2)
    assert np.array_equal(ctx.build_in_memory(t), orc.build_in_memory(t))


def _runs_text(n, seed):
    """Repeat DNA with one 60,000-symbol run and one periodic stretch."""
    from capssa import workloads
    t = workloads.dna_with_repeats(n, seed=seed).copy()
    t[1000:61000] = 0
    t[200000:230000] = np.tile(np.array([1, 3, 2], dtype=t.dtype), 10000)
    return t


@pytest.mark.parametrize("dtype", [np.uint8, np.uint32])
def test_large_text_runs_and_period(ctx, dtype):
    """2^22+ symbols with a 60,000-symbol run and a 90,000-symbol periodic
    stretch (large tied groups, deep rank doubling): bit-exact."""
    t = _runs_text((1 << 22) + 12345, seed=11).astype(dtype)
    got = ctx.build_in_memory(t)
    assert np.array_equal(got, orc.build_in_memory(t))


def test_rank_build_by_window_2p25(ctx):
    """Past 2^24 symbols the position-ordered ranks that rank doubling reads
    are built window by window (2^21 positions each, the last one partial):
    a 2^25+ text whose run and periodic stretch need rank doubling, bit-exact
    with and without segments."""
    t = _runs_text((1 << 25) + 4321, seed=14).astype(np.uint8)
    got = ctx.build_in_memory(t)
    assert ctx.stats()["refine_rounds"] > 5
    assert np.array_equal(got, orc.build_in_memory(t))
    rng = np.random.default_rng(6)
    ends = np.unique(np.concatenate([rng.integers(1, len(t), 200), [len(t)]])).tolist()
    lp, lo = limits_pair(len(t), ends, True)  # LongerFirst: a total order
    got = ctx.build_in_memory(t, lp)
    assert np.array_equal(got, orc.build_in_memory(t, None, lo))


def _runs_of_each_symbol(n, seed):
    """Random DNA with dozens of long runs of every symbol, some reaching a
    segment end, so that deep tied groups consist of run suffixes whose runs
    end in a smaller symbol, a larger one, or the end of the suffix."""
    rng = np.random.default_rng(seed)
    t = rng.integers(0, 4, n).astype(np.uint8)
    ends = np.unique(np.concatenate([rng.integers(1, n, 300), [n]]))
    for c in range(4):
        for _ in range(40):
            L = int(rng.integers(300, 3000))
            if rng.random() < 0.3:  # up to a segment end
                e = int(ends[rng.integers(0, len(ends))])
                a = max(0, e - L)
            else:
                a = int(rng.integers(0, n - L))
            t[a:a + L] = c
    return t, ends


def test_runs_of_one_symbol_deep_groups(ctx):
    """Groups of thousands of run suffixes tied far past the key: ordered by
    their run lengths and what ends each run.  PlainText and SegmentedText,
    bit-exact (the segmented case in the reference's tie order)."""
    t, ends = _runs_of_each_symbol(1 << 20, seed=21)
    got = ctx.build_in_memory(t)
    assert ctx.stats()["refine_rounds"] >= 3
    assert np.array_equal(got, orc.build_in_memory(t))
    lp, lo = limits_pair(len(t), ends)
    got = ctx.build_in_memory(t, lp, capssa.Opts(tie_order=capssa.TieOrder.REFERENCE))
    assert np.array_equal(got, orc.build_in_memory(t, None, lo))


def test_large_text_star_segments(ctx):
    t = _runs_text((1 << 22) + 777, seed=12).astype(np.uint8)
    rng = np.random.default_rng(5)
    ends = np.unique(np.concatenate([rng.integers(1, len(t), 300), [len(t)]])).tolist()
    check_against_oracle(ctx, t, ends=ends, longer_first=True)


def test_large_text_wide_alphabet(ctx):
    """A 5-bit alphabet (key of 11 symbols + length field) with a long run."""
    rng = np.random.default_rng(13)
    t = rng.integers(0, 20, (1 << 22) + 99).astype(np.uint8)
    t[5000:25000] = 7
    check_against_oracle(ctx, t)


def test_bounded_wait_times_out_and_context_survives(ctx):
    """Failure detection without a GPU fault: a device wait that nothing
    satisfies gives up after its poll limit, the call reports ETIMEOUT, and
    the same context keeps working."""
    with pytest.raises(capssa.CapsSaError) as ei:
        ctx.selftest_bounded_wait(4096)
    assert ei.value.status == capssa.Status.ETIMEOUT
    t = np.frombuffer(b"mississippi", np.uint8)
    assert ctx.build_in_memory(t).tolist() == py_brute(b"mississippi")


@pytest.mark.parametrize("index", [np.uint32, np.uint64])
def test_filter_source_matches_positions(ctx, index):
    """build_ext_mem_for_filter's position source on the GPU: the positions
    with lo <= text[p] < hi, sorted exactly like the same positions passed to
    build_in_memory_for_positions (segmented, ShorterFirst: canonical ties)."""
    rng = np.random.default_rng(31)
    from capssa import workloads
    t, ends, pos = workloads.segmented_filtered(300000, seed=9, run_max=5000, run_min=500)
    got = ctx.build_in_memory_for_filter(t, 0, 4, lp=capssa.SegmentedText(len(t), ends),
                                         index=index)
    want = ctx.build_in_memory_for_positions(t, pos.astype(index),
                                             capssa.SegmentedText(len(t), ends))
    assert got.dtype == np.dtype(index) and np.array_equal(got, want)
    # plain text, u16 symbols, a middle range; bit-exact against the oracle
    t2 = rng.integers(0, 700, 50000).astype(np.uint16)
    got2 = ctx.build_in_memory_for_filter(t2, 100, 400, index=index)
    keep = np.nonzero((t2 >= 100) & (t2 < 400))[0].astype(index)
    assert np.array_equal(got2, orc.build_in_memory(t2, keep, index=index))
    # nothing kept
    assert len(ctx.build_in_memory_for_filter(t2, 900, 1000, index=index)) == 0


def test_radix_autotuner_picks_a_shape_and_keeps_it():
    """The context's autotuner times the candidate tile shapes on its first
    large sort and reuses the choice; the output stays bit-exact."""
    from capssa import workloads
    c = capssa.Context(0)
    try:
        t = workloads.dna_with_repeats((1 << 22) + 5, seed=21)
        want = orc.build_in_memory(t)
        got1 = c.build_in_memory(t)
        s1 = c.stats()["radix_items"]
        got2 = c.build_in_memory(t)
        s2 = c.stats()["radix_items"]
        assert np.array_equal(got1, want) and np.array_equal(got2, want)
        assert s1 in (16, 20, 24) and s1 == s2
    finally:
        c.close()


@pytest.mark.parametrize("dtype", [np.uint8, np.uint16])
def test_flagless_short_suffix_placement(ctx, dtype):
    """n = 150,000 over 4 symbols: dropping the early-end flag saves a radix
    pass (12-symbol keys, 3 passes), so the 11 suffixes that end inside the
    key are placed after the sort.  Endings that tie them with many full
    suffixes (long runs of the smallest and largest code, a period-2 tail,
    an all-equal text) must still give the oracle's order."""
    rng = np.random.default_rng(150)
    n = 150000
    base = rng.integers(0, 4, n)
    endings = {
        "random": base,
        "zeros": np.concatenate([base[:n - 5000], np.zeros(5000, np.int64)]),
        "threes": np.concatenate([base[:n - 3000], np.full(3000, 3)]),
        "period2": np.concatenate([base[:n - 4000], np.tile([0, 1], 2000)]),
        "zero_then_one": np.concatenate([base[:n - 41], np.zeros(40, np.int64), [1]]),
        "all_equal": np.concatenate([np.zeros(n - 3, np.int64), [1, 2, 3]]),
    }
    for name, t in endings.items():
        t = t.astype(dtype)
        got = ctx.build_in_memory(t)
        st = ctx.stats()
        assert st["key_symbols"] == 12 and st["sort_passes"] <= 3, name
        assert np.array_equal(got, orc.build_in_memory(t)), name
    # LongerFirst keeps the flag (and its own order)
    t = endings["zeros"].astype(dtype)
    check_against_oracle(ctx, t, longer_first=True)


def test_flagless_with_context_bound_and_lcp(ctx):
    """Flagless keys (n = 150,000 over 4 symbols) combined with a finite
    max_context, a LongerFirst subset, and the LCP output."""
    rng = np.random.default_rng(151)
    n = 150000
    t = rng.integers(0, 4, n).astype(np.uint8)
    t[20000:26000] = t[60000:66000]      # a long repeat
    t[n - 3000:] = 0                     # a run at the end
    for max_ctx in (5, 40):
        check_against_oracle(ctx, t, max_ctx=max_ctx)
    sa, lcp = ctx.build_in_memory_lcp(t, index=np.uint64)
    want = orc.build_in_memory(t, index=np.uint64)
    assert np.array_equal(sa, want)
    assert lcp[0] == 0
    assert np.array_equal(lcp[1:], ctx.lcp(t, sa[:-1], sa[1:]))
    keep = np.nonzero(rng.random(n) < 0.5)[0]
    check_against_oracle(ctx, t, positions=keep, index=np.uint64)


# ---------------------------------------------------------------- subsets sorted on their own

def _subset(rng, n, m, with_empty=False):
    pos = rng.choice(n, size=m, replace=False).astype(np.uint64)
    if with_empty:
        pos = np.concatenate([pos, [n]]).astype(np.uint64)
    return pos


@pytest.mark.parametrize("index", [np.uint32, np.uint64])
def test_small_subset_sorted_alone_bit_exact(ctx, index):
    """m <= n / 8 distinct positions: only those suffixes are sorted (O(m)
    records), bit-exact against the oracle, the empty suffix included."""
    from capssa import workloads
    t = workloads.dna_with_repeats(1 << 21, seed=61)
    rng = np.random.default_rng(62)
    pos = _subset(rng, len(t), 1 << 15, with_empty=True).astype(index)
    got = ctx.build_in_memory_for_positions(t, pos)
    assert ctx.stats()["sparse_subset"] == 1
    want = orc.build_in_memory(t, pos, index=index)
    assert np.array_equal(got, want)
    # inside repeats: positions clustered in copies and their sources
    pos2 = np.unique(np.concatenate([np.arange(5000, 9000), np.arange(700000, 720000)]))
    got2 = ctx.build_in_memory_for_positions(t, pos2.astype(index))
    assert ctx.stats()["sparse_subset"] == 1
    assert np.array_equal(got2, orc.build_in_memory(t, pos2.astype(index), index=index))


def test_small_subset_segments_both_orders(ctx):
    rng = np.random.default_rng(63)
    t = rng.integers(0, 4, 300000).astype(np.uint8)
    ends = np.unique(np.concatenate([rng.integers(1, len(t), 2000), [len(t)]]))
    pos = _subset(rng, len(t), 30000, with_empty=True)
    check_against_oracle(ctx, t, positions=pos, ends=ends.tolist(), longer_first=True,
                         index=np.uint64)
    assert ctx.stats()["sparse_subset"] == 1
    check_against_oracle(ctx, t, positions=pos, ends=ends.tolist(), index=np.uint64)
    assert ctx.stats()["sparse_subset"] == 1


def test_small_subset_falls_back_when_needed(ctx):
    """Repeated positions, and suffixes inside a 100,000-symbol run (ties
    deeper than the direct comparisons reach), take the whole-text path:
    same output."""
    rng = np.random.default_rng(64)
    t = rng.integers(0, 4, 1 << 21).astype(np.uint8)
    pos = _subset(rng, len(t), 1000)
    dup = np.concatenate([pos, pos[:10]]).astype(np.uint64)
    got = ctx.build_in_memory_for_positions(t, dup)
    assert ctx.stats()["sparse_subset"] == 0
    assert np.array_equal(got, orc.build_in_memory(t, dup, index=np.uint64))
    t2 = t.copy()
    t2[100000:200000] = 1
    deep = np.arange(100000, 120000, dtype=np.uint64)
    got = ctx.build_in_memory_for_positions(t2, deep)
    assert ctx.stats()["sparse_subset"] == 0
    assert np.array_equal(got, orc.build_in_memory(t2, deep, index=np.uint64))
