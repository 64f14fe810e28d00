"""build_ext_mem / _for_positions / _for_filter through the C ABI against the
oracle, in the shapes of the reference's own ext-mem tests
(src/ext_mem.rs:2662-2935): every emitted stream is the suffix order,
bit-exact for PlainText."""
import numpy as np
import pytest

import oracle as orc
from golden.make_golden import brute as py_brute

pytestmark = pytest.mark.gpu

capssa = pytest.importorskip("capssa")


@pytest.fixture(scope="module")
def ctx():
    c = capssa.Context(0)
    yield c
    c.close()


def ext_sa(ctx, text, p=0, **kw):
    return ctx.build_ext_mem(text, capssa.ExtMemOpts(subproblem_count=p), **kw)


def brute_subset(text, positions):
    t = bytes(text)
    return sorted((int(p) for p in positions), key=lambda p: t[p:])


def test_ext_mem_small_fixtures(ctx):
    assert ext_sa(ctx, np.zeros(0, np.uint8), 4).tolist() == []
    for name, p in ((b"banana", 1), (b"abc", 10), (b"banana", 4), (b"mississippi", 3)):
        got = ext_sa(ctx, np.frombuffer(name, np.uint8), p)
        assert got.dtype == np.uint64
        assert got.tolist() == py_brute(name), name


def test_ext_mem_random_byte_texts(ctx):
    rng = np.random.default_rng(0xCAFE)
    for n in (16, 100, 1000, 5000):
        for p in (1, 2, 4, 16):
            t = rng.integers(0, 6, n).astype(np.uint8)
            assert ext_sa(ctx, t, p).tolist() == orc.build_in_memory(t).tolist()


def test_ext_mem_unique_terminator_and_repeats(ctx):
    rng = np.random.default_rng(0xF00D)
    for n in (10, 200, 2000):
        t = np.concatenate([rng.integers(0, 5, n), [200]]).astype(np.uint8)
        assert ext_sa(ctx, t, 3).tolist() == orc.build_in_memory(t).tolist()
    unit = np.frombuffer(b"ACGTACGTACGTACGTACGTACGTACGT", np.uint8)
    t = np.concatenate([np.tile(unit, 100), [200]]).astype(np.uint8)
    assert ext_sa(ctx, t, 8).tolist() == orc.build_in_memory(t).tolist()


def test_ext_mem_for_positions(ctx):
    t = np.frombuffer(b"mississippi", np.uint8)
    full = np.arange(len(t), dtype=np.uint64)
    assert ext_sa(ctx, t, 3, positions=full).tolist() == ext_sa(ctx, t, 3).tolist()
    half = full[::2]
    assert ext_sa(ctx, t, 4, positions=half).tolist() == brute_subset(t, half)
    rng = np.random.default_rng(0xC0DE)
    for n in (50, 500, 2000):
        t = rng.integers(0, 5, n).astype(np.uint8)
        pos = np.nonzero(rng.random(n) < 0.7)[0].astype(np.uint64)
        assert ext_sa(ctx, t, 3, positions=pos).tolist() == brute_subset(t, pos)


def test_ext_mem_for_filter(ctx):
    t = np.frombuffer(b"mississippi", np.uint8)
    assert ext_sa(ctx, t, 3, keep=(0, 256)).tolist() == ext_sa(ctx, t, 3).tolist()
    rng = np.random.default_rng(0xCA755A)
    for n in (50, 500, 2000, 200000):  # 200K: past a 64K-position block
        t = rng.integers(0, 6, n).astype(np.uint8)
        pos = np.nonzero(t < 4)[0].astype(np.uint64)
        want = ext_sa(ctx, t, 8, positions=pos)
        assert ext_sa(ctx, t, 8, keep=(0, 4)).tolist() == want.tolist()
        if n <= 2000:
            assert want.tolist() == orc.build_in_memory(t, pos).tolist()
    # sparse predicate (~5% kept)
    t = rng.integers(0, 20, 50000).astype(np.uint8)
    pos = np.nonzero(t < 1)[0].astype(np.uint64)
    got = ext_sa(ctx, t, 4, keep=(0, 1))
    assert got.tolist() == orc.build_in_memory(t, pos).tolist()
    # the kept count comes back from the call
    assert ctx.try_build_ext_mem(t, None, lambda b: None, keep=(0, 1)) == len(pos)
    with pytest.raises(TypeError):
        ctx.build_ext_mem(t, keep=lambda p: t[p] < 1)


def test_ext_mem_segmented_wide_symbols(ctx):
    """SegmentedText through ext-mem for u16 / u32 symbols: the reference's
    validity property (permutation, non-decreasing under suffix_cmp_with,
    src/sample_sort.rs:908-934) and equality with the in-memory builder."""
    rng = np.random.default_rng(41)
    for dtype, span in ((np.uint16, 3000), (np.uint32, 1 << 30)):
        lengths = rng.integers(1, 60, 80)
        ends = np.cumsum(lengths)
        n = int(ends[-1])
        t = (rng.integers(0, 3, n) * (span // 3)).astype(dtype)
        lp = capssa.SegmentedText(n, ends)
        got = ctx.build_ext_mem(t, lp=lp)
        assert sorted(got.tolist()) == list(range(n))
        lo = orc.Limits(n, ends.tolist(), False)
        for a, b in zip(got[:-1], got[1:]):
            assert orc.suffix_cmp(t, int(a), int(b), lo) <= 0
        assert got.tolist() == ctx.build_in_memory(t, lp, index=np.uint64).tolist()


def test_ext_mem_streams_several_batches(ctx):
    """More than one 4 Mi emit batch: the concatenated stream equals the
    in-memory builder's array, batches arrive in order."""
    from capssa import workloads
    t = workloads.dna_with_repeats((1 << 23) + 4321, seed=7)
    sizes, chunks = [], []

    def emit(b):
        sizes.append(len(b))
        chunks.append(b.copy())

    ctx.build_ext_mem(t, emit=emit)
    assert len(sizes) == 3 and sizes[0] == 1 << 22
    assert np.array_equal(np.concatenate(chunks), ctx.build_in_memory(t, index=np.uint64))


def test_try_ext_mem_returns_typed_emit_error(ctx):
    class Stop(Exception):
        pass

    def emit(batch):
        raise Stop()

    with pytest.raises(capssa.BuildError) as ei:
        ctx.try_build_ext_mem(np.frombuffer(b"banana", np.uint8),
                              capssa.ExtMemOpts(subproblem_count=2), emit)
    assert isinstance(ei.value.inner, Stop)
    with pytest.raises(capssa.BuildError):
        ctx.try_build_ext_mem(np.frombuffer(b"banana", np.uint8), None, emit, keep=(0, 256))
    assert ctx.build_in_memory(b"banana").tolist() == py_brute(b"banana")


def test_ext_mem_to_file_checksum_and_records(ctx, tmp_path):
    """The SA file of the CLI example, the ruSTAR checksum of the emitted
    stream, and SaLcp bucket records, all against the in-memory builder."""
    from capssa import formats
    from test_formats import py_checksum
    rng = np.random.default_rng(77)
    t = rng.integers(0, 4, 300000).astype(np.uint8)
    t[1000:9000] = t[50000:58000]
    want = ctx.build_in_memory(t, index=np.uint64)
    for width in (8, 4):
        path = tmp_path / ("sa%d.bin" % width)
        assert ctx.build_ext_mem_to_file(path, t, width=width) == len(t)
        assert np.array_equal(formats.read_sa(path, width), want)
    count, ck = ctx.ext_mem_checksum128(t, keep=(0, 3))
    kept = ctx.build_ext_mem(t, keep=(0, 3))
    assert count == len(kept) and ck == py_checksum(kept)
    for index in (np.uint32, np.uint64):
        sa, lcp = ctx.build_in_memory_lcp(t, index=index)
        rec = ctx.sa_lcp_records(sa, lcp)
        assert rec.dtype.itemsize == 2 * np.dtype(index).itemsize
        assert np.array_equal(rec["pos"], sa) and np.array_equal(rec["lcp"], lcp)
        p = tmp_path / "rec.bin"
        formats.write_sa_lcp_records(p, rec)
        back = formats.read_sa_lcp_records(p, np.dtype(index).itemsize)
        assert np.array_equal(back["pos"], sa)
