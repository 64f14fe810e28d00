"""Pin the CPU oracle (the restated reference algorithm) against the reference's
own known-answer fixtures and brute-force test oracles.  CPU only."""
import numpy as np
import pytest

import oracle as orc
from golden.make_golden import brute as py_brute, lcg_stream, spacer_ends


def _np(text):
    return np.array(text, dtype=np.uint8)


def canon_by_ties(sa, ties):
    """Sort each tie class by position so tie order does not matter."""
    out, i = [], 0
    for r in ties:
        out.extend(sorted(int(x) for x in sa[i:i + r]))
        i += r
    return out


def test_lcp_known_answers(golden):
    for c in golden["lcp_u8"]:
        mx = orc.UNBOUNDED if c["max"] is None else c["max"]
        assert orc.lcp(_np(c["text"]), c["p"], c["q"], mx) == c["want"], c["ref"]
        assert orc.lcp_scalar(_np(c["text"]), c["p"], c["q"], mx) == c["want"], c["ref"]
    for c in golden["lcp_u16"]:
        t = np.array(c["text"], dtype=np.uint16)
        assert orc.lcp(t, c["p"], c["q"]) == c["want"], c["ref"]


def test_lcp_matches_scalar_random():
    rng = np.random.default_rng(0xA5A5)
    for dt, sigma in ((np.uint8, 4), (np.uint16, 16), (np.uint32, 32)):
        for n in (1, 8, 9, 33, 200, 1000):
            t = rng.integers(0, sigma, n).astype(dt)
            for _ in range(20):
                p, q = rng.integers(0, n, 2)
                assert orc.lcp(t, p, q) == orc.lcp_scalar(t, p, q)


def test_suffix_cmp_known_answers(golden):
    for c in golden["suffix_cmp"]:
        assert orc.suffix_cmp(_np(c["text"]), c["p"], c["q"]) == c["want"]


def test_limits_known_answers(golden):
    L = golden["limits"]
    lp = orc.Limits(L["plain_100"]["n"])
    for p, want in L["plain_100"]["lim"].items():
        assert lp.lim_at(int(p)) == want
    s = L["seg_3_5_7"]
    lp = orc.Limits(s["n"], ends=np.cumsum(s["lengths"]))
    for p, want in s["lim"].items():
        assert lp.lim_at(int(p)) == want
    s = L["single_10"]
    lp = orc.Limits(s["n"], ends=[10])
    for p, want in s["lim"].items():
        assert lp.lim_at(int(p)) == want
    with pytest.raises(ValueError):
        orc.Limits(20, ends=np.cumsum([3, 5, 7]))
    with pytest.raises(ValueError):
        orc.Limits(15, ends=[3, 3, 15])
    orc.Limits(0, ends=np.zeros(0, dtype=np.uint64))


def test_limits_directory_matches_binary_search():
    lengths = [1 + i % 97 for i in range(2000)]  # src/limits.rs:390-405
    ends = np.cumsum(lengths)
    n = int(ends[-1])
    lp = orc.Limits(n, ends=ends)
    assert lp.has_directory()
    for p in range(n + 1):
        i = int(np.searchsorted(ends, p, side="right"))
        want = int(ends[i]) - p if i < len(ends) else n - p
        assert lp.lim_at(p) == want


@pytest.mark.parametrize("index", [np.uint32, np.uint64])
def test_sa_fixtures(golden, index):
    for c in golden["sa"]:
        t = _np(c["text"])
        lp = orc.Limits(len(t), ends=c["ends"], longer_first=c["longer_first"])
        mx = orc.UNBOUNDED if c["max_ctx"] is None else c["max_ctx"]
        pos = None if c["positions"] is None else np.array(c["positions"], dtype=index)
        sa, lcp = orc.build_in_memory(t, pos, lp, mx, index=index, with_lcp=True)
        if c["ends"] is not None and not c["longer_first"]:
            assert canon_by_ties(sa, c["ties"]) == c["sa"], c["name"]
        else:
            assert sa.tolist() == c["sa"], c["name"]
        if "lcp" in c:
            assert lcp.tolist() == c["lcp"], c["name"]


def test_segmented_tie_order_is_reference_merge_tree(golden):
    """The oracle restates the mid=n/2 merge tree, so its tie order is the
    reference's: on a tie the merge outputs stream B (src/sample_sort.rs:471-476)."""
    c = next(x for x in golden["sa"] if x["name"] == "segmented_hello")
    t = _np(c["text"])
    lp = orc.Limits(len(t), ends=c["ends"])
    a = orc.build_in_memory(t, None, lp, threads=1)
    b = orc.build_in_memory(t, None, lp, threads=8)
    assert a.tolist() == b.tolist()


def test_random_texts_match_python_brute():
    rng = np.random.default_rng(0xC0FFEE)
    for sigma in (2, 4, 6, 255):
        for n in (2, 3, 7, 16, 17, 63, 64, 65, 200, 1000):
            t = rng.integers(0, sigma, n).astype(np.uint8)
            assert orc.build_in_memory(t).tolist() == py_brute(bytes(t))


def test_random_segmented_and_star():
    rng = np.random.default_rng(0x5E6)
    for _ in range(20):
        lengths = rng.integers(5, 50, rng.integers(1, 10))
        ends = np.cumsum(lengths).tolist()
        n = ends[-1]
        t = rng.integers(0, 3, n).astype(np.uint8)
        star = orc.build_in_memory(t, None, orc.Limits(n, ends, longer_first=True))
        assert star.tolist() == py_brute(bytes(t), None, ends, True)
        seg = orc.build_in_memory(t, None, orc.Limits(n, ends))
        want = py_brute(bytes(t), None, ends)
        # permutation + non-decreasing under the comparator
        assert sorted(seg.tolist()) == list(range(n))
        lp = orc.Limits(n, ends)
        for a, b in zip(seg[:-1], seg[1:]):
            assert orc.suffix_cmp(t, a, b, lp) <= 0
        assert len(want) == n


def test_finite_context_matches_comparator_sort():
    rng = np.random.default_rng(0x0F117EC7)
    for c in (0, 1, 2, 4, 16):
        for n in (2, 3, 7, 64, 500):
            t = rng.integers(0, 3, n).astype(np.uint8)
            got = orc.build_in_memory(t, max_ctx=c)
            assert got.tolist() == py_brute(bytes(t), max_ctx=c)
            assert got.tolist() == orc.brute_sa(t, max_ctx=c).tolist()


def test_sample_sort_matches_build_in_memory(golden):
    for name in ("banana", "mississippi", "abracadabra"):
        c = next(x for x in golden["sa"] if x["name"] == name)
        for p in (0, 1, 4, 16):
            out, *_ = orc.sample_sort(_np(c["text"]), subproblem_count=p)
            assert out.tolist() == c["sa"]
    rng = np.random.default_rng(0xC0DEC0DE)
    for n in (16, 200, 2000):
        for p in (1, 4, 16):
            t = rng.integers(0, 6, n).astype(np.uint8)
            out, pv, piv, sizes = orc.sample_sort(t, subproblem_count=p)
            assert out.tolist() == orc.build_in_memory(t).tolist()
            assert pv == min(p, n) and int(sizes.sum()) == n and len(piv) == pv - 1


def test_sample_sort_for_positions_subset():
    rng = np.random.default_rng(0xCA755A)
    for n in (50, 500, 2000):
        for p in (1, 3, 8):
            t = rng.integers(0, 6, n).astype(np.uint8)
            pos = np.nonzero(t < 4)[0].astype(np.uint64)
            out, *_ = orc.sample_sort(t, pos, subproblem_count=p)
            assert out.tolist() == py_brute(bytes(t), pos.tolist())


def test_pack_policy_and_width(golden):
    P = golden["pack"]
    t = np.array(P["policy_text"], dtype=np.uint8)
    assert orc.pack_params(t, 0) is None
    assert orc.pack_params(t, 1) is None
    assert orc.pack_params(t, 2, len(t) - 1) is None
    assert orc.pack_params(t, 2, len(t)) is not None
    pk = orc.pack_params(np.arange(255, dtype=np.uint8), 1)
    assert (pk["bits"], pk["k"]) == (8, 8)
    assert orc.pack_params(np.arange(256, dtype=np.uint8), 1) is None
    d = P["depth"]
    assert orc.pack_params(np.array(d["text"], dtype=np.uint8), 1)["k"] == d["k"]


def _check_seed(text, lp, positions):
    t = np.array(text, dtype=np.uint8)
    pk = orc.pack_params(t, 1)
    assert pk is not None
    sa, lcp = orc.seed_subarray(t, pk, positions, lp)
    assert sorted(sa.tolist()) == sorted(int(x) for x in positions)
    assert lcp[0] == 0
    for i in range(1, len(sa)):
        a, b = int(sa[i - 1]), int(sa[i])
        assert orc.suffix_cmp(t, a, b, lp) <= 0
        cap = min(lp.lim_at(a), lp.lim_at(b))
        assert lcp[i] == orc.lcp(t, a, b, cap)


def test_seed_subarray_lcg_fixtures(golden):
    P = golden["pack"]
    st = lcg_stream(P["lcg_plain"]["seed"])
    t = [next(st) % 4 for _ in range(P["lcg_plain"]["n"])]
    assert t[:16] == P["lcg_plain"]["text_head"]
    _check_seed(t, orc.Limits(len(t)), np.arange(len(t)))
    for key, mod, run, lf in (("lcg_segmented", 617, 9, False), ("lcg_star", 411, 7, True)):
        st = lcg_stream(P[key]["seed"])
        t = [5 if i % mod < run else next(st) % 5 for i in range(P[key]["n"])]
        ends = spacer_ends(t)
        assert ends == P[key]["ends"]
        acgt = [i for i in range(len(t)) if t[i] < 4]
        _check_seed(t, orc.Limits(len(t), ends, longer_first=lf), acgt)
    d = P["depth"]
    ends = np.cumsum(d["lengths"])
    for lf in (False, True):
        _check_seed(d["text"], orc.Limits(len(d["text"]), ends, longer_first=lf), d["starts"])


def test_merge_restatement_on_halves():
    """merge() of two LCP-annotated sorted halves equals the full sort."""
    rng = np.random.default_rng(0x1357)
    for n in (2, 5, 64, 333):
        t = rng.integers(0, 3, n).astype(np.uint8)
        pos = rng.permutation(n).astype(np.uint32)
        h = n // 2
        x, lx = orc.build_in_memory(t, pos[:h], with_lcp=True)
        y, ly = orc.build_in_memory(t, pos[h:], with_lcp=True)
        z, lz = orc.merge(t, x, lx, y, ly)
        sa, lcp = orc.build_in_memory(t, with_lcp=True)
        assert z.tolist() == sa.tolist() and lz.tolist() == lcp.tolist()


def test_cdf_oracle_gradient_matches_finite_differences():
    """The CPU restatement of the learned CDF model: its analytic gradient
    agrees with central differences of its own forward pass."""
    rng = np.random.default_rng(7)
    params = rng.normal(0, 0.3, orc.CDF_PARAMS).astype(np.float32)
    x = (rng.integers(0, 2 ** 63, 300, dtype=np.uint64) << np.uint64(1)) | np.uint64(1)
    t = rng.random(300).astype(np.float32)
    loss, g = orc.cdf_loss_grad(params, x, t)

    def f(p):
        y = orc.cdf_forward(p, x)
        return float(np.mean((y - t.astype(np.float64)) ** 2))

    assert abs(loss - f(params)) < 1e-9
    eps = 1e-3
    for i in (0, 1, 7, 64, 100, 150, 200, 256):
        pp, pm = params.copy(), params.copy()
        pp[i] += eps
        pm[i] -= eps
        num = (f(pp) - f(pm)) / (2 * eps)
        assert abs(num - g[i]) <= 1e-3 * max(1.0, abs(g[i])), (i, num, g[i])


def test_cdf_oracle_features():
    f = orc.cdf_features(0)
    assert f.tolist() == [-1.0, -1.0]
    f = orc.cdf_features(1 << 63)
    assert f.tolist() == [0.0, -1.0]


def test_adjacent_cmp_and_tie_canonicalisation():
    """The checker's vectorised tie handling (used on outputs too large for a
    per-pair loop) agrees with per-pair suffix_cmp_with calls and with
    sorting each tie class by position."""
    rng = np.random.default_rng(21)
    for _ in range(100):
        n = int(rng.integers(2, 400))
        t = rng.integers(0, 2, n).astype(np.uint8)
        ends = np.unique(np.concatenate([rng.integers(1, n, max(1, n // 4)), [n]]))
        lo = orc.Limits(n, ends.astype(np.uint64))
        sa = orc.build_in_memory(t, None, lo)
        c = orc.adjacent_cmp(t, sa, lo)
        pair = [orc.suffix_cmp(t, int(sa[i]), int(sa[i + 1]), lo) for i in range(n - 1)]
        assert c.tolist() == [(x > 0) - (x < 0) for x in pair]
        out, i = [], 0
        while i < n:
            j = i + 1
            while j < n and c[j - 1] == 0:
                j += 1
            out.extend(sorted(int(x) for x in sa[i:j]))
            i = j
        assert orc.canonical_ties(sa, c).tolist() == out
