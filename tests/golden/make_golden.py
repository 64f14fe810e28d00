"""Write tests/golden/fixtures.json: the known-answer fixtures of caps-sa's own
unit tests for the in-memory suffix-array path, with expected outputs.

Two kinds of expected values are recorded:

* literal answers that appear in the reference's test source (LCP tables,
  lim_at tables, STAR "AAAA" -> [0,1,2,3], packer bits/k, policy outcomes),
  copied here as data with the file:line they come from;
* suffix arrays for the reference's fixed fixture texts, computed by this
  script with a pure-Python comparator sort.  That comparator is a direct
  restatement of the reference's own test oracles (brute_force_sa,
  segmented_cmp and star_brute_force_sa in src/sample_sort.rs:643-647,
  895-906, 1021-1040, and suffix_cmp_with in src/lcp.rs:184-201), written
  independently of the C oracle so that the C oracle can be checked
  against it.

Tie order: under SegmentedText's default boundary order two suffixes can
compare Equal.  The reference leaves their relative order unpinned
(src/sample_sort.rs:908-913); this script records ascending-position order
and also the tie classes, so tests can check class-by-class equality.

Run:  python tests/golden/make_golden.py   (deterministic; no RNG beyond
the reference's own LCG fixtures, src/pack.rs:353-358)
"""
from __future__ import annotations

import functools
import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))
UNB = None  # unbounded max_context


def lim_at(n, ends, p):
    """PlainText / SegmentedText::lim_at without the directory."""
    if ends is None:
        return n - p
    for e in ends:
        if e > p:
            return e - p
    return n - p


def make_cmp(text, ends=None, longer_first=False, max_ctx=UNB):
    n = len(text)

    def cmp(a, b):
        la, lb = lim_at(n, ends, a), lim_at(n, ends, b)
        lim = min(la, lb)
        if max_ctx is not None:
            lim = min(lim, max_ctx)
        ca, cb = text[a:a + lim], text[b:b + lim]
        if ca != cb:
            return -1 if ca < cb else 1
        if longer_first:
            if la != lb:
                return -1 if lb < la else 1
            return (a > b) - (a < b)
        return (la > lb) - (la < lb)

    return cmp


def brute(text, positions=None, ends=None, longer_first=False, max_ctx=UNB):
    cmp = make_cmp(text, ends, longer_first, max_ctx)
    pos = list(range(len(text))) if positions is None else list(positions)

    def key(a, b):
        c = cmp(a, b)
        return c if c != 0 else (a > b) - (a < b)

    return sorted(pos, key=functools.cmp_to_key(key))


def tie_classes(text, sa, ends=None, longer_first=False, max_ctx=UNB):
    """Lengths of maximal runs of comparator-Equal adjacent suffixes."""
    cmp = make_cmp(text, ends, longer_first, max_ctx)
    runs, cur = [], 1
    for i in range(1, len(sa)):
        if cmp(sa[i - 1], sa[i]) == 0:
            cur += 1
        else:
            runs.append(cur)
            cur = 1
    if sa:
        runs.append(cur)
    return runs


def naive_lcp(text, a, b, cap):
    i = 0
    while i < cap and text[a + i] == text[b + i]:
        i += 1
    return i


def lcp_array(text, sa, ends=None, max_ctx=UNB):
    n = len(text)
    out = [0] * len(sa)
    for i in range(1, len(sa)):
        a, b = sa[i - 1], sa[i]
        cap = min(lim_at(n, ends, a), lim_at(n, ends, b))
        if max_ctx is not None:
            cap = min(cap, max_ctx)
        out[i] = naive_lcp(text, a, b, cap)
    return out


def lcg_stream(seed):
    """The LCG of src/pack.rs:353-358."""
    state = seed
    while True:
        state = (state * 6364136223846793005 + 1442695040888963407) & ((1 << 64) - 1)
        yield state >> 33


def spacer_ends(text):
    """spacer_ends (src/pack.rs:566-584)."""
    ends, in_run = [], False
    for i, b in enumerate(text):
        if b == 5:
            if in_run:
                ends.append(i)
                in_run = False
        else:
            in_run = True
    if not ends or ends[-1] != len(text):
        ends.append(len(text))
    return ends


def main():
    fx = {"source": "caps-sa 0.7.0 unit tests (src/lcp.rs, src/limits.rs, "
                    "src/sample_sort.rs, src/pack.rs, src/ext_mem.rs)"}

    # ---- LCP known answers (src/lcp.rs:439-532) ----
    lcp_cases = [
        {"text": list(b"banana"), "p": 0, "q": 1, "max": None, "want": 0, "ref": "src/lcp.rs:442-443"},
        {"text": list(b"banana"), "p": 1, "q": 3, "max": None, "want": 3, "ref": "src/lcp.rs:446"},
        {"text": list(b"aaaaaa"), "p": 0, "q": 1, "max": 3, "want": 3, "ref": "src/lcp.rs:452"},
        {"text": list(b"abc"), "p": 0, "q": 2, "max": None, "want": 0, "ref": "src/lcp.rs:459"},
        {"text": list(b"abc"), "p": 1, "q": 1, "max": None, "want": 2, "ref": "src/lcp.rs:461"},
    ]
    for d in [0, 1, 31, 32, 33, 63, 64, 65, 100]:  # src/lcp.rs:482-491
        t = [ord("A")] * 400
        t[d] = ord("C")
        lcp_cases.append({"text": t, "p": 0, "q": 200, "max": None, "want": d,
                          "ref": "src/lcp.rs:482-491"})
    t = [ord("A")] * 200
    t[64] = ord("T")  # src/lcp.rs:508-516
    lcp_cases.append({"text": t, "p": 0, "q": 100, "max": None, "want": 64, "ref": "src/lcp.rs:508-516"})
    for d in [0, 1, 31, 32, 33, 63, 64, 65, 95, 96, 97, 127, 128, 200]:  # src/lcp.rs:523-532
        t = [ord("A")] * 512
        t[d] = ord("G")
        lcp_cases.append({"text": t, "p": 0, "q": 256, "max": None, "want": d,
                          "ref": "src/lcp.rs:523-532"})
    fx["lcp_u8"] = lcp_cases

    u16 = []
    for bd in [0, 1, 2, 3, 31, 32, 33, 63, 64, 65, 127, 128, 200]:  # src/lcp.rs:546-563
        t = [0xAAAA] * 256
        sym = bd // 2
        mask = 0x00FF if bd % 2 == 0 else 0xFF00
        t[sym] ^= mask & 0xAAAA
        u16.append({"text": t, "p": 0, "q": 128, "want": sym, "ref": "src/lcp.rs:546-563"})
    fx["lcp_u16"] = u16

    fx["suffix_cmp"] = [  # src/lcp.rs:465-473
        {"text": list(b"banana"), "p": 1, "q": 0, "want": -1},
        {"text": list(b"banana"), "p": 3, "q": 1, "want": -1},
        {"text": list(b"banana"), "p": 1, "q": 1, "want": 0},
    ]

    # ---- limits known answers (src/limits.rs:343-422) ----
    fx["limits"] = {
        "plain_100": {"n": 100, "lim": {"0": 100, "50": 50, "99": 1, "100": 0}},
        "seg_3_5_7": {"n": 15, "lengths": [3, 5, 7], "ends": [3, 8, 15],
                      "lim": {"0": 3, "1": 2, "2": 1, "3": 5, "5": 3, "7": 1, "8": 7, "14": 1,
                              "15": 0}},
        "single_10": {"n": 10, "lengths": [10], "lim": {"0": 10, "5": 5, "10": 0}},
        "directory": {"lengths_rule": "1 + i % 97 for i in range(2000)",
                      "ref": "src/limits.rs:390-405"},
        "undercoverage_rejected": {"n": 20, "lengths": [3, 5, 7]},
    }

    # ---- SA fixtures (src/sample_sort.rs:709-1070, src/ext_mem.rs:2785-2806) ----
    sa_cases = []

    def add(name, text, ref, positions=None, ends=None, longer_first=False, max_ctx=UNB,
            want_literal=None):
        sa = brute(text, positions, ends, longer_first, max_ctx)
        if want_literal is not None:
            assert sa == want_literal, (name, sa, want_literal)
        case = {"name": name, "text": list(text), "ref": ref, "positions": positions,
                "ends": ends, "longer_first": longer_first, "max_ctx": max_ctx, "sa": sa,
                "ties": tie_classes(text, sa, ends, longer_first, max_ctx)}
        if positions is None:
            case["lcp"] = lcp_array(text, sa, ends, max_ctx)
        sa_cases.append(case)

    for name, t in [("banana", b"banana"), ("mississippi", b"mississippi"),
                    ("abracadabra", b"abracadabra"), ("a36", b"a" * 36),
                    ("ab14", b"ab" * 14), ("a", b"a"), ("empty", b"")]:
        add(name, t, "src/sample_sort.rs:709-720, 791-811; src/ext_mem.rs:2785-2790")
    add("small_distinct_sentinel", bytes([0, 1, 2, 0, 1, 5, 0, 2, 1, 6]), "src/sample_sort.rs:814-821")
    add("run_7x2000", bytes([7] * 2000), "src/sample_sort.rs:737-738")
    add("periodic_mod3", bytes(i % 3 for i in range(2000)), "src/sample_sort.rs:739-740")
    mixed = bytes(i % 4 for i in range(500)) + bytes([4] * 1500) + bytes(i % 4 for i in range(500))
    add("mixed_run", mixed, "src/sample_sort.rs:742-746")
    rep = b"ACGTACGTACGTACGTACGTACGTACGT" * 100 + bytes([200])
    add("repetitive_unit", rep, "src/ext_mem.rs:2918-2940")
    add("mississippi_even", b"mississippi", "src/sample_sort.rs:835-843",
        positions=list(range(0, 11, 2)))
    hw = b"helloworldbananamississippi"
    hw_ends = [5, 10, 16, 27]
    add("segmented_hello", hw, "src/sample_sort.rs:936-946", ends=hw_ends)
    add("segmented_hello_even", hw, "src/sample_sort.rs:976-988", ends=hw_ends,
        positions=list(range(0, len(hw), 2)))
    add("segmented_single", b"mississippi", "src/sample_sort.rs:948-959", ends=[11])
    add("star_hello", hw, "src/sample_sort.rs:1042-1053", ends=hw_ends, longer_first=True)
    add("star_AAAA", b"AAAA", "src/sample_sort.rs:1059-1070", ends=[4], longer_first=True,
        want_literal=[0, 1, 2, 3])
    # finite context on fixed texts (src/sample_sort.rs:768-789 shapes)
    for c in [0, 1, 2, 4, 16]:
        add("mississippi_ctx%d" % c, b"mississippi", "src/sample_sort.rs:768-789", max_ctx=c)
        add("periodic_ctx%d" % c, bytes(i % 3 for i in range(64)), "src/sample_sort.rs:768-789",
            max_ctx=c)
    fx["sa"] = sa_cases

    # ---- pack known answers (src/pack.rs:423-563) ----
    st = lcg_stream(12345)
    plain_text = [next(st) % 4 for _ in range(4096)]
    st = lcg_stream(999)
    seg_text = [5 if i % 617 < 9 else next(st) % 5 for i in range(8192)]
    st = lcg_stream(4242)
    star_text = [5 if i % 411 < 7 else next(st) % 5 for i in range(8192)]
    k = 32
    segs = [[0] * (k - 1) + [1], [0] * (k - 1) + [2], [1] * k + [0], [1] * k + [2],
            [2] * (k + 1) + [0], [2] * (k + 1) + [1], [0] * (k + 2), [0] * (k + 2)]
    depth_text, starts = [], []
    for s in segs:
        starts.append(len(depth_text))
        depth_text.extend(s)
    fx["pack"] = {
        "lcg_plain": {"seed": 12345, "text_head": plain_text[:16], "n": 4096,
                      "ref": "src/pack.rs:432-437"},
        "lcg_segmented": {"seed": 999, "n": 8192, "ends": spacer_ends(seg_text),
                          "ref": "src/pack.rs:439-458"},
        "lcg_star": {"seed": 4242, "n": 8192, "ends": spacer_ends(star_text),
                     "ref": "src/pack.rs:460-480"},
        "policy_text": [0, 2, 0, 2, 0, 2, 0, 2],
        "policy_want": {"disabled": False, "dense": False, "remap_short": False,
                        "remap_exact": True, "ref": "src/pack.rs:483-513"},
        "bytes_0_254": {"bits": 8, "k": 8, "ref": "src/pack.rs:515-522"},
        "bytes_0_255": {"available": False, "ref": "src/pack.rs:524-527"},
        "depth": {"text": depth_text, "lengths": [len(s) for s in segs], "starts": starts,
                  "k": 32, "ref": "src/pack.rs:530-563"},
    }

    out = os.path.join(HERE, "fixtures.json")
    with open(out, "w") as f:
        json.dump(fx, f, separators=(",", ":"))
    print("wrote", out, os.path.getsize(out), "bytes")


if __name__ == "__main__":
    main()
