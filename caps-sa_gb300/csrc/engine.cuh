// engine.cuh — the suffix sort behind every builder.
//
// Replaces the reference's merge_sort + LCP-merge recursion
// (src/sample_sort.rs:168-348) and the packed-prefix seed
// (src/pack.rs:241-321) with a GPU pipeline that produces the same order:
//
//  1. alphabet scan -> order-preserving dense codes (Packer::new,
//     src/pack.rs:103-167), b bits per symbol;
//  2. one composite record per text position: the first k symbols of the
//     suffix, truncated at its limit (min(k, lim_at(p)), as key_at_bounded
//     does, src/pack.rs:187-203), padded, followed by a length field (the
//     number of symbols taken), a one-bit "ended early" flag (plain texts),
//     or nothing (flagless plain texts, whose k - 1 short suffixes are left
//     out of the sort and placed afterwards); the position rides below the
//     key when it fits, and a segment index above it in segment-major order.
//     Key order never contradicts suffix_cmp_with (src/lcp.rs:184-201);
//  3. stable LSD radix sort of the records;
//  4. the groups still tied are resolved by size class: direct comparison
//     on a bit-packed copy of the text for groups of up to 2048 members and
//     depths up to 4096 symbols, rank doubling for the rest (a suffix p of
//     a group of depth h is re-keyed by the rank of p + h, or by "ended"
//     when lim_at(p) == h; ranks are group-head SA indices, so equal rank ==
//     equal comparison so far).

// Boundary orders: ShorterFirst (the default boundary_order) leaves suffixes
// that end together with equal content tied; their output order is
// ascending position.  LongerFirst (STAR) orders them by position, which the
// stable sorts produce directly.
#pragma once

#include "common.cuh"

namespace capssa {

struct EngineArgs {
    const void *text;      // device, padded with >= 64 zero bytes
    int sym_bytes;         // 1, 2, 4
    uint64_t n;
    DevLimits lim;
    uint64_t max_ctx;      // CAPSSA_UNBOUNDED or finite
    const void *positions; // device or nullptr (= every position)
    int pos_bytes;         // 4 or 8
    // instead of positions: one bit per kept position (device, n bits), m of
    // them set; the kept suffixes come out in suffix order
    const uint32_t *keep_bits;
    uint64_t m;
    void *out_sa;          // device, m (or n) entries of out_bytes
    int out_bytes;         // 4 or 8
    void *out_lcp;         // device or nullptr
    int seg_major;         // 1: sort by (segment, suffix): every segment's suffixes
                           // contiguous, in their own order (many independent texts)
    uint64_t seg_max_len;  // seg_major: the longest segment
    // sample-sort partition plan (build_in_memory_sample_sort's phases 1-3,
    // src/ext_mem.rs:1191-1428), computed after the sort when part_p > 0
    uint32_t part_p;         // subproblems
    int part_mode;           // CAPSSA_PARTITION_SPLITTERS or CAPSSA_PARTITION_LEARNED
    uint64_t *part_pivots;   // host, part_p - 1 entries (out) or nullptr
    uint64_t *part_sizes;    // host, part_p entries (out) or nullptr
    int part_first;          // 1: partition before the sort (CAPSSA_SAMPLING_PARTITION_FIRST)
    int tie_ref;             // 1: tie classes in the reference's merge order (ties.cu)
};

// Runs the whole sort; all buffers are device buffers.
capssa_status engine_build_u8(Ctx &c, const EngineArgs &a);
capssa_status engine_build_u16(Ctx &c, const EngineArgs &a);
capssa_status engine_build_u32(Ctx &c, const EngineArgs &a);

inline capssa_status engine_build(Ctx &c, const EngineArgs &a) {
    switch (a.sym_bytes) {
    case 1: return engine_build_u8(c, a);
    case 2: return engine_build_u16(c, a);
    default: return engine_build_u32(c, a);
    }
}

// Key geometry for b bits per symbol and n symbols (api.cu).
struct KeyGeom {
    int b;         // bits per symbol
    int k;         // symbols per key
    int lbits;     // bits of the length field
    int total;     // k*b + lbits
    int flag_len;  // 1: the length field is one "ended early" flag (plain texts)
    int vbits;     // > 0: the position is packed below the key in vbits bits
    // 1: no length field at all (lbits 0, flag_len 2).  Only for ShorterFirst
    // plain texts, when the flag bit alone would cost a radix pass: the k - 1
    // suffixes that end inside the key are left out of the sort and placed
    // afterwards (a short suffix precedes exactly the full suffixes whose
    // key is >= its zero-padded key).
    int flagless;
    // 1: the packed position is local to its segment (segment-major keys)
    int local_pos;
};
// plain: the limits are PlainText's (only the last k-1 suffixes end early);
// hbits: entropy of the symbols in bits (<= b).
// top_bits: bits the caller keeps above the key (a segment index), n_k: the
// longest run of symbols a key has to tell apart (n when 0), allow_flagless:
// a ShorterFirst plain text may drop the early-end flag (see KeyGeom);
// seg_flag: a segment-major ShorterFirst sort may mark the suffixes that end
// inside the key with one flag bit instead of a length field.
KeyGeom key_geom(int b, uint64_t n, bool plain, double hbits, int top_bits = 0,
                 uint64_t n_k = 0, bool allow_flagless = false, bool seg_flag = false);

// Key geometry of a partition-first sort: a bucket index of bucket_bits
// above a window of k symbols taken after the bucket's common prefix, a
// flag (plain) or length field, and the global position below (k = 0: no
// geometry packs the position with at least one symbol).
KeyGeom pf_geom(int b, uint64_t n, bool plain, double hbits, int bucket_bits);

}  // namespace capssa
