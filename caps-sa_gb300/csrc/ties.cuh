// ties.cuh — the reference's order inside comparator tie classes (ties.cu).
#pragma once

#include "common.cuh"

namespace capssa {

// One suffix order whose tie classes (runs of suffixes the comparator calls
// Equal) are in ascending input order, to be put in the reference's order.
struct TieArgs {
    const void *text;       // device text, sym_bytes per symbol, padded
    int sym_bytes;
    DevLimits lim;
    uint64_t max_ctx;
    void *out;              // m positions in suffix order (u32 or u64), rewritten in place
    int out_bytes;
    uint64_t m;
    const uint32_t *key;    // per slot of `out`, equal exactly within a tie class; null:
                            // adjacent suffixes are compared
    const void *positions;  // the caller's positions in input order (device); null: out
                            // is a permutation of 0..m-1 (a whole-text build)
    int pos_bytes;
};

// Reorders every tie class of t.out (m >= 2 suffixes, ShorterFirst) as the
// reference's merge sort emits it; reports the class count in stats.
capssa_status reference_tie_order(Ctx &c, const TieArgs &t);

}  // namespace capssa
