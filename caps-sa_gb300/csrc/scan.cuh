// scan.cuh — device-wide u32 scan (scan.cu).
#pragma once

#include "common.cuh"

namespace capssa {

// out[i] = op(in[0..i]) (inclusive) or op(in[0..i)) (exclusive; 0 for
// i == 0), op = sum or max.  In place is allowed.
capssa_status scan_u32(Ctx &c, const uint32_t *in, uint32_t *out, uint64_t n, bool max_op,
                       bool inclusive);

// out[off + r] = the r-th entry of sa[0..n) whose bit in `bits` is set (bit
// v of the bitmap for entry value v), as u32 (out_bytes 4) or u64 (8); one
// pass with a decoupled look-back over tile counts.
capssa_status select_bits(Ctx &c, const uint32_t *sa, uint64_t n, const uint32_t *bits,
                          uint64_t off, void *out, int out_bytes);

// dst[idx[i]] = vals ? vals[i] : i for i < m (idx distinct, < n_dst).
// Destinations beyond L2 go window by window through `pairs` (m words) and
// `hist` (scatter_hist_words(m) words); either null scatters directly.
size_t scatter_hist_words(uint64_t m);
capssa_status scatter_u32(Ctx &c, const uint32_t *idx, const uint32_t *vals, uint64_t m,
                          uint32_t *dst, uint64_t n_dst, uint64_t *pairs, uint32_t *hist);

}  // namespace capssa
