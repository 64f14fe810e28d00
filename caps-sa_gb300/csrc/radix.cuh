// radix.cuh — interface of the onesweep LSD radix sort (radix.cu).
#pragma once

#include "common.cuh"

namespace capssa {
namespace radix {

constexpr int kMaxPasses = 8;

// Stable sort of n (key, value) pairs by key bits [begin_bit, end_bit).
// Input in (keys_a, vals_a); the result ends in the "a" or "b" buffers as
// reported by *result_in_b.  With gen_vals the input values are not read:
// value i is val_base + i.  Uses the context's radix workspace slots and
// synchronises once (to read the digit histograms).
capssa_status sort_pairs(Ctx &c, uint64_t *keys_a, uint32_t *vals_a, uint64_t *keys_b,
                         uint32_t *vals_b, uint32_t n, int begin_bit, int end_bit,
                         bool gen_vals, uint32_t val_base, bool *result_in_b,
                         int *passes_run = nullptr, bool hist_ready = false);

// Stable sort of n keys by bits [begin_bit, end_bit) (16 B of traffic per
// key and pass instead of 24): for keys that carry their value in the bits
// below begin_bit.  Same buffers protocol as sort_pairs.
capssa_status sort_keys(Ctx &c, uint64_t *keys_a, uint64_t *keys_b, uint32_t n, int begin_bit,
                        int end_bit, bool *result_in_b, int *passes_run = nullptr,
                        bool hist_ready = false);

// The histogram buffer sort_pairs reads ([pass][256] u32 counts of the
// digits at bits begin_bit + 8*pass).  A producer that already saw every key
// can fill it and pass hist_ready = true to skip the histogram read.
uint32_t *hist_buffer(Ctx &c);

}  // namespace radix
}  // namespace capssa
