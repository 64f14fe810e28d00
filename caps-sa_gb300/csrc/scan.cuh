// scan.cuh — device-wide u32 scan (scan.cu).
#pragma once

#include "common.cuh"

namespace capssa {

// out[i] = op(in[0..i]) (inclusive) or op(in[0..i)) (exclusive; 0 for
// i == 0), op = sum or max.  In place is allowed.
capssa_status scan_u32(Ctx &c, const uint32_t *in, uint32_t *out, uint64_t n, bool max_op,
                       bool inclusive);

}  // namespace capssa
