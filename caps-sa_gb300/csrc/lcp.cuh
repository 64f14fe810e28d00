// lcp.cuh — warp-cooperative longest-common-prefix search.
//
// GB300 counterpart of LcpDispatch::lcp (src/lcp.rs:125-153) and its
// AVX-512/AVX2/NEON byte kernels (src/lcp.rs:292-431).  Like the reference,
// the text is viewed as bytes and the symbol LCP is byte_lcp / sizeof(S).
// One warp compares 512 bytes per step: each lane takes 16 bytes of both
// suffixes (five aligned 32-bit read-only loads, funnel-shifted to the
// suffix's alignment), XORs them, and __ballot_sync/__ffs pick the first
// lane with a difference.  Device text buffers carry >= 64 bytes of zero
// padding, so the aligned over-read past the last compared byte stays in
// bounds.
#pragma once

#include "common.cuh"

namespace capssa {

// 16 bytes of `t` starting at byte offset `off` (any alignment), as four
// little-endian words.
__device__ __forceinline__ void load16_unaligned(const uint8_t *__restrict__ t, uint64_t off,
                                                 uint32_t w[4]) {
    const uint32_t *base = reinterpret_cast<const uint32_t *>(t + (off & ~3ull));
    const uint32_t sh = (uint32_t)(off & 3) * 8;
    uint32_t r0 = __ldg(base), r1 = __ldg(base + 1), r2 = __ldg(base + 2), r3 = __ldg(base + 3),
             r4 = __ldg(base + 4);
    w[0] = __funnelshift_r(r0, r1, sh);
    w[1] = __funnelshift_r(r1, r2, sh);
    w[2] = __funnelshift_r(r2, r3, sh);
    w[3] = __funnelshift_r(r3, r4, sh);
}

// Index (0..16) of the first differing byte of two 16-byte windows.
__device__ __forceinline__ uint32_t first_diff16(const uint32_t a[4], const uint32_t b[4]) {
#pragma unroll
    for (int i = 0; i < 4; i++) {
        uint32_t x = a[i] ^ b[i];
        if (x) return (uint32_t)i * 4 + ((uint32_t)__ffs((int)x) - 1) / 8;
    }
    return 16;
}

// First differing byte of t[pa..] and t[pb..] below `lim` bytes; every lane
// of the (full) warp must call it with the same arguments and gets the
// same result.
__device__ __forceinline__ uint64_t warp_lcp_bytes(const uint8_t *__restrict__ t, uint64_t pa,
                                                   uint64_t pb, uint64_t lim) {
    const uint32_t lane = threadIdx.x & 31;
    for (uint64_t i = 0; i < lim; i += 512) {
        uint64_t off = i + (uint64_t)lane * 16;
        uint32_t d = 16;
        if (off < lim) {
            uint32_t wa[4], wb[4];
            load16_unaligned(t, pa + off, wa);
            load16_unaligned(t, pb + off, wb);
            d = first_diff16(wa, wb);
            if (off + d >= lim) d = 16;  // differences at or past lim do not count
        }
        unsigned ball = __ballot_sync(0xffffffffu, d < 16);
        if (ball) {
            int src = __ffs((int)ball) - 1;
            uint64_t at = __shfl_sync(0xffffffffu, off + d, src);
            return at < lim ? at : lim;
        }
    }
    return lim;
}

// One thread's LCP: 16 bytes per step; for short LCPs (the common case on
// high-entropy text) this beats waking a whole warp.
__device__ __forceinline__ uint64_t thread_lcp_bytes(const uint8_t *__restrict__ t, uint64_t pa,
                                                     uint64_t pb, uint64_t lim) {
    for (uint64_t i = 0; i < lim; i += 16) {
        uint32_t wa[4], wb[4];
        load16_unaligned(t, pa + i, wa);
        load16_unaligned(t, pb + i, wb);
        uint32_t d = first_diff16(wa, wb);
        if (d < 16) return i + d < lim ? i + d : lim;
    }
    return lim;
}

__device__ __forceinline__ uint64_t sat_mul_dev(uint64_t a, uint64_t b) {
    if (a == 0 || b == 0) return 0;
    if (a > ~0ull / b) return ~0ull;
    return a * b;
}

__device__ __forceinline__ uint64_t sym_at(const void *text, int sym_bytes, uint64_t i) {
    if (sym_bytes == 1) return ((const uint8_t *)text)[i];
    if (sym_bytes == 2) return ((const uint16_t *)text)[i];
    return ((const uint32_t *)text)[i];
}

// LcpDispatch::lcp: symbol LCP of text[p..], text[q..] bounded by
// min(n - p, n - q, max_ctx) (src/lcp.rs:125-153).  Warp-wide.
__device__ __forceinline__ uint64_t warp_sym_lcp(const void *text, int sym_bytes, uint64_t n,
                                                 uint64_t p, uint64_t q, uint64_t max_ctx) {
    uint64_t lp = n > p ? n - p : 0, lq = n > q ? n - q : 0;
    uint64_t lim = lp < lq ? lp : lq;
    if (max_ctx < lim) lim = max_ctx;
    const uint64_t k = (uint64_t)sym_bytes;
    uint64_t b = warp_lcp_bytes((const uint8_t *)text, p * k, q * k, lim * k);
    return b / k;
}

// Host-side entry points implemented in lcp.cu.
capssa_status lcp_array_sa(Ctx &c, const void *text, int sym_bytes, uint64_t n,
                           const DevLimits &L, uint64_t max_ctx, const uint32_t *sa, uint64_t m,
                           void *out_lcp, int out_bytes);
capssa_status lcp_pairs(Ctx &c, const void *text, int sym_bytes, uint64_t n, const uint64_t *p,
                        const uint64_t *q, uint64_t count, uint64_t max_ctx, uint64_t *out);
capssa_status suffix_cmp_pairs(Ctx &c, const void *text, int sym_bytes, const DevLimits &L,
                               const uint64_t *p, const uint64_t *q, uint64_t count,
                               uint64_t max_ctx, int8_t *out);
// Flags of adjacent SA pairs that agree through max_ctx symbols with both
// limits >= max_ctx: flag[i] for pair (sa[i-1], sa[i]); flag[0] = 0.
capssa_status ctx_run_flags(Ctx &c, const void *text, int sym_bytes, const DevLimits &L,
                            uint64_t max_ctx, const uint32_t *sa, uint64_t m, uint8_t *flags);
// sample_sort::merge on the device (merge path + LCP-carrying sequential
// segments); idx_bytes 4 or 8.
capssa_status merge_runs(Ctx &c, const void *text, int sym_bytes, const DevLimits &L,
                         const void *x, const void *lcp_x, uint64_t len_x, const void *y,
                         const void *lcp_y, uint64_t len_y, uint64_t max_ctx, void *z,
                         void *lcp_z, int idx_bytes);

}  // namespace capssa
