// engine_impl.cuh — kernels and host orchestration of the suffix sort
// (see engine.cuh for the algorithm and its correspondence to the
// reference).  Instantiated once per symbol type by engine_u8.cu,
// engine_u16.cu and engine_u32.cu.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <type_traits>
#include <vector>

#include "engine.cuh"
#include "cdf.cuh"
#include "lcp.cuh"
#include "radix.cuh"
#include "scan.cuh"
#include "ties.cuh"

namespace capssa {
namespace {  // every kernel and helper is private to its engine_*.cu unit
namespace eng {

constexpr uint32_t kSmallMax = 32;    // tied groups up to this size: one warp each (pairs: one thread)
constexpr uint32_t kMediumMax = 2048; // up to this size: one block, direct comparisons
constexpr uint64_t kDirectCap = 256;   // symbols compared past the shared prefix (at least it)
constexpr uint64_t kDirectMaxH = 4096; // deeper groups fall back to rank doubling
constexpr int kKeyThreads = 256;
constexpr int kKeyPer = 8;          // positions per thread in the key kernel
constexpr int kKeyTile = kKeyThreads * kKeyPer;

struct BigGroup {
    uint32_t start, len, toff;
    uint32_t depth;  // symbols its members are known to agree on (saturated)
};

// Work lists of one refinement round, by group size and depth.
enum GroupList : int {
    L_PAIR = 0,    // 2 members: one thread
    L_TINY = 1,    // 3..4 members: one thread
    L_SMALL = 2,   // 9..32 members: one warp
    L_MEDIUM = 3,  // 33..kMediumMax members: one block
    L_DEEP = 4,    // <= 32 members deeper than kDirectMaxH: rank doubling
    L_TINY8 = 5,   // 5..8 members: eight lanes
    kLists = 6     // larger groups: the radix (rank doubling) path
};
constexpr uint32_t kTinyMax = 8;
constexpr uint32_t kTiny4 = 4;
constexpr int kPairBurst = 4;  // windows the pair kernel loads in its first round trip

// Device counters of the refinement rounds, double-buffered by round parity.
struct Counters {
    uint32_t n[kLists][2];
    unsigned long long big_packed[2];  // (ordinal << 40) | element total
};
constexpr unsigned long long kBigOrdUnit = 1ull << 40;
constexpr unsigned long long kBigTotMask = kBigOrdUnit - 1;

// ---------------------------------------------------------------- alphabet

template <typename S>
__global__ void presence_kernel(const S *__restrict__ text, uint64_t n,
                                uint32_t *__restrict__ present) {
    // u8: per-block flags in shared memory, merged once per block; u16:
    // idempotent global flags, read first so repeats cost no write traffic.
    if (sizeof(S) == 1) {
        __shared__ uint32_t f[256];
        f[threadIdx.x & 255] = 0;
        __syncthreads();
        const uint64_t nv = n / 16;
        const uint4 *t4 = reinterpret_cast<const uint4 *>(text);
        for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nv;
             i += (uint64_t)gridDim.x * blockDim.x) {
            uint4 v = t4[i];
            uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int j = 0; j < 16; j++) f[(w[j >> 2] >> ((j & 3) * 8)) & 255] = 1;
        }
        for (uint64_t i = nv * 16 + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
             i += (uint64_t)gridDim.x * blockDim.x)
            f[(uint32_t)text[i]] = 1;
        __syncthreads();
        for (int i = threadIdx.x; i < 256; i += blockDim.x)
            if (f[i] && __ldcg(present + i) == 0) present[i] = 1;
        return;
    }
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t s = (uint32_t)text[i];
        if (__ldcg(present + s) == 0) present[s] = 1;
    }
}

// Every stride-th symbol (the entropy estimate's sample).
template <typename S>
__global__ void strided_sample_kernel(const S *__restrict__ text, uint64_t ns, uint64_t stride,
                                      S *__restrict__ out) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < ns;
         i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = text[i * stride];
}

__global__ void minmax_kernel(const uint32_t *__restrict__ text, uint64_t n,
                              uint32_t *__restrict__ mm) {
    uint32_t lo = 0xFFFFFFFFu, hi = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t s = text[i];
        lo = min(lo, s);
        hi = max(hi, s);
    }
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(mm, lo);
        atomicMax(mm + 1, hi);
    }
}

// ---------------------------------------------------------------- keys

// Code of one symbol: a u8/u16 table (order-preserving dense ranks) or an
// offset from the smallest symbol (u32 texts).
template <typename S>
struct Coder {
    const uint16_t *table;  // device, 256 or 65536 entries (nullptr: offset)
    uint32_t minv;
    __device__ __forceinline__ uint32_t operator()(S s) const {
        return table ? (uint32_t)__ldg(table + (uint32_t)s) : (uint32_t)s - minv;
    }
};

struct Packed {
    const uint64_t *w;  // MSB-first b-bit codes, zero padded
    int b;              // bits per symbol
    int spw;            // whole symbols per 64-bit window
    uint64_t mask;      // the spw*b leading bits
};

// 64-bit window of the packed text starting at symbol p.
__device__ __forceinline__ uint64_t window_at(const Packed &P, uint64_t p) {
    uint64_t s = p * (uint64_t)P.b;
    uint64_t wi = s >> 6;
    uint32_t sh = (uint32_t)(s & 63);
    uint64_t v = __ldg(P.w + wi);
    if (sh) v = (v << sh) | (__ldg(P.w + wi + 1) >> (64 - sh));
    return v & P.mask;
}

// Composite key of every text position (engine.cuh step 2), with the digit
// histograms of every radix pass accumulated on the way (so the sort needs
// no separate histogram read of the keys).  The k-symbol content of each
// suffix is read straight from the packed text (two 64-bit loads, shared by
// the neighbouring threads' positions); only suffixes that end inside the
// window (lim < k) are masked and padded.  Each thread owns kKeyPer
// consecutive positions of a tile (the segment end is tracked across
// them); blocks stride over the tiles and add their histograms to the
// global counts once.  With vbits > 0 the position is packed below the key
// (one 64-bit word per suffix).  kPlain: a PlainText text with no segment
// index (limits are n - p, nothing to track).
template <bool kPlain>
__global__ void __launch_bounds__(kKeyThreads)
    key_kernel(Packed P, uint64_t n, uint64_t n_rec, DevLimits L, int k, int lbits, int flag_len,
               int vbits, int lf, int n_passes, int seg_shift, int local_pos,
               uint64_t *__restrict__ keys, uint32_t *__restrict__ counts) {
    __shared__ uint32_t hist[8 * 256];
    for (int i = threadIdx.x; i < n_passes * 256; i += kKeyThreads) hist[i] = 0;
    __syncthreads();
    const int b = P.b;
    const int kbits = k * b;  // 1..63
    for (uint64_t t0 = (uint64_t)blockIdx.x * kKeyTile; t0 < n_rec;
         t0 += (uint64_t)gridDim.x * kKeyTile) {
        const uint64_t p0 = t0 + (uint64_t)threadIdx.x * kKeyPer;
        if (p0 >= n_rec) continue;
        // one past the last symbol of p0's suffix
        uint64_t end = kPlain ? n : p0 + dev_lim_at(L, p0);
        // segment-major keys carry the segment index above the key bits
        uint64_t seg = !kPlain && seg_shift ? dev_seg_at(L, p0) : 0;
        // first position of p0's segment (segment-local packed positions)
        uint64_t start = !kPlain && local_pos && seg ? __ldg(L.ends + seg - 1) : 0;
        uint64_t out[kKeyPer];
#pragma unroll
        for (int e = 0; e < kKeyPer; e++) {
            const uint64_t p = p0 + e;
            uint64_t key = 0;
            if (p < n_rec) {
                if (!kPlain && p >= end) {  // p == end: the next segment starts here
                    end = p + dev_lim_at(L, p);
                    seg++;
                    if (local_pos) start = p;
                }
                const uint64_t bit = p * (uint64_t)b;
                const uint64_t wi = bit >> 6;
                const uint32_t sh = (uint32_t)(bit & 63);
                const uint64_t w0 = __ldg(P.w + wi), w1 = __ldg(P.w + wi + 1);
                uint64_t content = ((w0 << sh) | ((w1 >> 1) >> (63 - sh))) >> (64 - kbits);
                const uint64_t lim = end - p;
                int take = k;
                if (lim < (uint64_t)k) {
                    take = (int)lim;
                    const uint64_t lowmask = (1ull << ((k - take) * b)) - 1;
                    content = lf ? (content | lowmask) : (content & ~lowmask);
                }
                // length field: symbols taken (ShorterFirst) or missing
                // (LongerFirst); or one flag that orders an early end first
                // (ShorterFirst) or last (LongerFirst) among equal contents
                const uint64_t field = flag_len ? (uint64_t)((take == k) != (lf != 0))
                                                : (uint64_t)(lf ? k - take : take);
                key = lbits ? (content << lbits) | field : content;
                if (!kPlain && seg_shift) key |= seg << seg_shift;
                const uint32_t lo = (uint32_t)key, hi = (uint32_t)(key >> 32);
#pragma unroll
                for (int ps = 0; ps < 8; ps++)
                    if (ps < n_passes)
                        atomicAdd(&hist[ps * 256 + (((ps < 4 ? lo : hi) >> (8 * (ps & 3))) & 255u)],
                                  1u);
                if (vbits) key = (key << vbits) | (p - start);
            }
            out[e] = key;
        }
        if (p0 + kKeyPer <= n_rec) {
            uint4 *dst = reinterpret_cast<uint4 *>(keys + p0);
#pragma unroll
            for (int e = 0; e < kKeyPer; e += 2)
                dst[e / 2] = make_uint4((uint32_t)out[e], (uint32_t)(out[e] >> 32),
                                        (uint32_t)out[e + 1], (uint32_t)(out[e + 1] >> 32));
        } else {
            for (int e = 0; e < kKeyPer; e++)
                if (p0 + e < n_rec) keys[p0 + e] = out[e];
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n_passes * 256; i += kKeyThreads)
        if (hist[i]) atomicAdd(&counts[i], hist[i]);
}

// key_kernel for a plain text in the flagless geometry when a radix digit
// holds whole symbols (b divides 8) and the key whole digits.  Every record
// is a full window (p <= n - k), so there is no limit, flag or segment
// logic; a thread's kKeyPer windows lie in the two packed words at its
// first position (its bit offset is a multiple of 8b, so offset + 7b < 64).
// Only pass 0's digit histogram is counted: key_hist_shift_kernel derives
// the other passes' from it.
__global__ void __launch_bounds__(kKeyThreads)
    key_flagless_kernel(Packed P, uint64_t n_rec, int kbits, int vbits,
                        uint64_t *__restrict__ keys, uint32_t *__restrict__ counts) {
    static_assert(kKeyThreads == 256 && kKeyPer == 8, "one thread per digit; 8 windows per word pair");
    __shared__ uint32_t hist[256];
    hist[threadIdx.x] = 0;
    __syncthreads();
    const int b = P.b;
    for (uint64_t t0 = (uint64_t)blockIdx.x * kKeyTile; t0 < n_rec;
         t0 += (uint64_t)gridDim.x * kKeyTile) {
        const uint64_t p0 = t0 + (uint64_t)threadIdx.x * kKeyPer;
        if (p0 >= n_rec) continue;
        const uint64_t bit0 = p0 * (uint64_t)b;
        const uint64_t w0 = __ldg(P.w + (bit0 >> 6)), w1 = __ldg(P.w + (bit0 >> 6) + 1);
        const uint32_t sh0 = (uint32_t)(bit0 & 63);
        uint64_t out[kKeyPer];
#pragma unroll
        for (int e = 0; e < kKeyPer; e++) {
            const uint32_t sh = sh0 + (uint32_t)(e * b);
            const uint64_t content = ((w0 << sh) | ((w1 >> 1) >> (63 - sh))) >> (64 - kbits);
            if (p0 + e < n_rec) atomicAdd(&hist[(uint32_t)content & 255u], 1u);
            out[e] = (content << vbits) | (p0 + e);
        }
        if (p0 + kKeyPer <= n_rec) {
            uint4 *dst = reinterpret_cast<uint4 *>(keys + p0);
#pragma unroll
            for (int e = 0; e < kKeyPer; e += 2)
                dst[e / 2] = make_uint4((uint32_t)out[e], (uint32_t)(out[e] >> 32),
                                        (uint32_t)out[e + 1], (uint32_t)(out[e + 1] >> 32));
        } else {
            for (int e = 0; e < kKeyPer; e++)
                if (p0 + e < n_rec) keys[p0 + e] = out[e];
        }
    }
    __syncthreads();
    if (hist[threadIdx.x]) atomicAdd(&counts[threadIdx.x], hist[threadIdx.x]);
}

// Digit histograms of radix passes 1.. from pass 0's (key_flagless_kernel).
// Digit j of record p is the s8 = 8 / b symbols at p + k - (j + 1) s8, which
// is digit 0 of record p - j s8.  So pass j counts pass 0's records except
// the last j s8, plus digit j of the first j s8 records (needs n_rec >= j s8).
// One block of 256 threads, one per digit value.
__global__ void key_hist_shift_kernel(Packed P, uint64_t n_rec, int kbits, int n_passes,
                                      uint32_t *__restrict__ counts) {
    const uint32_t x = threadIdx.x;
    const uint32_t h0 = counts[x];
    const uint64_t s8 = 8 / (uint64_t)P.b;
    for (int j = 1; j < n_passes; j++) {
        uint32_t h = h0;
        for (uint64_t q = 0; q < (uint64_t)j * s8; q++) {
            const uint64_t tail = window_at(P, n_rec - 1 - q) >> (64 - kbits);
            const uint64_t head = window_at(P, q) >> (64 - kbits);
            h -= ((uint32_t)tail & 255u) == x ? 1u : 0u;
            h += ((uint32_t)(head >> (8 * j)) & 255u) == x ? 1u : 0u;
        }
        counts[j * 256 + x] = h;
    }
}

// Composite key of each of m chosen positions (a subset sorted on its own):
// the same record as key_kernel's, read at pos[i] (distinct, ascending,
// < n), with the digit histograms of every radix pass.
template <bool kPlain>
__global__ void __launch_bounds__(kKeyThreads)
    sparse_key_kernel(Packed P, uint64_t n, const uint32_t *__restrict__ pos, uint64_t m,
                      DevLimits L, int k, int lbits, int flag_len, int vbits, int lf,
                      int n_passes, uint64_t *__restrict__ keys, uint32_t *__restrict__ counts) {
    __shared__ uint32_t hist[8 * 256];
    for (int i = threadIdx.x; i < n_passes * 256; i += kKeyThreads) hist[i] = 0;
    __syncthreads();
    const int b = P.b;
    const int kbits = k * b;
    for (uint64_t i = blockIdx.x * (uint64_t)kKeyThreads + threadIdx.x; i < m;
         i += (uint64_t)gridDim.x * kKeyThreads) {
        const uint64_t p = pos[i];
        const uint64_t lim = kPlain ? n - p : dev_lim_at(L, p);
        const uint64_t bit = p * (uint64_t)b;
        const uint64_t wi = bit >> 6;
        const uint32_t sh = (uint32_t)(bit & 63);
        const uint64_t w0 = __ldg(P.w + wi), w1 = __ldg(P.w + wi + 1);
        uint64_t content = ((w0 << sh) | ((w1 >> 1) >> (63 - sh))) >> (64 - kbits);
        int take = k;
        if (lim < (uint64_t)k) {
            take = (int)lim;
            const uint64_t lowmask = (1ull << ((k - take) * b)) - 1;
            content = lf ? (content | lowmask) : (content & ~lowmask);
        }
        const uint64_t field = flag_len ? (uint64_t)((take == k) != (lf != 0))
                                        : (uint64_t)(lf ? k - take : take);
        uint64_t key = lbits ? (content << lbits) | field : content;
        const uint32_t lo = (uint32_t)key, hi = (uint32_t)(key >> 32);
#pragma unroll
        for (int ps = 0; ps < 8; ps++)
            if (ps < n_passes)
                atomicAdd(&hist[ps * 256 + (((ps < 4 ? lo : hi) >> (8 * (ps & 3))) & 255u)], 1u);
        if (vbits) key = (key << vbits) | p;
        keys[i] = key;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n_passes * 256; i += kKeyThreads)
        if (hist[i]) atomicAdd(&counts[i], hist[i]);
}

// Population count of every bitmap word (the chosen positions per word).
__global__ void bits_popc_kernel(const uint32_t *__restrict__ bits, uint64_t nw,
                                 uint32_t *__restrict__ cnt) {
    for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < nw;
         w += (uint64_t)gridDim.x * blockDim.x)
        cnt[w] = (uint32_t)__popc(bits[w]);
}

// The set bits of the bitmap as ascending positions (incl = inclusive prefix
// of the word counts).
__global__ void bits_expand_kernel(const uint32_t *__restrict__ bits, uint64_t nw,
                                   const uint32_t *__restrict__ incl, uint32_t *__restrict__ pos) {
    for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < nw;
         w += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t x = bits[w];
        uint32_t o = incl[w] - (uint32_t)__popc(x);
        while (x) {
            const int j = __ffs((int)x) - 1;
            pos[o++] = (uint32_t)(w * 32 + (uint64_t)j);
            x &= x - 1;
        }
    }
}

// ---------------------------------------------------------------- groups

// First index of the run of `key` that contains sorted index i.
__device__ __forceinline__ uint32_t run_head(const uint64_t *__restrict__ keys, uint32_t lo,
                                             uint32_t i, uint64_t key, int vshift = 0) {
    uint32_t j = i;
    uint32_t stop = (i - lo > 32) ? i - 32 : lo;
    while (j > stop && (keys[j - 1] >> vshift) == key) j--;
    if (j > stop || j == lo) return j;
    // long run: binary search for the first index in [lo, j) equal to key
    uint32_t a = lo, z = j;
    while (a < z) {
        uint32_t mid = a + ((z - a) >> 1);
        if ((keys[mid] >> vshift) < key)
            a = mid + 1;
        else
            z = mid;
    }
    return a;
}

struct GroupLists {
    uint4 *list[kLists][2];  // (start, len, depth, 0)
    BigGroup *big[2];
    Counters *ctr;
};

// The lists are kernel parameters: indexing them with a runtime value would
// copy the whole struct to local memory in every thread, so pick by select.
__device__ __forceinline__ uint4 *list_ptr(const GroupLists &G, int l, int q) {
    uint4 *r = nullptr;
#pragma unroll
    for (int i = 0; i < kLists; i++) r = l == i ? (q ? G.list[i][1] : G.list[i][0]) : r;
    return r;
}
__device__ __forceinline__ BigGroup *big_ptr(const GroupLists &G, int q) {
    return q ? G.big[1] : G.big[0];
}

// List of a still-tied group whose members agree on `depth` symbols
// (kLists = the radix path).
__device__ __forceinline__ int list_of(uint32_t len, uint64_t depth) {
    if (len <= kSmallMax && depth > kDirectMaxH) return L_DEEP;
    if (len == 2) return L_PAIR;
    if (len <= kTiny4) return L_TINY;
    if (len <= kTinyMax) return L_TINY8;
    if (len <= kSmallMax) return L_SMALL;
    if (len <= kMediumMax && depth <= kDirectMaxH) return L_MEDIUM;
    return kLists;
}

// A pair entry that carries its two positions: (start, position at start,
// depth | kPairPos, position at start + 1), so the pair kernel reads no SA
// entries (group init writes these; pair depths stay below kDirectMaxH).
constexpr uint32_t kPairPos = 0x80000000u;

__device__ __forceinline__ uint4 group_entry(uint32_t start, uint32_t len, uint64_t depth) {
    return make_uint4(start, len, depth > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)depth, 0u);
}

__device__ __forceinline__ void append_big(const GroupLists &G, int nxt, uint32_t start,
                                           uint32_t len, uint64_t depth) {
    unsigned long long old = atomicAdd(&G.ctr->big_packed[nxt], kBigOrdUnit | len);
    uint32_t ord = (uint32_t)(old >> 40);
    BigGroup g;
    g.start = start;
    g.len = len;
    g.toff = (uint32_t)(old & kBigTotMask);
    g.depth = depth > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)depth;
    big_ptr(G, nxt)[ord] = g;
}

// Slot in a list for every thread of the warp that calls this together
// with the same `counter`: one atomic per warp instead of one per thread.
// Same-address atomics serialise in L2 (a few ns each), so the heavy
// producers use block_append below instead.
__device__ __forceinline__ uint32_t warp_append(uint32_t *counter) {
    const unsigned mask = __activemask();
    const unsigned peers = __match_any_sync(mask, (unsigned long long)counter);
    const int lane = threadIdx.x & 31;
    const int leader = __ffs((int)peers) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(counter, (uint32_t)__popc(peers));
    base = __shfl_sync(peers, base, leader);
    return base + (uint32_t)__popc(peers & ((1u << lane) - 1u));
}

// Route a still-tied group to the next round's list (any thread, any time).
__device__ __forceinline__ void append_group(const GroupLists &G, int nxt, uint32_t start,
                                             uint32_t len, uint64_t depth) {
    int l = list_of(len, depth);
    if (l == kLists) {
        append_big(G, nxt, start, len, depth);
        return;
    }
    uint32_t idx = warp_append(&G.ctr->n[l][nxt]);
    list_ptr(G, l, nxt)[idx] = group_entry(start, len, depth);
}

// Block-wide append: every thread of the block calls this at the same
// point with at most one group (want); one global atomic per list per
// block.  The block's entries of a list are contiguous.
__device__ __forceinline__ void block_append(const GroupLists &G, int nxt, bool want,
                                             uint32_t start, uint32_t len, uint64_t depth) {
    __shared__ uint32_t s_cnt[kLists], s_base[kLists];
    const int l = want ? list_of(len, depth) : -1;
    if (threadIdx.x < kLists) s_cnt[threadIdx.x] = 0;
    __syncthreads();
    uint32_t local = 0;
    if (l >= 0 && l < kLists) local = atomicAdd(&s_cnt[l], 1u);
    __syncthreads();
    if (threadIdx.x < kLists && s_cnt[threadIdx.x])
        s_base[threadIdx.x] = atomicAdd(&G.ctr->n[threadIdx.x][nxt], s_cnt[threadIdx.x]);
    __syncthreads();
    if (l >= 0 && l < kLists) list_ptr(G, l, nxt)[s_base[l] + local] = group_entry(start, len, depth);
    if (l == kLists) append_big(G, nxt, start, len, depth);
}

// Exclusive block-wide prefix of one u32 per thread; returns the block total.
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t *excl) {
    __shared__ uint32_t s_w[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_w[warp] = x;
    __syncthreads();
    uint32_t before = 0, total = 0;
    for (int w = 0; w < nw; w++) {
        uint32_t t = s_w[w];
        if (w < warp) before += t;
        total += t;
    }
    __syncthreads();
    *excl = before + x - v;
    return total;
}

// Exclusive block-wide prefix of one u64 per thread (used for several
// 16-bit counters packed in one word); returns the block total.
__device__ __forceinline__ uint64_t block_excl_scan64(uint64_t v, uint64_t *excl) {
    __shared__ uint64_t s_w64[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint64_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint64_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_w64[warp] = x;
    __syncthreads();
    uint64_t before = 0, total = 0;
    for (int w = 0; w < nw; w++) {
        uint64_t t = s_w64[w];
        if (w < warp) before += t;
        total += t;
    }
    __syncthreads();
    *excl = before + x - v;
    return total;
}

// The short suffixes of a flagless sort (KeyGeom::flagless), in device
// memory: ip[] ascending, one insertion point per short suffix (sorted record
// i moves up to SA index i + #{ip <= i}), and each short suffix's own SA
// slot and position.
struct ShortList {
    uint32_t n;
    uint32_t ip[63];
    uint32_t slot[63];
    uint32_t pos[63];
};

__device__ __forceinline__ uint32_t short_shift(const ShortList *S, uint32_t ns, uint32_t i) {
    uint32_t c = 0;
    for (uint32_t j = 0; j < ns; j++) c += __ldg(&S->ip[j]) <= i ? 1u : 0u;
    return c;
}

// Places the short suffixes n_rec + j of a flagless sort (one block): each
// one's key (first lim symbols, zero padded) and insertion point, the number
// of sorted records with a smaller key (a short suffix precedes every full
// suffix whose key is at least its padded key, ShorterFirst); ordered among
// themselves by key, equal keys shorter first.
__global__ void short_place_kernel(Packed P, uint64_t n, uint32_t n_rec, int k,
                                   const uint64_t *__restrict__ recs, int vbits,
                                   ShortList *__restrict__ S) {
    __shared__ uint64_t s_key[64];
    const uint32_t j = threadIdx.x;
    const uint32_t ns = (uint32_t)(n - n_rec);
    uint64_t key = 0;
    uint32_t ip = 0;
    if (j < ns) {
        const uint64_t sp = n_rec + (uint64_t)j;
        const int take = (int)(n - sp);  // < k
        key = window_at(P, sp) >> (64 - k * P.b);
        key &= ~((1ull << ((k - take) * P.b)) - 1);
        uint32_t lo = 0, hi = n_rec;
        while (lo < hi) {
            const uint32_t mid = lo + ((hi - lo) >> 1);
            if ((recs[mid] >> vbits) < key)
                lo = mid + 1;
            else
                hi = mid;
        }
        ip = lo;
        s_key[j] = key;
    }
    __syncthreads();
    if (j < ns) {
        uint32_t r = 0;  // short suffixes ordered before this one
        for (uint32_t q = 0; q < ns; q++)
            if (s_key[q] < key || (s_key[q] == key && q > j)) r++;
        S->ip[r] = ip;
        S->slot[r] = ip + r;
        S->pos[r] = n_rec + j;
    }
    if (j == 0) S->n = ns;
}

// The short suffixes' own SA slots (singleton groups).
__global__ void short_write_kernel(const ShortList *__restrict__ S, uint32_t *__restrict__ sa,
                                   uint32_t *__restrict__ hd) {
    const uint32_t j = threadIdx.x;
    if (j >= S->n) return;
    sa[S->slot[j]] = S->pos[j];
    hd[S->slot[j]] = S->slot[j];
}

constexpr int kInitPer = 16;  // sorted keys per thread in init_groups_kernel
constexpr int kInitTile = 256 * kInitPer;

// Group heads after the key sort, in SA order (hd[i] = first SA index of
// i's group; equal heads == equal comparison so far); tied groups that need
// more symbols become the first round's work (engine.cuh step 3 -> 4).
// A block stages its 256 * kInitPer sorted keys (and their neighbours) in
// shared memory once, unpacks the positions when they ride below the keys,
// and appends its groups with one atomic per list (per-list counts packed
// as 16-bit fields, 4096 keys per block at most).  The key layout (the
// length field's kind, whether positions ride below the keys and whether
// they are segment-local) is fixed per instantiation.
template <int FLAG_LEN, bool UNPACK, bool SEG>
__global__ void __launch_bounds__(256)
    init_groups_kernel(const uint64_t *__restrict__ keys, uint32_t n, int k, uint64_t lmask,
                       int lf, int vshift, uint32_t *__restrict__ hd,
                       uint32_t *__restrict__ sa_out, GroupLists G,
                       const ShortList *__restrict__ S, int seg_at,
                       const uint64_t *__restrict__ seg_ends) {
    constexpr int flag_len = FLAG_LEN;
    static_assert(kLists <= 8, "two packed words of four 16-bit counters");
    __shared__ uint64_t sk[kInitTile + 2];  // sk[l + 1] = key of sorted index base + l
    __shared__ uint32_t s_base[kLists];
    const uint32_t base = blockIdx.x * (uint32_t)kInitTile;
    const uint32_t valid = n - base < (uint32_t)kInitTile ? n - base : (uint32_t)kInitTile;
    const uint64_t vmask = (1ull << vshift) - 1;
    // SA index of sorted record i: i + (short suffixes inserted at or before
    // it), one shift for the whole block unless an insertion falls inside
    __shared__ uint32_t s_shift[2];
    // short suffixes exist only in a flagless sort
    const uint32_t ns = (FLAG_LEN == 2 && S) ? __ldg(&S->n) : 0u;
    if (threadIdx.x == 0) {
        const uint32_t lo = ns ? short_shift(S, ns, base) : 0u;
        s_shift[0] = lo;
        s_shift[1] = !ns || short_shift(S, ns, base + valid - 1) == lo;
    }
    __syncthreads();
    const uint32_t sh_lo = s_shift[0];
    const bool sh_flat = s_shift[1] != 0;
    auto shift_of = [&](uint32_t i) { return sh_flat ? sh_lo : short_shift(S, ns, i); };
    // the bulk of the tiles: full, neither the first nor the last, one shift
    // for all records; they take loops without bounds, edge or shift checks
    const bool fast = base > 0 && base + (uint32_t)kInitTile < n && sh_flat;
    auto stage = [&](auto fast_c) {
        constexpr bool FAST = decltype(fast_c)::value;
#pragma unroll 4
        for (int j = 0; j < kInitPer; j++) {
            const uint32_t l = j * 256 + threadIdx.x;
            if (!FAST && l >= valid) break;
            const uint64_t item = keys[base + l];
            sk[l + 1] = item >> vshift;
            if (UNPACK) {
                // segment-local positions (seg_at > 0): the segment index
                // above the key gives the segment's first position
                uint64_t pos = item & vmask;
                if (SEG) {
                    const uint64_t sg = item >> seg_at;
                    pos += sg ? __ldg(seg_ends + sg - 1) : 0ull;
                }
                sa_out[base + l + (FAST ? sh_lo : shift_of(base + l))] = (uint32_t)pos;
            }
        }
    };
    if (fast)
        stage(std::true_type{});
    else
        stage(std::false_type{});
    if (threadIdx.x == 0) sk[0] = base > 0 ? keys[base - 1] >> vshift : 0ull;
    if (threadIdx.x == 32) sk[valid + 1] = base + valid < n ? keys[base + valid] >> vshift : 0ull;
    __syncthreads();
    // run heads of the tile as a bitmap (bit l of the tile: local l heads a
    // run), the last word at or before each word that holds a head, and the
    // head of a run that entered the tile from an earlier one: every member
    // then finds its head in O(1) however long its run is
    __shared__ uint32_t s_hb[kInitTile / 32];
    __shared__ int s_prev[kInitTile / 32];
    __shared__ uint32_t s_carry;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // pass 1: the heads bitmap; singletons (the bulk) are finished here, and
    // the records in groups are marked for pass 2 (bit j of m_grp: record j;
    // m_head / m_last: it heads / ends its group)
    uint32_t m_grp = 0, m_head = 0, m_last = 0;
    auto heads = [&](auto fast_c) {
        constexpr bool FAST = decltype(fast_c)::value;
#pragma unroll 4
        for (int j = 0; j < kInitPer; j++) {
            const uint32_t l = j * 256 + threadIdx.x;
            const bool in = FAST || l < valid;
            const uint32_t i = base + l;
            bool head = false, last = false;
            if (in) {
                const uint64_t key = sk[l + 1];
                head = (!FAST && i == 0) || sk[l] != key;
                last = (!FAST && i == n - 1) || sk[l + 2] != key;
            }
            const uint32_t word = __ballot_sync(0xffffffffu, in && head);
            if (lane == 0) s_hb[j * 8 + warp] = word;
            if (in) {
                if (head && last) {
                    // an insertion point only ever falls on a group head, so
                    // a group moves by one shift
                    const uint32_t sh = FAST ? sh_lo : shift_of(i);
                    hd[i + sh] = i + sh;
                } else {
                    m_grp |= 1u << j;
                    m_head |= (head ? 1u : 0u) << j;
                    m_last |= (last ? 1u : 0u) << j;
                }
            }
        }
    };
    if (fast)
        heads(std::true_type{});
    else
        heads(std::false_type{});
    __syncthreads();
    if (warp == 0) {
        static_assert(kInitTile / 32 == 128, "four bitmap words per lane");
        int lp[4], last = -1;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            if (s_hb[4 * lane + q]) last = 4 * lane + q;
            lp[q] = last;
        }
        int x = last;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x = max(x, y);
        }
        int before = __shfl_up_sync(0xffffffffu, x, 1);
        if (lane == 0) before = -1;
#pragma unroll
        for (int q = 0; q < 4; q++) s_prev[4 * lane + q] = max(lp[q], before);
        if (lane == 0)
            s_carry = (base > 0 && valid && sk[0] == sk[1]) ? run_head(keys, 0, base, sk[1], vshift)
                                                            : base;
    }
    __syncthreads();
    // tie state of a key: complete (equal through both ends: nothing to
    // refine), and the depth its group's members are known to agree on
    // (0 for the early-ended suffixes of a flagged plain text)
    auto state = [&](uint64_t key, bool &complete, uint64_t &depth) {
        const uint32_t lenf = (uint32_t)(key & lmask);
        if (flag_len == 2) {  // no length field: every record is a full suffix
            complete = false;
            depth = (uint64_t)k;
        } else if (flag_len) {
            complete = false;
            depth = lenf == (lf ? 0u : 1u) ? (uint64_t)k : 0ull;
        } else {
            const int take = lf ? k - (int)lenf : (int)lenf;
            complete = take < k;
            depth = (uint64_t)k;
        }
    };
    // first sorted index of the run that holds local index l
    auto head_of = [&](uint32_t l) -> uint32_t {
        const uint32_t w = l >> 5;
        const uint32_t x = s_hb[w] & (0xffffffffu >> (31 - (l & 31)));
        if (x) return base + w * 32 + 31 - __clz(x);
        const int w2 = w ? s_prev[w - 1] : -1;
        if (w2 >= 0) return base + (uint32_t)w2 * 32 + 31 - __clz(s_hb[w2]);
        return s_carry;
    };
    uint64_t cnt_lo = 0, cnt_hi = 0;  // 16-bit counts: lists 0..3, lists 4..
    uint32_t ends = 0;                 // bit j: key j ends a group that needs refining
    // only LongerFirst with a length field separates complete ties by position
    const bool lf_field = lf && !flag_len;
    // pass 2: the group members' heads, and the groups this thread ends
    auto pass1 = [&](auto fast_c) {
        constexpr bool FAST = decltype(fast_c)::value;
        for (uint32_t mg = m_grp; mg; mg &= mg - 1) {
            const int j = __ffs((int)mg) - 1;
            const uint32_t l = j * 256 + threadIdx.x;
            const uint32_t i = base + l;
            const uint64_t key = sk[l + 1];
            const bool head = (m_head >> j) & 1u, last = (m_last >> j) & 1u;
            const uint32_t sh = FAST ? sh_lo : shift_of(i);
            const uint32_t g = head ? i : head_of(l);
            bool complete = false;
            uint64_t depth = (uint64_t)k;
            if (lf_field || (last && !head)) state(key, complete, depth);
            hd[i + sh] = ((complete && lf) ? i : g) + sh;
            if (!complete && last && !head) {
                const int li = list_of(i - g + 1, depth);
                if (li == kLists) {
                    append_big(G, 0, g + sh, i - g + 1, depth);
                } else {
                    if (li < 4)
                        cnt_lo += 1ull << (16 * li);
                    else
                        cnt_hi += 1ull << (16 * (li - 4));
                    ends |= 1u << j;
                }
            }
        }
    };
    if (fast)
        pass1(std::true_type{});
    else
        pass1(std::false_type{});
    uint64_t off_lo, off_hi;
    const uint64_t tot_lo = block_excl_scan64(cnt_lo, &off_lo);
    const uint64_t tot_hi = block_excl_scan64(cnt_hi, &off_hi);
    if (threadIdx.x < kLists) {
        const int li = (int)threadIdx.x;
        const uint32_t total =
            (uint32_t)(((li < 4 ? tot_lo : tot_hi) >> (16 * (li & 3))) & 0xFFFFu);
        if (total) s_base[li] = atomicAdd(&G.ctr->n[li][0], total);
    }
    __syncthreads();
    // pass 3: write the entries of the groups found in pass 2
    for (; ends; ends &= ends - 1) {
        const int j = __ffs((int)ends) - 1;
        const uint32_t l = j * 256 + threadIdx.x;
        const uint32_t i = base + l;
        const uint64_t key = sk[l + 1];
        bool complete;
        uint64_t depth;
        state(key, complete, depth);
        const uint32_t g = head_of(l);
        const int li = list_of(i - g + 1, depth);
        uint32_t slot = 0;
#pragma unroll
        for (int q = 0; q < kLists; q++) {
            if (li == q) {
                uint64_t &off = q < 4 ? off_lo : off_hi;
                const int sh = 16 * (q & 3);
                slot = s_base[q] + (uint32_t)((off >> sh) & 0xFFFFu);
                off += 1ull << sh;
            }
        }
        uint4 entry = group_entry(g + shift_of(i), i - g + 1, depth);
        if (UNPACK && li == L_PAIR) {  // the positions ride along (see kPairPos)
            auto pos_of = [&](uint32_t r) -> uint32_t {
                const uint64_t item = keys[r];
                uint64_t pos = item & vmask;
                if (SEG) {
                    const uint64_t sg = item >> seg_at;
                    pos += sg ? __ldg(seg_ends + sg - 1) : 0ull;
                }
                return (uint32_t)pos;
            };
            entry = make_uint4(entry.x, pos_of(g), entry.z | kPairPos, pos_of(i));
        }
        list_ptr(G, li, 0)[slot] = entry;
    }
}

// Sort key of suffix p for a round at depth h: the rank of p + h, or the
// "ended" value when the suffix's limit is exactly reached.
__device__ __forceinline__ uint64_t doubling_key(const DevLimits &L,
                                                 const uint32_t *__restrict__ rank, uint32_t p,
                                                 uint64_t h, int lf, uint64_t empty_lf) {
    uint64_t lim = dev_lim_at(L, p);
    if (lim > h) {
        uint32_t r = __ldcg(rank + p + h);
        return lf ? (uint64_t)r : (uint64_t)r + 1;
    }
    return lf ? empty_lf : 0ull;
}

__global__ void gather_small_kernel(const uint4 *__restrict__ groups, uint32_t count,
                                    const uint32_t *__restrict__ sa,
                                    const uint32_t *__restrict__ rank, DevLimits L, uint64_t h,
                                    int lf, uint64_t empty_lf, uint64_t *__restrict__ key2) {
    for (uint32_t gi = blockIdx.x * blockDim.x + threadIdx.x; gi < count;
         gi += gridDim.x * blockDim.x) {
        uint4 g = groups[gi];
        const uint64_t d = g.z > h ? (uint64_t)g.z : h;  // the group's own depth if deeper
        for (uint32_t t = 0; t < g.y; t++) {
            uint32_t i = g.x + t;
            key2[i] = doubling_key(L, rank, sa[i], d, lf, empty_lf);
        }
    }
}

// Rank-doubling keys of the big groups' members, one thread per member
// (a single group can hold millions: runs of one symbol): member t belongs
// to the group whose flattened offset range holds it (groups' offsets grow
// with their ordinals).
// Runs of one symbol (ShorterFirst).  A tied group whose members all start
// with c^h (c repeated through the depth h) is a run group: its members are
// ordered at once by how their runs end instead of by doubling through the
// run (a run of length L would take log2(L / h) rounds, each re-sorting the
// whole group).  Member p with run length rr = min(run of c from p, lim):
//   * ends at rr (the suffix is c^rr): below every continuation of c^rr;
//   * continues with x != c at rr: c^rr x.. < c^rr' .. for rr < rr' when
//     x < c, and > when x > c;
// so the order is class A (x < c, or ended), ascending rr; then the members
// whose run reaches the key's cap; then class B (x > c), descending rr; and
// inside equal (class, rr) the rank of the suffix p + rr (0: ended).  Equal
// keys then agree on rr + h symbols (ranks are exact to the round depth h),
// the depth their subgroup is queued with; a group deeper than h is sorted
// by the rank at its own depth d, and its subgroups agree on d + h.
// runs_s: the inclusive max-scan of "last index of a run" over the reversed
// text, from which the run from p ends at n - 1 - runs_s[n - 1 - p].
struct RunKeys {
    const uint32_t *runs_s;  // null: no run keys this round
    Packed P;
    uint64_t n;
    int rbits;               // bits of the run-length field (cap 2^rbits - 1)
};

__device__ __forceinline__ uint32_t code_at(const Packed &P, uint64_t q) {
    const uint64_t bit = q * (uint64_t)P.b;
    const uint32_t sh = (uint32_t)(bit & 63);
    const uint64_t w0 = __ldg(P.w + (bit >> 6));
    const uint64_t w1 = __ldg(P.w + (bit >> 6) + 1);
    const uint64_t v = sh ? (w0 << sh) | (w1 >> (64 - sh)) : w0;
    return (uint32_t)(v >> (64 - P.b));
}

__device__ __forceinline__ uint64_t run_from(const RunKeys &R, uint64_t p) {
    return R.n - 1 - (uint64_t)__ldg(R.runs_s + (R.n - 1 - p)) - p + 1;
}

__global__ void gather_big_kernel(const BigGroup *__restrict__ groups, uint32_t nb,
                                  uint32_t total, const uint32_t *__restrict__ sa,
                                  const uint32_t *__restrict__ rank, DevLimits L, uint64_t h,
                                  int lf, uint64_t empty_lf, int k2bits, RunKeys R,
                                  uint64_t *__restrict__ tkeys, uint32_t *__restrict__ tvals) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += gridDim.x * blockDim.x) {
        uint32_t lo = 0, hi = nb;  // last group with toff <= t
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (groups[mid].toff <= t)
                lo = mid;
            else
                hi = mid;
        }
        const BigGroup g = groups[lo];
        const uint32_t p = sa[g.start + (t - g.toff)];
        // the group's own depth when it is known to be deeper than the round's
        const uint64_t d = g.depth > h ? (uint64_t)g.depth : h;
        uint64_t key;
        // a run group (see RunKeys); its members agree on d symbols only when
        // the group's own depth reaches the round's
        if (R.runs_s && g.depth >= h && run_from(R, sa[g.start]) >= d) {
            const uint64_t cap = (1ull << R.rbits) - 1;
            const uint64_t lim = dev_lim_at(L, p);
            const uint64_t rl = run_from(R, p);
            const uint64_t rr = rl < lim ? rl : lim;
            uint64_t cls, rq, k2;
            if (rr >= cap) {  // past the cap: between the two classes, by the
                cls = 0;      // doubling key at offset cap (lim >= rr >= cap)
                rq = cap;
                k2 = lim > cap ? (uint64_t)__ldcg(rank + p + cap) + 1 : 0ull;
            } else if (rr == lim) {  // ends inside the run
                cls = 0;
                rq = rr;
                k2 = 0;
            } else {
                const uint32_t c = code_at(R.P, p), x = code_at(R.P, p + rr);
                cls = x < c ? 0 : 1;
                rq = x < c ? rr : cap - 1 - rr;
                k2 = (uint64_t)__ldcg(rank + p + rr) + 1;
            }
            key = ((((((uint64_t)lo << 1) | cls) << R.rbits) | rq) << k2bits) | k2;
        } else {
            const uint64_t k2 = doubling_key(L, rank, p, d, lf, empty_lf);
            key = ((uint64_t)lo << (R.runs_s ? k2bits + 1 + R.rbits : k2bits)) | k2;
        }
        tkeys[t] = key;
        tvals[t] = p;
    }
}

// runs_s input: rev[r] = r where text position n - 1 - r ends a run of one
// symbol (the next symbol differs, or the text ends), else 0.
__global__ void run_ends_kernel(const void *__restrict__ text, int sym_bytes, uint64_t n,
                                uint32_t *__restrict__ rev) {
    for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < n;
         r += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t q = n - 1 - r;
        const bool end = q == n - 1 || sym_at(text, sym_bytes, q) != sym_at(text, sym_bytes, q + 1);
        rev[r] = end ? (uint32_t)r : 0u;
    }
}

// One thread sorts one small tied group by (key, position), writes the new
// SA slice, the new ranks and the still-tied subgroups.
__global__ void sort_small_kernel(const uint4 *__restrict__ groups, uint32_t count,
                                  uint32_t *__restrict__ sa, const uint64_t *__restrict__ key2,
                                  uint32_t *__restrict__ hd, uint32_t *__restrict__ rank, int lf,
                                  uint64_t empty, uint64_t h, GroupLists G, int nxt) {
    for (uint32_t gi = blockIdx.x * blockDim.x + threadIdx.x; gi < count;
         gi += gridDim.x * blockDim.x) {
        uint4 g = groups[gi];
        const uint64_t next_depth = (g.z > h ? (uint64_t)g.z : h) + h;
        uint64_t kk[kSmallMax];
        uint32_t pp[kSmallMax];
        for (uint32_t t = 0; t < g.y; t++) {
            uint64_t k2 = key2[g.x + t];
            uint32_t p = sa[g.x + t];
            int j = (int)t - 1;
            while (j >= 0 && (kk[j] > k2 || (kk[j] == k2 && pp[j] > p))) {
                kk[j + 1] = kk[j];
                pp[j + 1] = pp[j];
                j--;
            }
            kk[j + 1] = k2;
            pp[j + 1] = p;
        }
        uint32_t t = 0;
        while (t < g.y) {
            uint32_t e = t + 1;
            while (e < g.y && kk[e] == kk[t]) e++;
            bool ended = kk[t] == empty;
            for (uint32_t u = t; u < e; u++) {
                uint32_t r = (ended && lf) ? g.x + u : g.x + t;
                sa[g.x + u] = pp[u];
                hd[g.x + u] = r;
                rank[pp[u]] = r;
            }
            if (!ended && e - t >= 2) append_group(G, nxt, g.x + t, e - t, next_depth);
            t = e;
        }
    }
}

// ---------------------------------------------------------------- direct resolution

// Small tied groups are resolved by comparing the suffixes themselves, as
// the reference's merge does with LcpDispatch::lcp (src/lcp.rs:125-153),
// but on a bit-packed copy of the text: one 64-bit window holds 64/b
// symbols (32 for DNA), so a suffix pair that differs within ~100 symbols
// costs a few sector reads instead of several rank-doubling rounds.
// Sequential reader of b-bit symbols from the packed text: one 64-bit
// load per window after the first.
struct PackedStream {
    const uint64_t *w;
    uint64_t wi;
    uint32_t sh;
    uint64_t cur, nxt;
    __device__ __forceinline__ void init(const Packed &P, uint64_t p) {
        uint64_t s = p * (uint64_t)P.b;
        w = P.w;
        wi = s >> 6;
        sh = (uint32_t)(s & 63);
        cur = __ldg(w + wi);
        nxt = __ldg(w + wi + 1);
    }
    __device__ __forceinline__ uint64_t get(uint64_t mask) const {
        return (sh ? (cur << sh) | (nxt >> (64 - sh)) : cur) & mask;
    }
    __device__ __forceinline__ void advance(uint32_t bits) {
        sh += bits;
        if (sh >= 64) {
            sh -= 64;
            wi++;
            cur = nxt;
            nxt = __ldg(w + wi + 1);
        }
    }
};

// A[q] for a runtime q < N without spilling the array to local memory.
template <int N>
__device__ __forceinline__ uint64_t pickn(const uint64_t (&A)[N], int q) {
    uint64_t v = A[0];
#pragma unroll
    for (int i = 1; i < N; i++) v = q == i ? A[i] : v;
    return v;
}

// Order of suffixes a and b, known to agree on their first `o` symbols:
// -1 / 1, 0 for a complete tie (ShorterFirst, equal limits), 2 when they
// still agree `cap` symbols further (undecided).  Mirrors suffix_cmp_with
// (src/lcp.rs:184-201) from offset o.
template <int kBurst = 4>
__device__ __forceinline__ int direct_cmp(const Packed &P, uint64_t a, uint64_t la, uint64_t b,
                                          uint64_t lb, uint64_t o, uint64_t cap, int lf) {
    const uint64_t lim = la < lb ? la : lb;
    const uint64_t end = lim < o + cap ? lim : o + cap;
    // the first kBurst windows of both suffixes are fetched with independent
    // loads (one round trip covers the common short-LCP case), later ones
    // stream one word per window
    uint64_t t = o;
    if (t < end) {
        uint64_t sa0 = (a + t) * (uint64_t)P.b, sb0 = (b + t) * (uint64_t)P.b;
        const uint64_t *wa = P.w + (sa0 >> 6), *wb = P.w + (sb0 >> 6);
        const uint32_t sha = (uint32_t)(sa0 & 63), shb = (uint32_t)(sb0 & 63);
        // words spanned by four windows: at most 5 (a window is <= 64 bits)
        uint64_t A[kBurst + 1], B[kBurst + 1];
        const uint32_t wbits = (uint32_t)(P.spw * P.b);
        const int nwa = (int)((sha + (kBurst - 1) * wbits) >> 6) + 2;
        const int nwb = (int)((shb + (kBurst - 1) * wbits) >> 6) + 2;
#pragma unroll
        for (int q = 0; q < kBurst + 1; q++) {
            A[q] = q < nwa ? __ldg(wa + q) : 0ull;
            B[q] = q < nwb ? __ldg(wb + q) : 0ull;
        }
        if (wbits == 64) {
            // whole-word windows (b divides 64, e.g. DNA): window s starts in
            // word s of both bursts, no runtime word selection
#pragma unroll
            for (int s = 0; s < kBurst; s++) {
                if (t >= end) break;
                const uint64_t va = sha ? (A[s] << sha) | (A[s + 1] >> (64 - sha)) : A[s];
                const uint64_t vb = shb ? (B[s] << shb) | (B[s + 1] >> (64 - shb)) : B[s];
                const uint64_t x = va ^ vb;
                if (x) {
                    const uint64_t d = (uint64_t)__clzll((long long)x) / (uint64_t)P.b;
                    if (t + d < end) return va < vb ? -1 : 1;
                    t = end;
                    break;
                }
                t += (uint64_t)P.spw;
            }
        } else {
        uint32_t bit_a = sha, bit_b = shb;
#pragma unroll
        for (int s = 0; s < kBurst; s++) {
            if (t >= end) break;
            int qa = (int)(bit_a >> 6), qb = (int)(bit_b >> 6);
            uint32_t ra = bit_a & 63, rb = bit_b & 63;
            uint64_t a0 = pickn(A, qa), a1 = pickn(A, qa + 1);
            uint64_t b0 = pickn(B, qb), b1 = pickn(B, qb + 1);
            uint64_t va = (ra ? (a0 << ra) | (a1 >> (64 - ra)) : a0) & P.mask;
            uint64_t vb = (rb ? (b0 << rb) | (b1 >> (64 - rb)) : b0) & P.mask;
            uint64_t x = va ^ vb;
            if (x) {
                uint64_t d = (uint64_t)__clzll((long long)x) / (uint64_t)P.b;
                if (t + d < end) return va < vb ? -1 : 1;
                t = end;
                break;
            }
            bit_a += (uint32_t)(P.spw * P.b);
            bit_b += (uint32_t)(P.spw * P.b);
            t += (uint64_t)P.spw;
        }
        }
    }
    if (t < end) {
        PackedStream sa_, sb_;
        sa_.init(P, a + t);
        sb_.init(P, b + t);
        const uint32_t step_bits = (uint32_t)(P.spw * P.b);
        for (; t < end; t += (uint64_t)P.spw) {
            uint64_t va = sa_.get(P.mask), vb = sb_.get(P.mask);
            uint64_t x = va ^ vb;
            if (x) {
                uint64_t d = (uint64_t)__clzll((long long)x) / (uint64_t)P.b;
                if (t + d < end) return va < vb ? -1 : 1;
                break;
            }
            sa_.advance(step_bits);
            sb_.advance(step_bits);
        }
    }
    if (end < lim) return 2;
    if (!lf) return (la > lb) - (la < lb);
    if (la != lb) return (lb > la) - (lb < la);
    return (a > b) - (a < b);
}

template <typename S>
__global__ void pack_text_kernel(const S *__restrict__ text, uint64_t n, Coder<S> coder, int b,
                                 uint64_t *__restrict__ words, uint64_t nwords) {
    for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < nwords;
         w += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t bit0 = w * 64;
        uint64_t i0 = bit0 / (uint64_t)b, i1 = (bit0 + 63) / (uint64_t)b;
        uint64_t v = 0;
        for (uint64_t i = i0; i <= i1; i++) {
            if (i >= n) break;
            uint64_t c = coder(text[i]);
            int64_t off = (int64_t)(i * (uint64_t)b) - (int64_t)bit0;
            int64_t shift = 64 - off - b;
            if (shift >= 0)
                v |= shift < 64 ? (c << shift) : 0ull;
            else
                v |= c >> (-shift);
        }
        words[w] = v;
    }
}

// pack_text_kernel for u8 text (16-byte aligned) whose code width b divides
// 64: word w holds exactly the 64 / b symbols from w * 64 / b, read with
// vector loads and coded through a shared copy of the code table.
__global__ void __launch_bounds__(256)
    pack_u8_kernel(const uint8_t *__restrict__ text, uint64_t n, const uint16_t *__restrict__ table,
                   int b, uint64_t *__restrict__ words, uint64_t nwords) {
    __shared__ uint16_t stab[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) stab[i] = table[i];
    __syncthreads();
    const int spw = 64 / b;  // 64, 32, 16 or 8 symbols
    for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < nwords;
         w += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t s0 = w * (uint64_t)spw;
        uint64_t v = 0;
        for (int q = 0; q < spw; q += 16) {
            const int cnt = spw < 16 ? spw : 16;
            const uint64_t p = s0 + q;
            uint32_t wv[4] = {0, 0, 0, 0};
            if (p + cnt <= n) {
                if (cnt == 16) {
                    const uint4 x = *reinterpret_cast<const uint4 *>(text + p);
                    wv[0] = x.x; wv[1] = x.y; wv[2] = x.z; wv[3] = x.w;
                } else {
                    const uint2 x = *reinterpret_cast<const uint2 *>(text + p);
                    wv[0] = x.x; wv[1] = x.y;
                }
            } else {
                for (int e = 0; e < cnt && p + e < n; e++)
                    wv[e >> 2] |= (uint32_t)text[p + e] << (8 * (e & 3));
            }
#pragma unroll
            for (int e = 0; e < 16; e++) {
                if (e < cnt) {
                    const uint32_t c =
                        p + e < n ? (uint32_t)stab[(wv[e >> 2] >> (8 * (e & 3))) & 255u] : 0u;
                    v = (v << b) | c;
                }
            }
        }
        words[w] = v;
    }
}

// Two-member tied groups (the bulk of the work on repeat-rich text): one
// thread compares the pair directly past their shared depth g.z, writes
// the SA slice and heads (and ranks once they exist), and passes a pair
// still undecided after max(g.z, kDirectCap) more symbols to the next
// round with that larger depth.
__global__ void __launch_bounds__(256, 5)
    direct_pair_kernel(const uint4 *__restrict__ groups, uint32_t count, uint32_t *__restrict__ sa,
                       uint32_t *__restrict__ hd, uint32_t *__restrict__ rank, DevLimits L,
                       Packed P, int lf, GroupLists G, int nxt) {
    const uint32_t gi = blockIdx.x * blockDim.x + threadIdx.x;
    bool again = false;
    uint4 g = make_uint4(0, 0, 0, 0);
    uint64_t cap = 0;
    uint64_t o = 0;
    if (gi < count) {
        g = groups[gi];
        const bool carried = (g.z & kPairPos) != 0;  // positions in the entry
        o = g.z & ~kPairPos;
        cap = o > kDirectCap ? o : kDirectCap;
        uint32_t p0 = carried ? g.y : sa[g.x], p1 = carried ? g.w : sa[g.x + 1];
        uint64_t l0 = dev_lim_at(L, p0), l1 = dev_lim_at(L, p1);
        int r = direct_cmp<kPairBurst>(P, p0, l0, p1, l1, o, cap, lf);
        if (r == 1 || ((r == 0 || r == 2) && p0 > p1)) {
            uint32_t t = p0;
            p0 = p1;
            p1 = t;
            if (r == 1) r = -1;
        }
        sa[g.x] = p0;
        sa[g.x + 1] = p1;
        uint32_t h1 = (r == -1) ? g.x + 1 : g.x;
        hd[g.x] = g.x;
        hd[g.x + 1] = h1;
        if (rank) {
            rank[p0] = g.x;
            rank[p1] = h1;
        }
        again = r == 2;
    }
    block_append(G, nxt, again, g.x, 2, o + cap);
}

// Four consecutive windows of the packed text from symbol p (five word
// loads, all independent).
__device__ __forceinline__ void windows4_at(const Packed &P, uint64_t p, uint64_t (&w)[4]) {
    const uint64_t s = p * (uint64_t)P.b;
    const uint64_t *q = P.w + (s >> 6);
    const uint32_t sh = (uint32_t)(s & 63);
    uint64_t x[5];
#pragma unroll
    for (int i = 0; i < 5; i++) x[i] = __ldg(q + i);
    const uint32_t wbits = (uint32_t)(P.spw * P.b);
    if (wbits == 64) {  // b divides 64 (DNA): window i starts in word i
#pragma unroll
        for (int i = 0; i < 4; i++) w[i] = sh ? (x[i] << sh) | (x[i + 1] >> (64 - sh)) : x[i];
        return;
    }
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const uint32_t bit = sh + i * wbits;  // < 256
        const int wi = (int)(bit >> 6);
        const uint32_t r = bit & 63;
        const uint64_t a0 = pickn(x, wi), a1 = pickn(x, wi + 1);
        w[i] = (r ? (a0 << r) | (a1 >> (64 - r)) : a0) & P.mask;
    }
}

template <int N>
__device__ __forceinline__ uint32_t pick32(const uint32_t (&A)[N], int q) {
    uint32_t v = A[0];
#pragma unroll
    for (int i = 1; i < N; i++) v = q == i ? A[i] : v;
    return v;
}

// Tied groups of 3..4 members: one thread per group, in rounds of four
// windows (128 DNA symbols): a round loads the next four windows of
// every member with independent loads (one round trip for the group) and
// settles every still-undecided member pair that differs in them.  Near a
// member's end (rare: the last symbols of a text or segment) the remaining
// pairs are settled one by one by direct_cmp.  A member's place is the
// count of members before it, so nothing moves until the final scatter;
// counts (4 bits per member) and pair relations (2 bits per pair) live in
// packed registers.
template <int M>
__global__ void __launch_bounds__(128)
    direct_tiny_kernel(const uint4 *__restrict__ groups, uint32_t count,
                       uint32_t *__restrict__ sa, uint32_t *__restrict__ hd,
                       uint32_t *__restrict__ rank, DevLimits L, Packed P, int lf, GroupLists G,
                       int nxt) {
    for (uint32_t gi = blockIdx.x * blockDim.x + threadIdx.x; gi < count;
         gi += gridDim.x * blockDim.x) {
        const uint4 g = groups[gi];
        const int len = (int)g.y;
        const uint64_t o = g.z;
        const uint64_t cap = o > kDirectCap ? o : kDirectCap;
        uint32_t pp[M], lm[M];
        uint64_t minend = o + cap;  // no comparison of the group looks past this
#pragma unroll
        for (int t = 0; t < M; t++) {
            if (t < len) {
                pp[t] = sa[g.x + t];
                lm[t] = (uint32_t)dev_lim_at(L, pp[t]);
                minend = lm[t] < minend ? lm[t] : minend;
            }
        }
        uint64_t und64 = 0;  // bit (i * M + j), i < j: pair not settled yet
#pragma unroll
        for (int i = 0; i < M; i++)
#pragma unroll
            for (int j = i + 1; j < M; j++)
                if (j < len) und64 |= 1ull << (i * M + j);
        uint32_t bef = 0;            // 4 bits per member: members placed before it
        uint64_t tie = 0, undc = 0;  // bit (i * M + j): complete tie / undecided at the cap
        const uint64_t span = 4 * (uint64_t)P.spw;
        uint64_t base = o;
        while (und64) {
            if (base + span <= minend) {
                uint64_t w[M][4];
#pragma unroll
                for (int t = 0; t < M; t++)
                    if (t < len) windows4_at(P, (uint64_t)pp[t] + base, w[t]);
#pragma unroll
                for (int i = 0; i < M; i++)
#pragma unroll
                    for (int j = i + 1; j < M; j++) {
                        const uint64_t bit = 1ull << (i * M + j);
                        if (j < len && (und64 & bit)) {
                            int r = 0;
#pragma unroll
                            for (int q = 3; q >= 0; q--)
                                r = w[i][q] != w[j][q] ? (w[i][q] < w[j][q] ? -1 : 1) : r;
                            if (r) {
                                bef += r < 0 ? (1u << (4 * j)) : (1u << (4 * i));
                                und64 &= ~bit;
                            }
                        }
                    }
                base += span;
            } else {
                // a member's end or the horizon is within reach: the rest
                // pair by pair (direct_cmp settles a pair at its end too)
                for (uint64_t m = und64; m; m &= m - 1) {
                    const int pi = __ffsll((long long)m) - 1;
                    const int i = pi / M, j = pi % M;
                    const uint32_t a = pick32(pp, i), b = pick32(pp, j);
                    const uint32_t la = pick32(lm, i), lb = pick32(lm, j);
                    const uint64_t done = base - o;  // symbols known equal past o
                    const int r = direct_cmp(P, a, la, b, lb, base, cap - done, lf);
                    const bool i_first = r == -1 || ((r == 0 || r == 2) && a < b);
                    bef += i_first ? (1u << (4 * j)) : (1u << (4 * i));
                    if (r == 0) tie |= 1ull << pi;
                    if (r == 2) undc |= 1ull << pi;
                }
                und64 = 0;
            }
        }
        // slot of each member, relation of each slot to the one before it
        uint32_t starts = 1u;  // bit s: slot s begins a tie run
        uint32_t undec = 0u;   // bit s: slot s is undecided against slot s-1
#pragma unroll
        for (int t = 0; t < M; t++) {
            if (t < len) {
                const uint32_t st = (bef >> (4 * t)) & 15u;
                bool tied = false, open = false;
#pragma unroll
                for (int u = 0; u < M; u++) {
                    if (u < len && u != t && ((bef >> (4 * u)) & 15u) + 1u == st) {
                        const int pi = u < t ? u * M + t : t * M + u;
                        tied = (tie >> pi) & 1ull;
                        open = (undc >> pi) & 1ull;
                    }
                }
                if (st > 0 && !tied && !open) starts |= 1u << st;
                if (st > 0 && open) undec |= 1u << st;
            }
        }
#pragma unroll
        for (int t = 0; t < M; t++) {
            if (t < len) {
                const uint32_t st = (bef >> (4 * t)) & 15u;
                const uint32_t head = 31u - (uint32_t)__clz((int)(starts & ((2u << st) - 1u)));
                sa[g.x + st] = pp[t];
                hd[g.x + st] = g.x + head;
                if (rank) rank[pp[t]] = g.x + head;
            }
        }
        // runs still undecided go to the next round, past this round's cap
#pragma unroll
        for (int s2 = 1; s2 < M; s2++) {
            if (s2 < len) {
                const bool run_end = s2 == len - 1 || ((starts >> (s2 + 1)) & 1u);
                const uint32_t head = 31u - (uint32_t)__clz((int)(starts & ((2u << s2) - 1u)));
                if (run_end && head < (uint32_t)s2 && ((undec >> s2) & 1u))
                    append_group(G, nxt, g.x + head, (uint32_t)s2 - head + 1, o + cap);
            }
        }
    }
}

// Tied groups of 5..kTinyMax members: S lanes per group (32/S groups per
// warp), one member per lane, in rounds of four windows: every lane loads
// the next four windows of its member (one round trip for the group),
// exchanges them with its group by shuffles and settles its undecided
// relations that differ in them.  Near a member's end or the horizon the
// rest is settled by direct_cmp, the other member's position and limit
// taken by shuffles in a loop every lane runs (no per-member arrays).  A
// member's place is the count of members before it.
template <int S>
__global__ void __launch_bounds__(128)
    direct_tiny_seg_kernel(const uint4 *__restrict__ groups, uint32_t count,
                           uint32_t *__restrict__ sa, uint32_t *__restrict__ hd,
                           uint32_t *__restrict__ rank, DevLimits L, Packed P, int lf,
                           GroupLists G, int nxt) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t sl = lane & (S - 1), sb = lane & ~(uint32_t)(S - 1);
    const uint64_t gi = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) / S;
    const uint4 g = gi < count ? groups[gi] : make_uint4(0, 0, 0, 0);
    const int len = (int)g.y;
    const bool mine = (int)sl < len;
    const uint64_t o = g.z;
    const uint64_t cap = o > kDirectCap ? o : kDirectCap;
    const uint64_t horizon = o + cap;
    const uint32_t my_p = mine ? sa[g.x + sl] : 0u;
    const uint32_t my_lim = mine ? (uint32_t)dev_lim_at(L, my_p) : 0xFFFFFFFFu;
    uint32_t lmin = my_lim;
#pragma unroll
    for (int x = 1; x < S; x <<= 1) lmin = min(lmin, __shfl_xor_sync(0xffffffffu, lmin, x));
    const uint64_t minend = lmin < horizon ? lmin : horizon;
    // bit u: relation with member u not settled yet
    uint32_t und = mine ? ((1u << len) - 1u) & ~(1u << sl) : 0u;
    uint32_t before = 0, tie = 0, undc = 0;  // tie / undc: bit u, relation with u
    const uint64_t span = 4 * (uint64_t)P.spw;
    uint64_t base = o;
    while (__any_sync(0xffffffffu, und != 0)) {
        const bool fast = base + span <= minend;
        const bool seg_busy = (__ballot_sync(0xffffffffu, und != 0) >> sb) & ((1u << S) - 1u);
        uint64_t w[4] = {0, 0, 0, 0};
        if (mine && fast && seg_busy) windows4_at(P, (uint64_t)my_p + base, w);
#pragma unroll
        for (int u = 0; u < S; u++) {
            int r = 0;
#pragma unroll
            for (int q = 3; q >= 0; q--) {
                const uint64_t wu = __shfl_sync(0xffffffffu, w[q], sb + u);
                r = w[q] != wu ? (w[q] < wu ? -1 : 1) : r;
            }
            if (fast && ((und >> u) & 1u) && r) {
                before += r > 0 ? 1u : 0u;
                und &= ~(1u << u);
            }
        }
        if (__any_sync(0xffffffffu, !fast && und != 0)) {
#pragma unroll 1
            for (int u = 0; u < S; u++) {
                const uint32_t b = __shfl_sync(0xffffffffu, my_p, sb + u);
                const uint32_t lb = __shfl_sync(0xffffffffu, my_lim, sb + u);
                if (!fast && ((und >> u) & 1u)) {
                    const int r = direct_cmp(P, my_p, my_lim, b, lb, base, horizon - base, lf);
                    const bool me_first = r == -1 || ((r == 0 || r == 2) && my_p < b);
                    before += me_first ? 0u : 1u;
                    if (r == 0) tie |= 1u << u;
                    if (r == 2) undc |= 1u << u;
                }
            }
        }
        if (fast)
            base += span;
        else
            und = 0;
    }
    // sorted slot, relation to the slot before, tie-run heads
    const uint32_t slot = before;
    bool ptie = false, popen = false;
#pragma unroll
    for (int u = 0; u < S; u++) {
        const uint32_t su = __shfl_sync(0xffffffffu, slot, sb + u);
        if (mine && u != (int)sl && u < len && su + 1 == slot) {
            ptie = (tie >> u) & 1u;
            popen = (undc >> u) & 1u;
        }
    }
    uint32_t starts = (mine && (slot == 0 || (!ptie && !popen))) ? (1u << slot) : 0u;
    uint32_t undec = (mine && slot > 0 && popen) ? (1u << slot) : 0u;
#pragma unroll
    for (int x = 1; x < S; x <<= 1) {
        starts |= __shfl_xor_sync(0xffffffffu, starts, x);
        undec |= __shfl_xor_sync(0xffffffffu, undec, x);
    }
    if (mine) {
        const uint32_t head = 31u - (uint32_t)__clz((int)(starts & ((2u << slot) - 1u)));
        sa[g.x + slot] = my_p;
        hd[g.x + slot] = g.x + head;
        if (rank) rank[my_p] = g.x + head;
        const bool run_end = (int)slot == len - 1 || ((starts >> (slot + 1)) & 1u);
        if (run_end && head < slot && ((undec >> slot) & 1u))
            append_group(G, nxt, g.x + head, slot - head + 1, o + cap);
    }
}

// Tied groups of 9..32 members: one warp per group, one lane per member, in
// rounds of four windows like direct_tiny_seg_kernel: every lane whose
// member is still undecided loads its next four windows (one round trip
// for the group) and compares them with every other member's through
// shuffles, settling the relations that differ in them (relations settle
// in both lanes at once, so a settled member's windows are not needed
// again).  Near a member's end or the horizon the rest is settled by
// direct_cmp (ties by position).  A member's place is the count of members
// before it, so the relation to its sorted predecessor is already known.
// Groups deeper than kDirectMaxH are left to rank doubling.
__global__ void direct_warp_kernel(const uint4 *__restrict__ groups, uint32_t count,
                                   uint32_t *__restrict__ sa, uint32_t *__restrict__ hd,
                                   uint32_t *__restrict__ rank, DevLimits L, Packed P, int lf,
                                   GroupLists G, int nxt) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const uint64_t span = 4 * (uint64_t)P.spw;
    for (uint64_t gi = warp; gi < count; gi += nwarps) {
        const uint4 g = groups[gi];
        const uint32_t len = g.y;
        const uint64_t o = g.z;
        const uint64_t cap = o > kDirectCap ? o : kDirectCap;
        const uint64_t horizon = o + cap;
        const bool mine = lane < len;
        const uint32_t my_p = mine ? sa[g.x + lane] : 0u;
        const uint32_t my_l = mine ? (uint32_t)dev_lim_at(L, my_p) : 0xFFFFFFFFu;
        const uint32_t lmin = __reduce_min_sync(0xffffffffu, my_l);
        const uint64_t minend = lmin < horizon ? lmin : horizon;
        const uint32_t members = len >= 32 ? 0xFFFFFFFFu : (1u << len) - 1u;
        uint32_t und = mine ? members & ~(1u << lane) : 0u;  // bit u: not settled with u
        uint32_t before = 0, tie = 0, undc = 0;  // tie / undc: bit u, relation with u
        uint64_t base = o;
        while (__any_sync(0xffffffffu, und != 0)) {
            if (base + span <= minend) {
                uint64_t w[4] = {0, 0, 0, 0};
                if (und) windows4_at(P, (uint64_t)my_p + base, w);
                for (uint32_t u = 0; u < len; u++) {
                    int r = 0;
#pragma unroll
                    for (int q = 3; q >= 0; q--) {
                        const uint64_t wu = __shfl_sync(0xffffffffu, w[q], u);
                        r = w[q] != wu ? (w[q] < wu ? -1 : 1) : r;
                    }
                    if (((und >> u) & 1u) && r) {
                        before += r > 0 ? 1u : 0u;
                        und &= ~(1u << u);
                    }
                }
                base += span;
            } else {
                for (uint32_t u = 0; u < len; u++) {
                    const uint32_t b = __shfl_sync(0xffffffffu, my_p, u);
                    const uint32_t lb = __shfl_sync(0xffffffffu, my_l, u);
                    if ((und >> u) & 1u) {
                        const int r = direct_cmp(P, my_p, my_l, b, lb, base, horizon - base, lf);
                        const bool me_first = r == -1 || ((r == 0 || r == 2) && my_p < b);
                        before += me_first ? 0u : 1u;
                        if (r == 0) tie |= 1u << u;
                        if (r == 2) undc |= 1u << u;
                    }
                }
                und = 0;
            }
        }
        // sorted slot, relation to the slot before, tie-run heads
        const uint32_t slot = before;
        bool ptie = false, popen = false;
        for (uint32_t u = 0; u < len; u++) {
            const uint32_t su = __shfl_sync(0xffffffffu, slot, u);
            if (mine && u != lane && su + 1 == slot) {
                ptie = (tie >> u) & 1u;
                popen = (undc >> u) & 1u;
            }
        }
        const uint32_t starts = __reduce_or_sync(
            0xffffffffu, (mine && (slot == 0 || (!ptie && !popen))) ? (1u << slot) : 0u);
        const uint32_t undec =
            __reduce_or_sync(0xffffffffu, (mine && slot > 0 && popen) ? (1u << slot) : 0u);
        if (mine) {
            const uint32_t head = 31u - (uint32_t)__clz((int)(starts & ((2u << slot) - 1u)));
            sa[g.x + slot] = my_p;
            hd[g.x + slot] = g.x + head;
            if (rank) rank[my_p] = g.x + head;
            // slot == 31 only when len == 32, so the shift below stays < 32
            const bool run_end = slot + 1 == len || ((starts >> (slot + 1)) & 1u);
            if (run_end && head < slot && ((undec >> slot) & 1u))
                append_group(G, nxt, g.x + head, slot - head + 1, o + cap);
        }
    }
}

// One block sorts one medium tied group (17..kMediumMax members, all
// agreeing on h symbols) with a bitonic network over direct comparisons,
// then splits it into subgroups like direct_warp_kernel.
constexpr int kMedThreads = 256;

__global__ void __launch_bounds__(kMedThreads)
    direct_medium_kernel(const uint4 *__restrict__ groups, uint32_t count,
                         uint32_t *__restrict__ sa, uint32_t *__restrict__ hd,
                         uint32_t *__restrict__ rank, DevLimits L, Packed P, int lf,
                         GroupLists G, int nxt) {
    __shared__ uint32_t spos[kMediumMax];
    __shared__ uint64_t slim[kMediumMax];
    __shared__ int8_t rel[kMediumMax];
    __shared__ uint32_t shead[kMediumMax];
    __shared__ uint32_t wmax[kMedThreads / 32];
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (uint32_t gi = blockIdx.x; gi < count; gi += gridDim.x) {
        const uint4 g = groups[gi];
        const uint32_t len = g.y;
        const uint64_t h = g.z;
        const uint64_t cap = h > kDirectCap ? h : kDirectCap;
        uint32_t p2 = 1;
        while (p2 < len) p2 <<= 1;
        for (uint32_t t = tid; t < p2; t += kMedThreads) {
            if (t < len) {
                uint32_t p = sa[g.x + t];
                spos[t] = p;
                slim[t] = dev_lim_at(L, p);
            } else {
                spos[t] = 0xFFFFFFFFu;  // padding sorts last
                slim[t] = 0;
            }
        }
        __syncthreads();
        for (uint32_t kk = 2; kk <= p2; kk <<= 1) {
            for (uint32_t j = kk >> 1; j > 0; j >>= 1) {
                for (uint32_t i = tid; i < p2; i += kMedThreads) {
                    uint32_t ixj = i ^ j;
                    if (ixj <= i) continue;
                    uint32_t pa = spos[i], pb = spos[ixj];
                    bool a_after;
                    if (pa == 0xFFFFFFFFu || pb == 0xFFFFFFFFu) {
                        a_after = pa == 0xFFFFFFFFu && pb != 0xFFFFFFFFu;
                    } else {
                        int r = direct_cmp(P, pa, slim[i], pb, slim[ixj], h, cap, lf);
                        a_after = r == 1 || ((r == 0 || r == 2) && pa > pb);
                    }
                    bool up = (i & kk) == 0;
                    if (up == a_after) {
                        spos[i] = pb;
                        spos[ixj] = pa;
                        uint64_t tl = slim[i];
                        slim[i] = slim[ixj];
                        slim[ixj] = tl;
                    }
                }
                __syncthreads();
            }
        }
        // relation of each member to its predecessor: -1 starts a subgroup
        for (uint32_t t = tid; t < len; t += kMedThreads) {
            int r = -1;
            if (t > 0) {
                r = direct_cmp(P, spos[t - 1], slim[t - 1], spos[t], slim[t], h, cap, lf);
                if (r != 0 && r != 2) r = -1;
            }
            rel[t] = (int8_t)r;
        }
        __syncthreads();
        // subgroup head of every member: block max-scan of (start ? t : 0)
        constexpr uint32_t kPer = kMediumMax / kMedThreads;
        uint32_t base = tid * kPer, run = 0;
        uint32_t loc[kPer];
#pragma unroll
        for (uint32_t q = 0; q < kPer; q++) {
            uint32_t t = base + q;
            if (t < len && rel[t] == -1) run = t;
            loc[q] = run;
        }
        uint32_t x = run;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if ((int)lane >= o) x = max(x, y);
        }
        if (lane == 31) wmax[warp] = x;
        __syncthreads();
        uint32_t carry = 0;
        for (uint32_t w = 0; w < warp; w++) carry = max(carry, wmax[w]);
        uint32_t prev = __shfl_up_sync(0xffffffffu, x, 1);
        if (lane == 0) prev = 0;
        carry = max(carry, prev);
#pragma unroll
        for (uint32_t q = 0; q < kPer; q++) {
            uint32_t t = base + q;
            if (t < len) shead[t] = max(carry, loc[q]);
        }
        __syncthreads();
        for (uint32_t t = tid; t < len; t += kMedThreads) {
            uint32_t head = shead[t];
            sa[g.x + t] = spos[t];
            hd[g.x + t] = g.x + head;
            if (rank) rank[spos[t]] = g.x + head;
            bool last = t + 1 == len || rel[t + 1] == -1;
            if (last && t > head && rel[t] == 2)
                append_group(G, nxt, g.x + head, t - head + 1, h + cap);
        }
        __syncthreads();
    }
}

// After the big groups' (ordinal, key) pairs are sorted: scatter back into
// the SA, re-rank, and emit the still-tied subgroups.
__global__ void split_big_kernel(const uint64_t *__restrict__ tkeys,
                                 const uint32_t *__restrict__ tvals, uint32_t total,
                                 const BigGroup *__restrict__ groups, uint32_t n_groups,
                                 int k2bits, int ord_shift, RunKeys R,
                                 uint32_t *__restrict__ sa, uint32_t *__restrict__ hd,
                                 uint32_t *__restrict__ rank, int lf,
                                 uint64_t empty, uint64_t h, GroupLists G, int nxt) {
    const uint64_t k2mask = (k2bits >= 64) ? ~0ull : ((1ull << k2bits) - 1);
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += gridDim.x * blockDim.x) {
        uint64_t key = tkeys[t];
        uint32_t ord = (uint32_t)(key >> ord_shift);
        if (ord >= n_groups) continue;  // unreachable unless a sort step failed (flagged)
        BigGroup g = groups[ord];
        uint32_t local = t - g.toff;
        if (t < g.toff || local >= g.len) continue;
        uint32_t p = tvals[t];
        sa[g.start + local] = p;
        bool head = (t == g.toff) || tkeys[t - 1] != key;
        uint32_t h0 = head ? t : run_head(tkeys, g.toff, t, key);
        bool ended = (key & k2mask) == empty;
        uint32_t r = (ended && lf) ? g.start + local : g.start + (h0 - g.toff);
        hd[g.start + local] = r;
        rank[p] = r;
        bool last = (t == g.toff + g.len - 1) || tkeys[t + 1] != key;
        if (!ended && last && t > h0) {
            // the depth the subgroup's members now agree on (see RunKeys)
            const uint64_t d = g.depth > h ? (uint64_t)g.depth : h;
            uint64_t next_depth = d + h;
            if (R.runs_s && g.depth >= h && run_from(R, tvals[g.toff]) >= d) {
                const uint64_t cap = (1ull << R.rbits) - 1;
                const uint64_t rq = (key >> k2bits) & cap;
                const bool cls_b = (key >> (k2bits + R.rbits)) & 1ull;
                next_depth = (cls_b ? cap - 1 - rq : rq) + h;
            }
            append_group(G, nxt, g.start + (h0 - g.toff), t - h0 + 1, next_depth);
        }
    }
}

// ---------------------------------------------------------------- output

template <typename IT>
__global__ void widen_kernel(const uint32_t *__restrict__ in, IT *__restrict__ out, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = (IT)in[i];
}

// Subset output: key = (rank of the suffix, position).  Position n is the
// empty suffix: first under ShorterFirst, last under LongerFirst.
template <typename PT>
__global__ void subset_key_kernel(const PT *__restrict__ pos, uint64_t m, uint64_t n,
                                  const uint32_t *__restrict__ rank, int lf,
                                  uint64_t *__restrict__ keys, uint32_t *__restrict__ vals,
                                  int *__restrict__ bad) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t p = (uint64_t)pos[i];
        uint64_t rk;
        if (p > n) {
            atomicExch(bad, 1);
            p = n;
        }
        if (p == n)
            rk = lf ? 0xFFFFFFFFull : 0ull;
        else
            rk = (uint64_t)__ldg(rank + p) + 1;
        keys[i] = (rk << 32) | p;
        vals[i] = (uint32_t)p;
    }
}

}  // namespace eng


namespace eng {

// ---------------------------------------------------------------- bounded context

// Bounded max_context: the sort above uses the unbounded comparator; the
// two comparators differ only for suffixes that agree through max_context
// symbols with both limits >= max_context, and those form contiguous runs
// of the unbounded SA.  suffix_cmp_with orders such suffixes by
// boundary_order on their full limits (src/lcp.rs:192-200), i.e. by limit
// (ShorterFirst) or by descending limit then position (LongerFirst).
__global__ void run_head_value_kernel(const uint8_t *__restrict__ flags, uint32_t n,
                                      uint32_t *__restrict__ hv, uint32_t *__restrict__ in_run) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        bool f = flags[i];
        hv[i] = f ? 0u : i;
        in_run[i] = (f || (i + 1 < n && flags[i + 1])) ? 1u : 0u;
    }
}

__global__ void run_compact_kernel(const uint8_t *__restrict__ flags, uint32_t n,
                                   const uint32_t *__restrict__ sa,
                                   const uint32_t *__restrict__ run_id,
                                   const uint32_t *__restrict__ dst, DevLimits L, int lf,
                                   uint64_t *__restrict__ keys, uint32_t *__restrict__ vals) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        bool in = flags[i] || (i + 1 < n && flags[i + 1]);
        if (!in) continue;
        uint32_t p = sa[i];
        uint64_t lim = dev_lim_at(L, p);
        uint64_t lk = lf ? (uint64_t)L.n - lim : lim;
        keys[dst[i]] = (lk << 32) | p;
        vals[dst[i]] = run_id[i];
    }
}

__global__ void run_swap_kernel(const uint64_t *__restrict__ k1, const uint32_t *__restrict__ v1,
                                uint32_t total, uint64_t *__restrict__ k2,
                                uint32_t *__restrict__ v2) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += gridDim.x * blockDim.x) {
        k2[t] = v1[t];
        v2[t] = (uint32_t)(k1[t] & 0xFFFFFFFFull);
    }
}

__global__ void run_writeback_kernel(const uint64_t *__restrict__ runk,
                                     const uint32_t *__restrict__ pos, uint32_t total,
                                     uint32_t *__restrict__ sa, uint32_t n) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += gridDim.x * blockDim.x) {
        uint64_t r = runk[t];
        uint32_t hd = (t == 0 || runk[t - 1] != r) ? t : run_head(runk, 0, t, r);
        uint64_t at = r + (t - hd);
        if (at < n) sa[at] = pos[t];
    }
}

__global__ void isa_kernel(const uint32_t *__restrict__ sa, uint32_t n, uint32_t *__restrict__ isa) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        isa[sa[i]] = i;
}

// Subset output key: the suffix's index in the full SA (whose tie classes
// are in ascending position), with the empty suffix at n first under
// ShorterFirst and last under LongerFirst.
template <typename PT>
__global__ void subset_isa_key_kernel(const PT *__restrict__ pos, uint64_t m, uint64_t n,
                                      const uint32_t *__restrict__ isa, int lf,
                                      uint64_t *__restrict__ keys, uint32_t *__restrict__ vals,
                                      int *__restrict__ bad) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t p = (uint64_t)pos[i];
        if (p > n) {
            atomicExch(bad, 1);
            p = n;
        }
        uint64_t rk;
        if (p == n)
            rk = lf ? n + 1 : 0ull;
        else
            rk = (uint64_t)__ldg(isa + p) + 1;
        keys[i] = rk;
        vals[i] = (uint32_t)p;
    }
}

// Subsets of distinct positions: one bit per requested position (p < n),
// set by warp-combined atomics. flags[0]: a position beyond n; flags[1]: a
// position requested twice; count[0]: requests of the empty suffix n.  Every
// lane of a warp takes the same number of steps (the match and reduction
// below need them together).
template <typename PT>
__global__ void subset_bits_kernel(const PT *__restrict__ pos, uint64_t m, uint64_t n,
                                   uint32_t *__restrict__ bits, int *__restrict__ flags,
                                   unsigned long long *__restrict__ count) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t base = warp * 32; base < m; base += nwarps * 32) {
        const uint64_t i = base + lane;
        const bool valid = i < m;
        const uint64_t p = valid ? (uint64_t)pos[i] : 0ull;
        if (valid && p > n) atomicExch(&flags[0], 1);
        if (valid && p == n) atomicAdd(count, 1ull);
        const bool set = valid && p < n;
        const unsigned active = __ballot_sync(0xffffffffu, set);
        if (set) {
            const uint32_t w = (uint32_t)(p >> 5);
            const unsigned peers = __match_any_sync(active, w);
            const uint32_t mask = __reduce_or_sync(peers, 1u << (uint32_t)(p & 31));
            if ((int)lane == __ffs((int)peers) - 1) {
                const uint32_t old = atomicOr(&bits[w], mask);
                if ((old & mask) != 0u || __popc(mask) != __popc(peers)) atomicExch(&flags[1], 1);
            }
        }
    }
}

// ---------------------------------------------------------------- sample-sort partition

// Comparison keys of the sorted text for the partition: suffixes that
// suffix_cmp_with (src/lcp.rs:184-201) calls Equal form contiguous runs of
// the sorted order, and every suffix's key is 1 + the SA index where its run
// starts, so key order is exactly the comparator's order (ties included);
// the empty suffix (position n) gets 0 (ShorterFirst) or n + 1
// (LongerFirst).  Ties exist only under SegmentedText with ShorterFirst
// (equal limits, equal symbols through min(limit, max_context)); head[j] =
// j for a run start, else 0, and a max-scan spreads the starts.
__global__ void tie_head_kernel(const uint32_t *__restrict__ sa, uint32_t n,
                                const uint8_t *__restrict__ text, int sym_bytes, DevLimits L,
                                uint64_t max_ctx, uint32_t *__restrict__ head) {
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        bool tie = false;
        if (j > 0) {
            const uint32_t a = sa[j - 1], b = sa[j];
            const uint64_t la = dev_lim_at(L, a), lb = dev_lim_at(L, b);
            if (la == lb) {
                const uint64_t lim = la < max_ctx ? la : max_ctx;
                const uint64_t k = (uint64_t)sym_bytes;
                tie = thread_lcp_bytes(text, (uint64_t)a * k, (uint64_t)b * k, lim * k) >= lim * k;
            }
        }
        head[j] = tie ? 0u : j;
    }
}

__global__ void head_key_kernel(const uint32_t *__restrict__ sa, uint32_t n,
                                const uint32_t *__restrict__ head, int lf,
                                uint32_t *__restrict__ hkey) {
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x)
        hkey[sa[j]] = (head ? head[j] : j) + 1;
    if (blockIdx.x == 0 && threadIdx.x == 0) hkey[n] = lf ? n + 1 : 0u;
}

// Chunk-major order of the sorted suffixes (full text): record = chunk of
// the position above the SA index, in SA order; a stable sort on the chunk
// bits then lists every chunk's suffixes in sorted order, each by its rank
// (the record's low 32 bits).
__global__ void chunk_key_kernel(const uint32_t *__restrict__ sa, uint32_t n, uint32_t chunk,
                                 uint64_t *__restrict__ keys) {
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x)
        keys[j] = ((uint64_t)(sa[j] / chunk) << 32) | j;
}

// Subsets: key = (chunk of the input index, rank of the suffix), value =
// the position.
template <typename PT>
__global__ void chunk_key_subset_kernel(const PT *__restrict__ pos, uint64_t m, uint64_t n,
                                        uint32_t chunk, const uint32_t *__restrict__ isa, int lf,
                                        int rbits, uint64_t *__restrict__ keys,
                                        uint32_t *__restrict__ vals) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t p = (uint64_t)pos[i];
        const uint64_t rk = p >= n ? (lf ? n + 1 : 0ull) : (uint64_t)__ldg(isa + p) + 1;
        keys[i] = ((i / chunk) << rbits) | rk;
        vals[i] = (uint32_t)p;
    }
}

// Evenly spaced midpoints of every sorted chunk (evenly_spaced,
// src/ext_mem.rs:1291-1305), with each sample's rank key.  `isa` null: the
// chunks hold SA indices (full text), which are the ranks.
__global__ void sample_kernel(const uint32_t *__restrict__ chunked,
                              const uint64_t *__restrict__ chunked_rec, uint64_t m, uint32_t chunk,
                              uint32_t p, uint32_t per, const uint32_t *__restrict__ soff,
                              uint64_t n, const uint32_t *__restrict__ isa, int lf,
                              uint64_t *__restrict__ skey, uint32_t *__restrict__ spos) {
    const uint64_t total = (uint64_t)p * per;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total;
         t += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t i = (uint32_t)(t / per), sidx = (uint32_t)(t % per);
        const uint64_t start = (uint64_t)i * chunk;
        if (start >= m) continue;
        const uint64_t len = m - start < chunk ? m - start : chunk;
        const uint64_t cnt = per < len ? per : len;
        if (sidx >= cnt) continue;
        const uint64_t at = cnt >= len ? sidx : (2 * (uint64_t)sidx + 1) * len / (2 * cnt);
        const uint32_t q = chunked ? chunked[start + at] : (uint32_t)chunked_rec[start + at];
        const uint32_t o = soff[i] + sidx;
        spos[o] = q;
        skey[o] = !isa ? (uint64_t)q + 1
                       : (q >= n ? (lf ? n + 1 : 0ull) : (uint64_t)__ldg(isa + q) + 1);
    }
}

// Pivots samples[j * ns / p] (phase 2, src/ext_mem.rs:1309-1342) with their
// comparison keys.  `sa` non-null: the samples are SA indices (full text),
// keyed by their tie-run head (or themselves), and the pivot is sa[q].
__global__ void pivot_kernel(const uint32_t *__restrict__ sorted_samples, uint32_t ns, uint32_t p,
                             const uint32_t *__restrict__ hkey, const uint32_t *__restrict__ sa,
                             const uint32_t *__restrict__ head, uint32_t *__restrict__ piv_pos,
                             uint32_t *__restrict__ piv_key) {
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j + 1 < p;
         j += gridDim.x * blockDim.x) {
        const uint32_t q = sorted_samples[(uint64_t)(j + 1) * ns / p];
        piv_pos[j] = sa ? sa[q] : q;
        piv_key[j] = sa ? (head ? head[q] : q) + 1 : hkey[q];
    }
}

// Training set of the learned CDF model: every stride-th sorted sample,
// its packed prefix and its rank fraction among all ns samples.
__global__ void train_set_kernel(const uint32_t *__restrict__ sorted_samples, uint32_t ns,
                                 uint32_t stride, uint32_t tn, Packed P,
                                 const uint32_t *__restrict__ sa, uint64_t *__restrict__ x,
                                 float *__restrict__ t) {
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < tn; j += gridDim.x * blockDim.x) {
        const uint32_t q = j * stride;
        const uint32_t s = sorted_samples[q];
        x[j] = window_at(P, sa ? sa[s] : s);
        t[j] = ((float)q + 0.5f) / (float)ns;
    }
}

// Partition of every suffix (phase 3, src/ext_mem.rs:1361-1428, with
// upper_bound_by_pivot :1705-1734): b = the number of pivots that compare
// less than the suffix, every comparison an exact suffix_cmp_with read from
// the comparison keys.  SPLITTERS: binary search over the pivots.  LEARNED:
// the CDF model predicts b from the suffix's packed prefix; the prediction
// is checked against its two neighbouring pivots and moved until both hold.
// `sa` non-null (full text): the suffixes are visited in SA order, item j
// keyed by its tie-run head (or j) and its prefix read at sa[j]; otherwise
// `items` lists the subset's positions in sorted order, keyed by hkey.
// b must never decrease along the sorted order (checked by the caller).
// Pivot keys and the bucket histogram live in shared memory.
template <bool LEARNED>
__global__ void __launch_bounds__(256)
    partition_kernel(const uint32_t *__restrict__ items, uint32_t m, Packed P,
                     const uint32_t *__restrict__ hkey, const uint32_t *__restrict__ sa,
                     const uint32_t *__restrict__ head, const uint32_t *__restrict__ piv_key,
                     uint32_t n_piv, uint32_t p, const __nv_bfloat16 *__restrict__ w,
                     uint32_t *__restrict__ bucket_of, unsigned long long *__restrict__ sizes,
                     unsigned long long *__restrict__ stats) {
    extern __shared__ __align__(16) unsigned char psm[];
    uint32_t *sk = reinterpret_cast<uint32_t *>(psm);
    uint32_t *hist = sk + n_piv;
    __nv_bfloat16 *sw = reinterpret_cast<__nv_bfloat16 *>(hist + p);
    for (uint32_t j = threadIdx.x; j < n_piv; j += blockDim.x) sk[j] = piv_key[j];
    for (uint32_t j = threadIdx.x; j < p; j += blockDim.x) hist[j] = 0;
    if (LEARNED)
        for (int j = threadIdx.x; j < cdf::kParams; j += blockDim.x) sw[j] = w[j];
    __syncthreads();
    unsigned long long probes = 0, mis = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
        const uint32_t s = items ? items[i] : i;
        const uint32_t ks = sa ? (head ? head[i] : i) + 1 : hkey[s];
        uint32_t b;
        if (LEARNED) {
            const float y = cdf::infer_bf16(sw, window_at(P, sa ? sa[i] : s));
            float g = floorf(y * (float)p);
            g = g < 0.0f ? 0.0f : (g > (float)n_piv ? (float)n_piv : g);
            b = (uint32_t)g;
            const uint32_t guess = b;
            while (b > 0 && (probes++, !(sk[b - 1] < ks))) b--;
            if (b == guess)
                while (b < n_piv && (probes++, sk[b] < ks)) b++;
            mis += b != guess ? 1u : 0u;
        } else {
            uint32_t lo = 0, hi = n_piv;
            while (lo < hi) {
                const uint32_t mid = (lo + hi) >> 1;
                probes++;
                if (sk[mid] < ks)
                    lo = mid + 1;
                else
                    hi = mid;
            }
            b = lo;
        }
        atomicAdd(&hist[b], 1u);
        bucket_of[i] = b;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        probes += __shfl_xor_sync(0xffffffffu, probes, o);
        mis += __shfl_xor_sync(0xffffffffu, mis, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&stats[0], probes);
        atomicAdd(&stats[1], mis);
    }
    __syncthreads();
    for (uint32_t j = threadIdx.x; j < p; j += blockDim.x)
        if (hist[j]) atomicAdd(&sizes[j], (unsigned long long)hist[j]);
}

// Partitions along the sorted order never decrease (else flag); `sa`
// non-null: bucket_of is indexed by position and the order is sa's.
__global__ void partition_check_kernel(const uint32_t *__restrict__ bucket_of,
                                       const uint32_t *__restrict__ sa, uint32_t m,
                                       int *__restrict__ bad) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x + 1; i < m;
         i += gridDim.x * blockDim.x) {
        const uint32_t b0 = bucket_of[sa ? sa[i - 1] : i - 1], b1 = bucket_of[sa ? sa[i] : i];
        if (b1 < b0) atomicExch(bad, 1);
    }
}

// ---------------------------------------------------------------- partition-first sample sort
//
// build_in_memory_sample_sort with the partition ahead of the sort: the
// splitter sample is sorted on its own, every suffix finds its bucket by
// comparing itself with the pivots (phase 3, src/ext_mem.rs:1361-1428 and
// upper_bound_by_pivot :1705-1734) inside the kernel that builds its sort
// record, and the bucket becomes the top field of that record.  Every
// member of bucket b (pivot[b-1] < s <= pivot[b]) starts with the common
// prefix of its two pivots (ell[b] symbols), so the record's key window
// starts there: the bucket carries the prefix, the window the symbols after
// it.  The one radix sort of (bucket, window, field, position) then leaves
// every bucket contiguous and in suffix order up to the window, and the
// usual refinement finishes each bucket (phase 4, src/ext_mem.rs:1745-2108).

constexpr uint64_t kPfCmpCap = 1ull << 16;  // symbols an exact sample comparison may read
constexpr uint64_t kPfPivotCap = 1ull << 12;  // symbols a suffix-vs-pivot comparison may read
constexpr uint32_t kPfTieMax = 64;          // largest run of equal sample keys sorted exactly
constexpr uint32_t kPfEllCap = 0xFFFFu;     // window offsets are capped (any prefix length works)
constexpr uint32_t kPfTrainSamples = 16384;  // learned model: training samples (of the sorted sample)
constexpr int kPfTrainSteps = 32;            // Adam steps after the interpolating start

// Comparison key of a suffix on its first spw symbols: the packed window,
// truncated at the limit and padded low (ShorterFirst) or high
// (LongerFirst).  Strictly smaller keys mean strictly smaller suffixes under
// suffix_cmp_with (src/lcp.rs:184-201); equal keys need an exact compare.
__device__ __forceinline__ uint64_t prefix_key(const Packed &P, uint64_t p, uint64_t lim, int lf) {
    uint64_t w = window_at(P, p);
    if (lim < (uint64_t)P.spw) {
        const uint32_t keep = (uint32_t)lim * (uint32_t)P.b;  // < 64
        const uint64_t low = ~0ull >> keep;                    // the bits after the kept symbols
        w = lf ? (w | low) : (w & ~low);
    }
    return w;
}

// Sample of the input order: ns evenly spaced midpoints of the text, each
// with its comparison key.
__global__ void pf_sample_kernel(Packed P, DevLimits L, uint64_t n, uint32_t ns, int lf,
                                 uint64_t *__restrict__ keys, uint32_t *__restrict__ pos) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += gridDim.x * blockDim.x) {
        const uint64_t p = ((2 * (uint64_t)i + 1) * n) / (2 * (uint64_t)ns);
        keys[i] = prefix_key(P, p, dev_lim_at(L, p), lf);
        pos[i] = (uint32_t)p;
    }
}

// Runs of equal keys in the key-sorted sample, each put in exact suffix
// order by one thread (insertion sort, exact compares); a run longer than
// kPfTieMax or a compare deeper than kPfCmpCap sets *fallback.
__global__ void pf_sample_ties_kernel(const uint64_t *__restrict__ keys, uint32_t *__restrict__ pos,
                                      uint32_t ns, Packed P, DevLimits L, int lf,
                                      int *__restrict__ fallback) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i + 1 < ns;
         i += gridDim.x * blockDim.x) {
        const uint64_t k = keys[i];
        if ((i > 0 && keys[i - 1] == k) || keys[i + 1] != k) continue;  // not the head of a run
        uint32_t j = i + 1;
        while (j < ns && keys[j] == k && j - i <= kPfTieMax) j++;
        if (j - i > kPfTieMax) {
            atomicExch(fallback, 1);
            continue;
        }
        for (uint32_t a = i + 1; a < j; a++) {  // insertion sort, stable
            const uint32_t x = pos[a];
            const uint64_t lx = dev_lim_at(L, x);
            uint32_t b = a;
            while (b > i) {
                const uint32_t y = pos[b - 1];
                const int c = direct_cmp(P, y, dev_lim_at(L, y), x, lx, 0, kPfCmpCap, lf);
                if (c == 2) atomicExch(fallback, 1);
                if (c <= 0 || c == 2) break;
                pos[b] = y;
                b--;
            }
            pos[b] = x;
        }
    }
}

// Pivots samples[(j + 1) * ns / p] (phase 2, src/ext_mem.rs:1309-1342) with
// their keys and limits.
__global__ void pf_pivot_kernel(const uint32_t *__restrict__ spos, uint32_t ns, uint32_t p,
                                Packed P, DevLimits L, int lf, uint64_t *__restrict__ pkey,
                                uint32_t *__restrict__ ppos, uint64_t *__restrict__ plim) {
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j + 1 < p;
         j += gridDim.x * blockDim.x) {
        const uint32_t q = spos[(uint64_t)(j + 1) * ns / p];
        const uint64_t lim = dev_lim_at(L, q);
        ppos[j] = q;
        plim[j] = lim;
        pkey[j] = prefix_key(P, q, lim, lf);
    }
}

// Key-window offset of every bucket: the common prefix of its two pivots
// (0 for the first and last buckets, which have one pivot), capped.
__global__ void pf_ell_kernel(const uint32_t *__restrict__ ppos, const uint64_t *__restrict__ plim,
                              uint32_t p, Packed P, uint16_t *__restrict__ ell) {
    for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < p; b += gridDim.x * blockDim.x) {
        uint64_t t = 0;
        if (b > 0 && b + 1 < p) {
            const uint64_t x = ppos[b - 1], y = ppos[b];
            uint64_t lim = plim[b - 1] < plim[b] ? plim[b - 1] : plim[b];
            if (lim > kPfEllCap) lim = kPfEllCap;
            while (t < lim) {
                const uint64_t d = window_at(P, x + t) ^ window_at(P, y + t);
                if (d) {
                    t += (uint64_t)__clzll((long long)d) / (uint64_t)P.b;
                    break;
                }
                t += (uint64_t)P.spw;
            }
            if (t > lim) t = lim;
        }
        ell[b] = (uint16_t)t;
    }
}

// Top-bits index of the pivot keys: tbl[t] = the number of pivots whose
// key's top kPfTableBits bits are below t (t = 0 .. 2^kPfTableBits), so the
// pivots a key can fall between are [tbl[top], tbl[top + 1]).
constexpr int kPfTableBits = 12;
__global__ void pf_table_kernel(const uint64_t *__restrict__ pkey, uint32_t n_piv,
                                uint16_t *__restrict__ tbl) {
    const uint32_t nt = (1u << kPfTableBits) + 1;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += gridDim.x * blockDim.x) {
        uint32_t lo = 0, hi = n_piv;
        if (t >= (1u << kPfTableBits)) {
            lo = n_piv;
        } else {
            const uint64_t key = (uint64_t)t << (64 - kPfTableBits);
            while (lo < hi) {
                const uint32_t mid = (lo + hi) >> 1;
                if (pkey[mid] < key)
                    lo = mid + 1;
                else
                    hi = mid;
            }
        }
        tbl[t] = (uint16_t)lo;
    }
}

// Sort record of every text position with its bucket (the fused partition):
// bucket b = the number of pivots that compare less than the suffix, found
// by binary search over the pivot keys in shared memory (SPLITTERS) or
// predicted by the learned CDF model from the suffix's packed prefix and
// walked until both neighbouring pivots agree (LEARNED); key ties with a
// pivot are settled by an exact comparison.  The record is
//   bucket | window of k symbols from ell[b] | length field | position,
// with the digit histograms of every radix pass and the bucket sizes
// accumulated on the way (shared memory, then one global add per block).
// kPlain: PlainText limits (n - p).
template <bool kPlain, bool LEARNED>
__global__ void __launch_bounds__(kKeyThreads)
    pf_key_kernel(Packed P, uint64_t n, DevLimits L, int k, int lbits, int flag_len, int vbits,
                  int lf, int n_passes, int bucket_shift, const uint64_t *__restrict__ pkey,
                  const uint32_t *__restrict__ ppos, const uint64_t *__restrict__ plim,
                  const uint16_t *__restrict__ ell, const uint16_t *__restrict__ tbl, uint32_t p,
                  const __nv_bfloat16 *__restrict__ w, int bisect,
                  uint64_t *__restrict__ keys, uint32_t *__restrict__ counts,
                  unsigned long long *__restrict__ sizes, unsigned long long *__restrict__ stats,
                  int *__restrict__ fallback) {
    extern __shared__ __align__(16) unsigned char pfs[];
    const uint32_t n_piv = p - 1;
    constexpr uint32_t kTbl = (1u << kPfTableBits) + 1;
    uint64_t *sk = reinterpret_cast<uint64_t *>(pfs);           // n_piv pivot keys
    uint32_t *bh = reinterpret_cast<uint32_t *>(sk + n_piv);    // p bucket counts
    uint32_t *hist = bh + p;                                     // 8 * 256 digit counts
    uint16_t *sell = reinterpret_cast<uint16_t *>(hist + 8 * 256);  // p window offsets
    uint16_t *stbl = sell + p;                                   // kTbl top-bits index
    __nv_bfloat16 *sw = reinterpret_cast<__nv_bfloat16 *>(stbl + kTbl + 1);
    for (uint32_t j = threadIdx.x; j < n_piv; j += kKeyThreads) sk[j] = pkey[j];
    for (uint32_t j = threadIdx.x; j < p; j += kKeyThreads) {
        sell[j] = ell[j];
        bh[j] = 0;
    }
    for (uint32_t j = threadIdx.x; j < kTbl; j += kKeyThreads) stbl[j] = tbl[j];
    for (int i = threadIdx.x; i < 8 * 256; i += kKeyThreads) hist[i] = 0;
    if (LEARNED)
        for (int j = threadIdx.x; j < cdf::kParams; j += kKeyThreads) sw[j] = w[j];
    __syncthreads();
    const int b = P.b;
    const int kbits = k * b;  // 1..63
    unsigned long long probes = 0, mis = 0;
    bool deep = false;
    // each thread takes kKeyPer consecutive positions, in three phases so
    // that their loads overlap: prefix keys, buckets, then the windows after
    // the buckets' common prefixes
    cdf::MmaWeights MW;
    if (LEARNED) MW = cdf::mma_weights(sw);
    for (uint64_t t0 = (uint64_t)blockIdx.x * kKeyTile; t0 < n;
         t0 += (uint64_t)gridDim.x * kKeyTile) {
        // every lane stays in the loop (the model runs warp-wide); lanes past
        // the end work on the last position and store nothing
        const uint64_t p0 = t0 + (uint64_t)threadIdx.x * kKeyPer;
        uint64_t K[kKeyPer], lim[kKeyPer];
#pragma unroll
        for (int e = 0; e < kKeyPer; e++) {
            const uint64_t q = p0 + e < n ? p0 + e : n - 1;
            lim[e] = kPlain ? n - q : dev_lim_at(L, q);
            K[e] = prefix_key(P, q, lim[e], lf);
        }
        float yp[kKeyPer];
        if (LEARNED) {
#pragma unroll
            for (int e = 0; e < kKeyPer; e++) yp[e] = cdf::infer_mma(MW, K[e]);
        }
        uint32_t bk[kKeyPer];
#pragma unroll
        for (int e = 0; e < kKeyPer; e++) {
            const uint64_t q = p0 + e;
            // suffix q > pivot j ?  (key order, an exact compare on key ties)
            auto greater = [&](uint32_t j) -> bool {
                probes++;
                const uint64_t pk = sk[j];
                if (K[e] != pk) return K[e] > pk;
                const uint32_t pj = __ldg(ppos + j);
                if (pj == q) return false;  // the pivot itself
                const int c = direct_cmp(P, q, lim[e], pj, __ldg(plim + j), 0, kPfPivotCap, lf);
                if (c == 2) deep = true;
                return c == 1;
            };
            if (q >= n) {
                bk[e] = 0;
                continue;
            }
            if (LEARNED) {
                // the model's guess, checked against its two neighbouring
                // pivots; a wrong guess gallops away from it and bisects
                float g = floorf(yp[e] * (float)p);
                g = g < 0.0f ? 0.0f : (g > (float)n_piv ? (float)n_piv : g);
                const uint32_t guess = (uint32_t)g;
                uint32_t lo, hi;  // the bucket lies in [lo, hi]
                if (guess > 0 && !greater(guess - 1)) {  // below the guess
                    hi = guess - 1;
                    uint32_t d = 1;
                    for (;;) {
                        if (hi < d) {
                            lo = 0;
                            break;
                        }
                        const uint32_t j = hi - d;
                        if (greater(j)) {
                            lo = j + 1;
                            break;
                        }
                        hi = j;
                        d *= 2;
                    }
                } else if (guess < n_piv && greater(guess)) {  // above the guess
                    lo = guess + 1;
                    uint32_t d = 1;
                    for (;;) {
                        if (lo + d - 1 >= n_piv) {
                            hi = n_piv;
                            break;
                        }
                        const uint32_t j = lo + d - 1;
                        if (!greater(j)) {
                            hi = j;
                            break;
                        }
                        lo = j + 1;
                        d *= 2;
                    }
                } else {
                    lo = hi = guess;
                }
                while (lo < hi) {
                    const uint32_t mid = (lo + hi) >> 1;
                    if (greater(mid))
                        lo = mid + 1;
                    else
                        hi = mid;
                }
                bk[e] = lo;
                mis += lo != guess ? 1u : 0u;
            } else {
                // binary search between the pivots that share the key's top
                // bits (or over all of them: bisect)
                const uint32_t top = (uint32_t)(K[e] >> (64 - kPfTableBits));
                uint32_t lo = bisect ? 0u : stbl[top], hi = bisect ? n_piv : stbl[top + 1];
                while (lo < hi) {
                    const uint32_t mid = (lo + hi) >> 1;
                    if (greater(mid))
                        lo = mid + 1;
                    else
                        hi = mid;
                }
                bk[e] = lo;
            }
        }
        uint64_t out[kKeyPer];
#pragma unroll
        for (int e = 0; e < kKeyPer; e++) {
            const uint64_t q = p0 + e;
            uint64_t rec = 0;
            if (q < n) {
                atomicAdd(&bh[bk[e]], 1u);
                // window of k symbols after the bucket's common prefix
                const uint64_t off = sell[bk[e]];
                const uint64_t rest = lim[e] > off ? lim[e] - off : 0;
                const uint64_t bit = (q + off) * (uint64_t)b;
                const uint64_t wi = bit >> 6;
                const uint32_t sh = (uint32_t)(bit & 63);
                const uint64_t w0 = __ldg(P.w + wi), w1 = __ldg(P.w + wi + 1);
                uint64_t content = ((w0 << sh) | ((w1 >> 1) >> (63 - sh))) >> (64 - kbits);
                int take = k;
                if (rest < (uint64_t)k) {
                    take = (int)rest;
                    const uint64_t lowmask = (1ull << ((k - take) * b)) - 1;
                    content = lf ? (content | lowmask) : (content & ~lowmask);
                }
                const uint64_t field = flag_len ? (uint64_t)((take == k) != (lf != 0))
                                                : (uint64_t)(lf ? k - take : take);
                rec = (lbits ? (content << lbits) | field : content) |
                      ((uint64_t)bk[e] << bucket_shift);
                const uint32_t rlo = (uint32_t)rec, rhi = (uint32_t)(rec >> 32);
#pragma unroll
                for (int ps = 0; ps < 8; ps++)
                    if (ps < n_passes)
                        atomicAdd(&hist[ps * 256 + (((ps < 4 ? rlo : rhi) >> (8 * (ps & 3))) & 255u)],
                                  1u);
                rec = (rec << vbits) | q;
            }
            out[e] = rec;
        }
        if (p0 + kKeyPer <= n) {
            uint4 *dst = reinterpret_cast<uint4 *>(keys + p0);
#pragma unroll
            for (int e = 0; e < kKeyPer; e += 2)
                dst[e / 2] = make_uint4((uint32_t)out[e], (uint32_t)(out[e] >> 32),
                                        (uint32_t)out[e + 1], (uint32_t)(out[e + 1] >> 32));
        } else {
            for (int e = 0; e < kKeyPer; e++)
                if (p0 + e < n) keys[p0 + e] = out[e];
        }
    }
    if (deep) atomicExch(fallback, 1);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        probes += __shfl_xor_sync(0xffffffffu, probes, o);
        mis += __shfl_xor_sync(0xffffffffu, mis, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&stats[0], probes);
        atomicAdd(&stats[1], mis);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n_passes * 256; i += kKeyThreads)
        if (hist[i]) atomicAdd(&counts[i], hist[i]);
    for (uint32_t j = threadIdx.x; j < p; j += kKeyThreads)
        if (bh[j]) atomicAdd(&sizes[j], (unsigned long long)bh[j]);
}

// Learned mode: the model's bucket for every sample of the exactly sorted
// sample, evaluated exactly as the fused kernel evaluates suffixes (the
// same tensor-core inference from the same BF16 weights).
__global__ void __launch_bounds__(256)
    pf_sample_bucket_kernel(const uint32_t *__restrict__ spos, uint32_t ns, Packed P, DevLimits L,
                            int lf, uint32_t p, const __nv_bfloat16 *__restrict__ w,
                            uint32_t *__restrict__ mb) {
    __shared__ __nv_bfloat16 sw[cdf::kParams + 1];
    for (int j = threadIdx.x; j < cdf::kParams; j += blockDim.x) sw[j] = w[j];
    __syncthreads();
    const cdf::MmaWeights MW = cdf::mma_weights(sw);
    // whole warps step together (the model runs warp-wide)
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < ns; base += stride) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t q = spos[i < ns ? i : ns - 1];
        const uint64_t key = prefix_key(P, q, dev_lim_at(L, q), lf);
        const float y = cdf::infer_mma(MW, key);
        float g = floorf(y * (float)p);
        g = g < 0.0f ? 0.0f : (g > (float)(p - 1) ? (float)(p - 1) : g);
        if (i < ns) mb[i] = (uint32_t)g;
    }
}

// Learned mode's pivots: pivot j - 1 (j = 1 .. p - 1) is the first sorted
// sample whose running-maximum model bucket reaches j, so a suffix between
// two samples of one predicted bucket is predicted exactly and only the
// suffixes next to a bucket boundary can be one bucket off.  mx = inclusive
// running maximum of the samples' buckets; pivots no sample reaches take the
// last sample.
__global__ void pf_model_pivot_kernel(const uint32_t *__restrict__ spos,
                                      const uint32_t *__restrict__ mx, uint32_t ns, uint32_t p,
                                      Packed P, DevLimits L, int lf, uint64_t *__restrict__ pkey,
                                      uint32_t *__restrict__ ppos, uint64_t *__restrict__ plim) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += gridDim.x * blockDim.x) {
        const uint32_t lo = i == 0 ? 0u : mx[i - 1];
        uint32_t hi = mx[i];
        if (i + 1 == ns) hi = p - 1;  // the last sample also takes every pivot above it
        if (hi <= lo) continue;
        const uint32_t q = spos[i];
        const uint64_t lim = dev_lim_at(L, q);
        const uint64_t key = prefix_key(P, q, lim, lf);
        for (uint32_t j = lo + 1; j <= hi && j < p; j++) {
            ppos[j - 1] = q;
            plim[j - 1] = lim;
            pkey[j - 1] = key;
        }
    }
}

// Training set of the learned model from the exactly sorted sample: every
// stride-th sample's comparison key and its rank fraction.
__global__ void pf_train_set_kernel(const uint32_t *__restrict__ spos,
                                    const uint64_t *__restrict__ skeys_unused, uint32_t ns,
                                    uint32_t stride, uint32_t tn, Packed P, DevLimits L, int lf,
                                    uint64_t *__restrict__ x, float *__restrict__ t) {
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < tn; j += gridDim.x * blockDim.x) {
        const uint32_t q = j * stride;
        const uint32_t s = spos[q];
        x[j] = prefix_key(P, s, dev_lim_at(L, s), lf);
        t[j] = ((float)q + 0.5f) / (float)ns;
    }
}

}  // namespace eng

// ---------------------------------------------------------------- host

inline int bits_for(uint64_t v) {  // bits to represent 0..v
    int b = 0;
    while (b < 64 && (v >> b) != 0) b++;
    return b == 0 ? 1 : b;
}

// A subset sorted on its own (records for the m chosen positions only,
// instead of the whole text): the positions, distinct and ascending.
struct SparseRun {
    const uint32_t *pos = nullptr;  // device, m positions < n
    uint64_t m = 0;
    bool fell_back = false;  // out: a tied group needs rank doubling; nothing returned
};

// Request and outcome of a partition-first core_sort (the sample sort's
// buckets computed before the sort and leading its records).
struct PfRun {
    uint32_t p = 0;
    bool learned = false;
    bool bisect = false;  // splitter search over all pivots, without the top-bits index
    bool fell_back = false;                  // out: a comparison ran too deep; nothing sorted
    const uint32_t *d_pivots = nullptr;      // out: device, p - 1 pivot positions
    const unsigned long long *d_sizes = nullptr;  // out: device, p bucket sizes + 2 stats
};

// The partition-first front of core_sort: the splitter sample (the same
// count as the reference's sampler, as evenly spaced midpoints of the text)
// sorted exactly, its pivots and their common prefixes, the learned model
// (LEARNED), then the fused partition + record kernel over every position.
// A sample run longer than kPfTieMax, a sample comparison deeper than
// kPfCmpCap symbols or a pivot comparison deeper than kPfPivotCap sets
// pf->fell_back (checked after the sample sort and after the fused kernel).
template <typename S>
capssa_status pf_keys(Ctx &c, const EngineArgs &a, const eng::Packed &P, const KeyGeom &geo,
                      int bucket_bits, int key_passes, uint64_t *keys, uint32_t *counts,
                      PfRun *pf) {
    using namespace eng;
    const uint64_t n = a.n;
    const int lf = a.lim.longer_first;
    const uint32_t p = pf->p;
    // sample count of the reference's sampler (src/ext_mem.rs:1282-1287)
    double ln_n = std::log((double)n);
    if (ln_n < 1.0) ln_n = 1.0;
    uint64_t total = (uint64_t)p * (uint64_t)std::ceil(4.0 * ln_n);
    total = std::min<uint64_t>(std::max<uint64_t>(total, p), n);
    const uint32_t per = (uint32_t)((total + p - 1) / p);
    const uint32_t ns = (uint32_t)std::min<uint64_t>((uint64_t)per * p, n);
    const size_t nsb = (size_t)ns + 64;
    const size_t bytes = nsb * 8 * 2 + nsb * 4 * 2 + (size_t)p * (8 + 4 + 8 + 4) +
                         ((size_t)p + 4) * 8 + (size_t)65536 * 12 + cdf::kParams * 6 + 16 * 256;
    char *w = (char *)ws_get(c, WS_PART, bytes);
    if (!w) return set_err(c, CAPSSA_ENOMEM, "partition-first workspace");
    auto carve = [&](size_t sz) {
        char *r = w;
        w += (sz + 255) & ~(size_t)255;
        return r;
    };
    uint64_t *sk_a = (uint64_t *)carve(nsb * 8), *sk_b = (uint64_t *)carve(nsb * 8);
    uint32_t *sp_a = (uint32_t *)carve(nsb * 4), *sp_b = (uint32_t *)carve(nsb * 4);
    uint64_t *pkey = (uint64_t *)carve((size_t)p * 8);
    uint32_t *ppos = (uint32_t *)carve((size_t)p * 4);
    uint64_t *plim = (uint64_t *)carve((size_t)p * 8);
    uint16_t *ell = (uint16_t *)carve((size_t)p * 2);
    uint16_t *tbl = (uint16_t *)carve(((size_t)1 << kPfTableBits) * 2 + 16);
    unsigned long long *sizes = (unsigned long long *)carve(((size_t)p + 4) * 8);
    uint64_t *tx = (uint64_t *)carve((size_t)65536 * 8);
    float *tt = (float *)carve((size_t)65536 * 4);
    float *params = (float *)carve(cdf::kParams * 4);
    __nv_bfloat16 *wbf = (__nv_bfloat16 *)carve(cdf::kParams * 2);
    int *fb = c.d_flags + 1;
    CAPSSA_CUDA(c, cudaMemsetAsync(fb, 0, 4, c.stream));
    // 1. sample, sorted by key, then exactly
    pf_sample_kernel<<<grid_for(ns, 256), 256, 0, c.stream>>>(P, a.lim, n, ns, lf, sk_a, sp_a);
    CAPSSA_LAUNCHED(c);
    bool in_b = false;
    const int kb = P.spw * P.b;
    capssa_status s = radix::sort_pairs(c, sk_a, sp_a, sk_b, sp_b, ns, 64 - kb, 64, false, 0, &in_b);
    if (s != CAPSSA_OK) return s;
    const uint64_t *skeys = in_b ? sk_b : sk_a;
    uint32_t *spos = in_b ? sp_b : sp_a;
    pf_sample_ties_kernel<<<grid_for(ns, 256), 256, 0, c.stream>>>(skeys, spos, ns, P, a.lim, lf,
                                                                   fb);
    CAPSSA_LAUNCHED(c);
    int *h_fb = (int *)c.h_scratch;
    CAPSSA_CUDA(c, cudaMemcpyAsync(h_fb, fb, 4, cudaMemcpyDeviceToHost, c.stream));
    CAPSSA_CUDA(c, cudaStreamSynchronize(c.stream));
    if (*h_fb) {  // a degenerate sample: sort first instead
        pf->fell_back = true;
        return CAPSSA_OK;
    }
    // 2. the learned CDF model on the sorted sample (learned mode)
    if (pf->learned) {
        const uint32_t tn = std::min<uint32_t>(ns, kPfTrainSamples);
        const uint32_t stride = (ns + tn - 1) / tn;
        const uint32_t tn_eff = (ns + stride - 1) / stride;
        pf_train_set_kernel<<<grid_for(tn_eff, 256), 256, 0, c.stream>>>(
            spos, skeys, ns, stride, tn_eff, P, a.lim, lf, tx, tt);
        CAPSSA_LAUNCHED(c);
        cudaEvent_t t0, t1;
        cudaEventCreate(&t0);
        cudaEventCreate(&t1);
        cudaEventRecord(t0, c.stream);
        float loss = 0.0f;
        s = cdf::train(c, tx, tt, tn_eff, kPfTrainSteps, params, wbf, &loss, /*knot_start=*/true);
        cudaEventRecord(t1, c.stream);
        cudaEventSynchronize(t1);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, t0, t1);
        cudaEventDestroy(t0);
        cudaEventDestroy(t1);
        if (s != CAPSSA_OK) return s;
        c.stats.train_ms = ms;
        c.stats.model_loss = loss;
        c.stats.train_samples = tn_eff;
    }
    // 3. pivots: samples[(j + 1) * ns / p] (splitters), or where the model's
    // predicted bucket steps (learned); then the buckets' common prefixes
    if (pf->learned) {
        uint32_t *mb = (uint32_t *)ws_get(c, WS_MISC, (size_t)ns * 4 + 64);
        if (!mb) return set_err(c, CAPSSA_ENOMEM, "model buckets");
        pf_sample_bucket_kernel<<<grid_for(ns, 256), 256, 0, c.stream>>>(spos, ns, P, a.lim, lf, p,
                                                                         wbf, mb);
        CAPSSA_LAUNCHED(c);
        s = scan_u32(c, mb, mb, ns, /*max_op=*/true, /*inclusive=*/true);
        if (s != CAPSSA_OK) return s;
        pf_model_pivot_kernel<<<grid_for(ns, 256), 256, 0, c.stream>>>(spos, mb, ns, p, P, a.lim,
                                                                       lf, pkey, ppos, plim);
        CAPSSA_LAUNCHED(c);
    } else {
        pf_pivot_kernel<<<grid_for(p, 256), 256, 0, c.stream>>>(spos, ns, p, P, a.lim, lf, pkey,
                                                                ppos, plim);
        CAPSSA_LAUNCHED(c);
    }
    pf_ell_kernel<<<grid_for(p, 256), 256, 0, c.stream>>>(ppos, plim, p, P, ell);
    CAPSSA_LAUNCHED(c);
    pf_table_kernel<<<grid_for((1u << kPfTableBits) + 1, 256), 256, 0, c.stream>>>(pkey, p - 1,
                                                                                    tbl);
    CAPSSA_LAUNCHED(c);
    // 4. the fused partition + record kernel (the sample's sort used the
    // histogram buffer: clear it for the records' digit counts)
    CAPSSA_CUDA(c, cudaMemsetAsync(counts, 0, radix::kMaxPasses * 256 * 4, c.stream));
    CAPSSA_CUDA(c, cudaMemsetAsync(sizes, 0, ((size_t)p + 4) * 8, c.stream));
    const size_t smem = (size_t)(p - 1) * 8 + (size_t)p * 4 + 8 * 256 * 4 + (size_t)p * 2 +
                        (((size_t)1 << kPfTableBits) + 2) * 2 + cdf::kParams * 2 + 16;
    const bool plain = !a.lim.segmented;
    const unsigned grid = std::min<unsigned>(grid_for(n, kKeyTile), (unsigned)c.sm_count * 8);
    cudaEvent_t q0, q1;
    cudaEventCreate(&q0);
    cudaEventCreate(&q1);
#define CAPSSA_PF_LAUNCH(PL, LE)                                                                  \
    do {                                                                                          \
        cudaFuncSetAttribute(pf_key_kernel<PL, LE>, cudaFuncAttributeMaxDynamicSharedMemorySize,  \
                             (int)smem);                                                          \
        pf_key_kernel<PL, LE><<<grid, kKeyThreads, smem, c.stream>>>(                             \
            P, n, a.lim, geo.k, geo.lbits, geo.flag_len, geo.vbits, lf, key_passes, geo.total,    \
            pkey, ppos, plim, ell, tbl, p, wbf, pf->bisect ? 1 : 0, keys, counts, sizes, sizes + p, \
            fb);                                                                                   \
    } while (0)
    cudaEventRecord(q0, c.stream);
    if (plain && pf->learned)
        CAPSSA_PF_LAUNCH(true, true);
    else if (plain)
        CAPSSA_PF_LAUNCH(true, false);
    else if (pf->learned)
        CAPSSA_PF_LAUNCH(false, true);
    else
        CAPSSA_PF_LAUNCH(false, false);
#undef CAPSSA_PF_LAUNCH
    CAPSSA_LAUNCHED(c);
    cudaEventRecord(q1, c.stream);
    CAPSSA_CUDA(c, cudaMemcpyAsync(h_fb, fb, 4, cudaMemcpyDeviceToHost, c.stream));
    CAPSSA_CUDA(c, cudaStreamSynchronize(c.stream));
    float pms = 0.0f;
    cudaEventElapsedTime(&pms, q0, q1);
    cudaEventDestroy(q0);
    cudaEventDestroy(q1);
    c.stats.partition_ms = pms;
    pf->fell_back = *h_fb != 0;
    pf->d_pivots = ppos;
    pf->d_sizes = sizes;
    (void)bucket_bits;
    return CAPSSA_OK;
}

// Steps 1-4 of engine.cuh over every text position under the unbounded
// comparator; *sa_out receives the device SA (n entries).  With `pf`, the
// records lead with the sample sort's bucket (partition first).
template <typename S>
capssa_status core_sort(Ctx &c, const EngineArgs &a, uint32_t **sa_out, eng::Packed *pk_out,
                        PfRun *pf = nullptr, SparseRun *sp = nullptr) {
    using namespace eng;
    const uint64_t n = a.n;
    const int lf = a.lim.longer_first;
    const S *text = (const S *)a.text;
    cudaEventRecord(c.pev[0], c.stream);

    // ---- 1. alphabet -> codes
    const uint16_t *table = nullptr;
    uint32_t minv = 0;
    uint64_t sigma_span = 1;
    if (sizeof(S) <= 2) {
        const uint32_t nvals = sizeof(S) == 1 ? 256u : 65536u;
        uint32_t *present = (uint32_t *)ws_get(c, WS_CODES, nvals * 4 + nvals * 2 + 64);
        if (!present) return set_err(c, CAPSSA_ENOMEM, "alphabet table");
        CAPSSA_CUDA(c, cudaMemsetAsync(present, 0, nvals * 4, c.stream));
        presence_kernel<S><<<std::min<unsigned>(grid_for(n, 256), c.sm_count * 8), 256, 0,
                             c.stream>>>(text, n, present);
        CAPSSA_LAUNCHED(c);
        std::vector<uint32_t> h_present(nvals);
        CAPSSA_CUDA(c, cudaMemcpyAsync(h_present.data(), present, nvals * 4,
                                       cudaMemcpyDeviceToHost, c.stream));
        CAPSSA_CUDA(c, cudaStreamSynchronize(c.stream));
        std::vector<uint16_t> h_code(nvals);
        uint32_t next = 0;
        for (uint32_t v = 0; v < nvals; v++) {
            h_code[v] = (uint16_t)next;
            if (h_present[v]) next++;
        }
        sigma_span = next ? next : 1;
        uint16_t *d_code = (uint16_t *)(present + nvals);
        CAPSSA_CUDA(c, cudaMemcpyAsync(d_code, h_code.data(), nvals * 2, cudaMemcpyHostToDevice,
                                       c.stream));
        CAPSSA_CUDA(c, cudaStreamSynchronize(c.stream));  // h_code goes out of scope
        table = d_code;
    } else {
        uint32_t *mm = (uint32_t *)ws_get(c, WS_CODES, 64);
        if (!mm) return set_err(c, CAPSSA_ENOMEM, "alphabet table");
        uint32_t init[2] = {0xFFFFFFFFu, 0u};
        CAPSSA_CUDA(c, cudaMemcpyAsync(mm, init, 8, cudaMemcpyHostToDevice, c.stream));
        minmax_kernel<<<std::min<unsigned>(grid_for(n, 256), c.sm_count * 8), 256, 0, c.stream>>>(
            (const uint32_t *)text, n, mm);
        CAPSSA_LAUNCHED(c);
        uint32_t h_mm[2];
        CAPSSA_CUDA(c, cudaMemcpyAsync(h_mm, mm, 8, cudaMemcpyDeviceToHost, c.stream));
        CAPSSA_CUDA(c, cudaStreamSynchronize(c.stream));
        minv = h_mm[0];
        sigma_span = (uint64_t)h_mm[1] - h_mm[0] + 1;
    }
    const int b = bits_for(sigma_span > 1 ? sigma_span - 1 : 1);
    // order-0 entropy of the symbols from an evenly strided sample: the key
    // must hold about log2(n) / H + 3 symbols to leave few random ties
    // (the b-bit code width overstates H for skewed alphabets)
    double hbits = (double)b;
    if (n >= (1u << 20) && b > 1) {  // small texts: ties are cheap either way
        const uint64_t ns = 65536, stride = n / ns;
        S *d_hs = (S *)ws_get(c, WS_MISC3, ns * sizeof(S) + 64);
        if (!d_hs) return set_err(c, CAPSSA_ENOMEM, "entropy sample");
        strided_sample_kernel<S><<<grid_for(ns, 256), 256, 0, c.stream>>>(text, ns, stride, d_hs);
        CAPSSA_LAUNCHED(c);
        std::vector<S> hs(ns);
        CAPSSA_CUDA(c, cudaMemcpyAsync(hs.data(), d_hs, ns * sizeof(S), cudaMemcpyDeviceToHost,
                                       c.stream));
        CAPSSA_CUDA(c, cudaStreamSynchronize(c.stream));
        double hsum = 0.0;
        auto add = [&](uint64_t cnt) {
            const double q = (double)cnt / (double)ns;
            hsum -= q * std::log2(q);
        };
        if (sizeof(S) <= 2) {  // counts per value
            std::vector<uint32_t> cnt(sizeof(S) == 1 ? 256 : 65536, 0);
            for (S v : hs) cnt[v]++;
            for (uint32_t x : cnt)
                if (x) add(x);
        } else {
            std::sort(hs.begin(), hs.end());
            for (uint64_t i = 0; i < ns;) {
                uint64_t j = i;
                while (j < ns && hs[j] == hs[i]) j++;
                add(j - i);
                i = j;
            }
        }
        // within 3% of the code width counts as full (sampling noise)
        hbits = hsum >= 0.97 * b ? (double)b : std::max<double>(hsum, 0.25);
    }
    // segment-major order: the segment index sits above the key bits, and
    // the key only has to tell apart the suffixes of one segment
    int seg_bits =
        a.seg_major && a.lim.segmented && a.lim.n_ends > 1 ? bits_for(a.lim.n_ends - 1) : 0;
    if (seg_bits + b + 1 > 64) seg_bits = 0;  // no room: the caller splits by segment itself
    // one segment is already in segment-major order
    c.seg_major_done = a.seg_major && (seg_bits > 0 || a.lim.n_ends <= 1);
    // a ShorterFirst plain text may drop the early-end flag when that saves a
    // radix pass
    const bool allow_flagless = !a.lim.segmented && !lf && n <= 0xFFFFFFFEull && !pf && !sp;
    KeyGeom geo;
    if (pf) {  // the bucket index leads the record
        seg_bits = bits_for(pf->p - 1);
        geo = pf_geom(b, n, !a.lim.segmented, hbits, seg_bits);
        if (geo.k == 0) {
            pf->fell_back = true;
            return CAPSSA_OK;
        }
    } else {
        geo = key_geom(b, n, !a.lim.segmented, hbits, seg_bits,
                       seg_bits ? a.seg_max_len : (sp ? sp->m : 0), allow_flagless,
                       a.seg_major && !lf);
    }
    // records the radix sort orders: every suffix, or the full ones only
    const uint64_t n_short = geo.flagless ? (uint64_t)geo.k - 1 : 0;
    // suffixes in the output: every position, or the chosen subset's
    const uint64_t N = sp ? sp->m : n;
    const uint64_t n_rec = N - n_short;
    const int sort_bits = geo.total + seg_bits;
    c.stats.key_symbols = geo.k;
    c.stats.key_bits_per_symbol = geo.b;

    // ---- 2+3. composite keys of every position, stable radix sort
    const uint32_t nn = (uint32_t)N;
    uint64_t *keys_a = (uint64_t *)ws_get(c, WS_KEYS_A, (size_t)N * 8);
    uint64_t *keys_b = (uint64_t *)ws_get(c, WS_KEYS_B, (size_t)N * 8);
    uint32_t *vals_a = (uint32_t *)ws_get(c, WS_VALS_A, (size_t)N * 4);
    uint32_t *vals_b = (uint32_t *)ws_get(c, WS_VALS_B, (size_t)N * 4);
    // position-indexed ranks: only rank doubling reads them, which a subset
    // sorted on its own never reaches
    uint32_t *rank = (uint32_t *)ws_get(c, WS_RANK, (size_t)(sp ? 1 : n) * 4 + 64);
    uint64_t *key2 = (uint64_t *)ws_get(c, WS_KEY2, (size_t)N * 8);
    if (!keys_a || !keys_b || !vals_a || !vals_b || !rank || !key2)
        return set_err(c, CAPSSA_ENOMEM, "suffix-sort workspace");
    Coder<S> coder{table, minv};
    // when key and position fit one word, the sort moves 8 B per suffix and
    // pass instead of 12
    const int vbits = geo.vbits;
    const int local_pos = vbits && seg_bits && geo.local_pos ? 1 : 0;
    const int key_passes = (sort_bits + 7) / 8;
    uint32_t *counts = radix::hist_buffer(c);
    if (!counts) return set_err(c, CAPSSA_ENOMEM, "radix histograms");
    CAPSSA_CUDA(c, cudaMemsetAsync(counts, 0, radix::kMaxPasses * 256 * 4, c.stream));
    // bit-packed copy of the text: the key windows, and the direct
    // comparisons of small groups
    const uint64_t nwords = (n * (uint64_t)geo.b + 63) / 64 + 4;
    uint64_t *packed = (uint64_t *)ws_get(c, WS_PACKED, nwords * 8);
    if (!packed) return set_err(c, CAPSSA_ENOMEM, "packed text");
    if (sizeof(S) == 1 && table && 64 % geo.b == 0 && ((uintptr_t)text & 15) == 0)
        pack_u8_kernel<<<grid_for(nwords, 256), 256, 0, c.stream>>>(
            (const uint8_t *)text, n, table, geo.b, packed, nwords);
    else
        pack_text_kernel<S><<<grid_for(nwords, 256), 256, 0, c.stream>>>(text, n, coder, geo.b,
                                                                         packed, nwords);
    CAPSSA_LAUNCHED(c);
    Packed P;
    P.w = packed;
    P.b = geo.b;
    P.spw = 64 / geo.b;
    P.mask = P.spw * P.b >= 64 ? ~0ull : (~0ull << (64 - P.spw * P.b));
    const unsigned kgrid = std::min<unsigned>(grid_for(n_rec, kKeyTile), c.sm_count * 8);
    if (pf) {
        capssa_status s0 = pf_keys<S>(c, a, P, geo, seg_bits, key_passes, keys_a, counts, pf);
        if (s0 != CAPSSA_OK || pf->fell_back) return s0;
    } else if (sp) {
        const unsigned sg = std::min<unsigned>(grid_for(N, kKeyThreads), c.sm_count * 8);
        if (!a.lim.segmented)
            sparse_key_kernel<true><<<sg, kKeyThreads, 0, c.stream>>>(
                P, n, sp->pos, N, a.lim, geo.k, geo.lbits, geo.flag_len, vbits, lf, key_passes,
                keys_a, counts);
        else
            sparse_key_kernel<false><<<sg, kKeyThreads, 0, c.stream>>>(
                P, n, sp->pos, N, a.lim, geo.k, geo.lbits, geo.flag_len, vbits, lf, key_passes,
                keys_a, counts);
        CAPSSA_LAUNCHED(c);
        if (!vbits)  // the record's value is its position
            CAPSSA_CUDA(c, cudaMemcpyAsync(vals_a, sp->pos, (size_t)N * 4, cudaMemcpyDeviceToDevice,
                                           c.stream));
    } else if (!a.lim.segmented && !seg_bits && geo.flagless && vbits && 8 % geo.b == 0 &&
               geo.total % 8 == 0 && key_passes == geo.total / 8 && n_rec >= 64) {
        key_flagless_kernel<<<kgrid, kKeyThreads, 0, c.stream>>>(P, n_rec, geo.total, vbits,
                                                                 keys_a, counts);
        CAPSSA_LAUNCHED(c);
        key_hist_shift_kernel<<<1, 256, 0, c.stream>>>(P, n_rec, geo.total, key_passes, counts);
        CAPSSA_LAUNCHED(c);
    } else if (!a.lim.segmented && !seg_bits) {
        key_kernel<true><<<kgrid, kKeyThreads, 0, c.stream>>>(
            P, n, n_rec, a.lim, geo.k, geo.lbits, geo.flag_len, vbits, lf, key_passes, 0, 0,
            keys_a, counts);
        CAPSSA_LAUNCHED(c);
    } else {
        key_kernel<false><<<kgrid, kKeyThreads, 0, c.stream>>>(
            P, n, n_rec, a.lim, geo.k, geo.lbits, geo.flag_len, vbits, lf, key_passes,
            seg_bits ? geo.total : 0, local_pos, keys_a, counts);
        CAPSSA_LAUNCHED(c);
    }
    cudaEventRecord(c.pev[1], c.stream);
    bool in_b = false;
    int passes = 0;
    capssa_status s =
        vbits ? radix::sort_keys(c, keys_a, keys_b, (uint32_t)n_rec, vbits, vbits + sort_bits,
                                 &in_b, &passes, /*hist_ready=*/true)
              : radix::sort_pairs(c, keys_a, vals_a, keys_b, vals_b, nn, 0, sort_bits, !sp, 0,
                                  &in_b, &passes, /*hist_ready=*/true);
    if (s != CAPSSA_OK) return s;
    c.stats.sort_passes = (uint32_t)passes;
    c.stats.sort_item_bytes = vbits ? 8u : 12u;
    cudaEventRecord(c.pev[2], c.stream);
    const uint64_t *skeys = in_b ? keys_b : keys_a;
    // packed positions are unpacked into vals_a by init_groups
    uint32_t *sa = (in_b && !vbits) ? vals_b : vals_a;
    // packed records are unpacked straight into a u32 output of a full build,
    // which then needs no final copy
    if (vbits && !a.positions && !a.keep_bits && a.out_bytes == 4 && a.out_sa)
        sa = (uint32_t *)a.out_sa;
    uint32_t *spare_vals = sa == vals_a ? vals_b : vals_a;

    // ---- 4. tied groups: direct comparison while shallow, rank doubling when deep
    // list capacities from the smallest group each list can hold
    const size_t cap_of[kLists] = {(size_t)N / 2 + 2,  (size_t)N / 3 + 2, (size_t)N / 9 + 2,
                                   (size_t)N / 33 + 2, (size_t)N / 2 + 2, (size_t)N / 5 + 2};
    const size_t big_cap = (size_t)N / (kSmallMax + 1) + 2;
    size_t list_bytes = 256 + big_cap * 16 * 2;
    for (int l = 0; l < kLists; l++) list_bytes += cap_of[l] * 16 * 2;
    GroupLists G;
    char *gl = (char *)ws_get(c, WS_GROUPS_A, list_bytes);
    uint32_t *hd = (uint32_t *)ws_get(c, WS_GROUPS_B, (size_t)N * 4 + 64);
    if (!gl || !hd) return set_err(c, CAPSSA_ENOMEM, "group lists");
    G.ctr = (Counters *)gl;
    uint4 *cursor = (uint4 *)(gl + 256);
    for (int l = 0; l < kLists; l++)
        for (int q = 0; q < 2; q++) {
            G.list[l][q] = cursor;
            cursor += cap_of[l];
        }
    G.big[0] = (BigGroup *)cursor;
    G.big[1] = G.big[0] + big_cap;
    uint64_t h = (uint64_t)geo.k;
    KernelTimes kt(profile_on());
    kt.start(c.stream);
    // flagless: where the short suffixes go among the sorted full ones
    ShortList *d_short = nullptr;
    if (n_short) {
        d_short = (ShortList *)ws_get(c, WS_SAMPLE, sizeof(ShortList) + 64);
        if (!d_short) return set_err(c, CAPSSA_ENOMEM, "short suffixes");
        short_place_kernel<<<1, 64, 0, c.stream>>>(P, n, (uint32_t)n_rec, geo.k, skeys, vbits,
                                                   d_short);
        CAPSSA_LAUNCHED(c);
    }
    CAPSSA_CUDA(c, cudaMemsetAsync(G.ctr, 0, sizeof(Counters), c.stream));
    {
        const unsigned ig = grid_for(n_rec, kInitTile);
        const uint64_t lm = (1ull << geo.lbits) - 1;
        const int seg_at = local_pos ? vbits + geo.total : 0;
#define CAPSSA_IG(FL, UN, SG)                                                                  \
    init_groups_kernel<FL, UN, SG><<<ig, 256, 0, c.stream>>>(skeys, (uint32_t)n_rec, geo.k, lm, \
                                                             lf, vbits, hd, sa, G, d_short,      \
                                                             seg_at, a.lim.ends)
        if (!vbits) {
            if (geo.flag_len == 0) CAPSSA_IG(0, false, false);
            else if (geo.flag_len == 1) CAPSSA_IG(1, false, false);
            else CAPSSA_IG(2, false, false);
        } else if (seg_at) {
            if (geo.flag_len == 0) CAPSSA_IG(0, true, true);
            else if (geo.flag_len == 1) CAPSSA_IG(1, true, true);
            else CAPSSA_IG(2, true, true);
        } else {
            if (geo.flag_len == 0) CAPSSA_IG(0, true, false);
            else if (geo.flag_len == 1) CAPSSA_IG(1, true, false);
            else CAPSSA_IG(2, true, false);
        }
#undef CAPSSA_IG
    }
    CAPSSA_LAUNCHED(c);
    if (n_short) {
        short_write_kernel<<<1, 64, 0, c.stream>>>(d_short, sa, hd);
        CAPSSA_LAUNCHED(c);
    }
    kt.mark(c.stream, "groups");
    kt.print();

    const int k2bits = bits_for(n + 1);
    const uint64_t empty_lf = (1ull << k2bits) - 1;  // above every rank
    const uint64_t empty = lf ? empty_lf : 0ull;
    bool ranks_ready = false;
    uint32_t *runs_s = nullptr;  // run ends, for the run keys of deep rounds
    int cur = 0;
    Counters *hc = (Counters *)c.h_scratch;
    for (;;) {
        CAPSSA_CUDA(c, cudaMemcpyAsync(hc, G.ctr, sizeof(Counters), cudaMemcpyDeviceToHost,
                                       c.stream));
        CAPSSA_CUDA(c, cudaStreamSynchronize(c.stream));
        uint32_t cnt[kLists];
        uint32_t any = 0;
        for (int l = 0; l < kLists; l++) any |= (cnt[l] = hc->n[l][cur]);
        const uint32_t nb = (uint32_t)(hc->big_packed[cur] >> 40);
        const uint32_t big_total = (uint32_t)(hc->big_packed[cur] & kBigTotMask);
        if (profile_on())
            std::fprintf(stderr,
                         "capssa profile  round %u depth %llu: pairs %u tiny %u+%u small %u "
                         "medium %u deep %u big %u (%u suffixes)\n",
                         c.stats.refine_rounds + 1, (unsigned long long)h, cnt[L_PAIR],
                         cnt[L_TINY], cnt[L_TINY8], cnt[L_SMALL], cnt[L_MEDIUM], cnt[L_DEEP],
                         nb, big_total);
        if (!any && !nb) break;
        if (sp && (nb || cnt[L_DEEP])) {  // deep ties: the subset needs the whole text's ranks
            sp->fell_back = true;
            return CAPSSA_OK;
        }
        if (c.stats.refine_rounds >= 70)
            return set_err(c, CAPSSA_EINVAL, "rank doubling did not converge");
        c.stats.refine_rounds++;
        const int nxt = cur ^ 1;
        // rank doubling reads position-ordered ranks; they are built from the
        // SA-ordered heads the first time a round needs them
        kt.start(c.stream);
        if ((nb || cnt[L_DEEP]) && !ranks_ready) {
            // beyond L2 the sorted keys' buffers (dead once the groups are
            // listed) hold the window pairs and counts
            s = scatter_u32(c, sa, hd, nn, rank, n, keys_a, (uint32_t *)keys_b);
            if (s != CAPSSA_OK) return s;
            ranks_ready = true;
            kt.mark(c.stream, "ranks");
        }
        uint32_t *rk = ranks_ready ? rank : nullptr;
        for (int l = 0; l < kLists; l++)
            CAPSSA_CUDA(c, cudaMemsetAsync(&G.ctr->n[l][nxt], 0, 4, c.stream));
        CAPSSA_CUDA(c, cudaMemsetAsync(&G.ctr->big_packed[nxt], 0, 8, c.stream));
        // the direct kernels work on disjoint groups and only append to the
        // next round's lists: the four small-group kinds run on side streams
        // next to the medium kernel on the main one (each alone is latency-
        // bound and leaves the SMs half idle), joined before rank doubling
        CAPSSA_CUDA(c, cudaEventRecord(c.fork_ev, c.stream));
        int forked = 0;
        auto side = [&]() -> cudaStream_t {
            cudaStream_t st = c.side[forked];
            cudaStreamWaitEvent(st, c.fork_ev, 0);
            forked++;
            return st;
        };
        if (cnt[L_PAIR]) {
            direct_pair_kernel<<<grid_for(cnt[L_PAIR], 256), 256, 0, side()>>>(
                G.list[L_PAIR][cur], cnt[L_PAIR], sa, hd, rk, a.lim, P, lf, G, nxt);
            CAPSSA_LAUNCHED(c);
        }
        if (cnt[L_TINY]) {
            direct_tiny_kernel<kTiny4><<<grid_for(cnt[L_TINY], 128), 128, 0, side()>>>(
                G.list[L_TINY][cur], cnt[L_TINY], sa, hd, rk, a.lim, P, lf, G, nxt);
            CAPSSA_LAUNCHED(c);
        }
        if (cnt[L_TINY8]) {
            direct_tiny_seg_kernel<kTinyMax>
                <<<grid_for((uint64_t)cnt[L_TINY8] * kTinyMax, 128), 128, 0, side()>>>(
                    G.list[L_TINY8][cur], cnt[L_TINY8], sa, hd, rk, a.lim, P, lf, G, nxt);
            CAPSSA_LAUNCHED(c);
        }
        if (cnt[L_SMALL]) {
            direct_warp_kernel<<<grid_for((uint64_t)cnt[L_SMALL] * 32, 128), 128, 0, side()>>>(
                G.list[L_SMALL][cur], cnt[L_SMALL], sa, hd, rk, a.lim, P, lf, G, nxt);
            CAPSSA_LAUNCHED(c);
        }
        if (cnt[L_MEDIUM]) {
            direct_medium_kernel<<<std::min<unsigned>(cnt[L_MEDIUM], c.sm_count * 8), kMedThreads,
                                   0, c.stream>>>(G.list[L_MEDIUM][cur], cnt[L_MEDIUM], sa, hd,
                                                  rk, a.lim, P, lf, G, nxt);
            CAPSSA_LAUNCHED(c);
        }
        for (int i = 0; i < forked; i++) {
            CAPSSA_CUDA(c, cudaEventRecord(c.join_ev[i], c.side[i]));
            CAPSSA_CUDA(c, cudaStreamWaitEvent(c.stream, c.join_ev[i], 0));
        }
        kt.mark(c.stream, "direct");
        // rank doubling last: the direct kernels above rewrote the ranks of
        // every group they resolved, which only refines them (equal ranks
        // still agree through h symbols) and settles the depth-0 groups of
        // early-ended suffixes, whose ranks agree on nothing yet
        if (cnt[L_DEEP]) {
            gather_small_kernel<<<grid_for(cnt[L_DEEP], 128), 128, 0, c.stream>>>(
                G.list[L_DEEP][cur], cnt[L_DEEP], sa, rank, a.lim, h, lf, empty_lf, key2);
            CAPSSA_LAUNCHED(c);
            sort_small_kernel<<<grid_for(cnt[L_DEEP], 128), 128, 0, c.stream>>>(
                G.list[L_DEEP][cur], cnt[L_DEEP], sa, key2, hd, rank, lf, empty, h, G, nxt);
            CAPSSA_LAUNCHED(c);
            kt.mark(c.stream, "deep");
        }
        const int ord_bits = nb > 1 ? bits_for(nb - 1) : 1;
        if (nb) {
            // run keys for ShorterFirst whole texts, when a run-length field
            // of at least 12 bits fits beside the ordinal and the rank
            RunKeys R{nullptr, P, n, 0};
            const int rbits = std::min(24, 64 - ord_bits - 1 - k2bits);
            if (!lf && !sp && rbits >= 12 && h >= 2 * (uint64_t)geo.k) {
                if (!runs_s) {  // built once, the first deep round that can use it
                    runs_s = (uint32_t *)ws_get(c, WS_RUNS, (size_t)n * 4 + 64);
                    if (!runs_s) return set_err(c, CAPSSA_ENOMEM, "run lengths");
                    run_ends_kernel<<<grid_for(n, 256), 256, 0, c.stream>>>(a.text, a.sym_bytes,
                                                                            n, runs_s);
                    CAPSSA_LAUNCHED(c);
                    s = scan_u32(c, runs_s, runs_s, n, /*max_op=*/true, /*inclusive=*/true);
                    if (s != CAPSSA_OK) return s;
                }
                R.runs_s = runs_s;
                R.rbits = rbits;
            }
            const int ord_shift = R.runs_s ? k2bits + 1 + rbits : k2bits;
            gather_big_kernel<<<grid_for(big_total, 256), 256, 0, c.stream>>>(
                G.big[cur], nb, big_total, sa, rank, a.lim, h, lf,
                                                        empty_lf, k2bits, R, keys_a, spare_vals);
            CAPSSA_LAUNCHED(c);
            bool tb = false;
            uint32_t *tv_b = (uint32_t *)key2;  // free once sort_small has run
            s = radix::sort_pairs(c, keys_a, spare_vals, keys_b, tv_b, big_total, 0,
                                  ord_shift + ord_bits, false, 0, &tb);
            if (s != CAPSSA_OK) return s;
            const uint64_t *tk = tb ? keys_b : keys_a;
            const uint32_t *tv = tb ? tv_b : spare_vals;
            split_big_kernel<<<grid_for(big_total, 256), 256, 0, c.stream>>>(
                tk, tv, big_total, G.big[cur], nb, k2bits, ord_shift, R, sa, hd, rank, lf, empty,
                h, G, nxt);
            CAPSSA_LAUNCHED(c);
            kt.mark(c.stream, "big");
        }
        kt.print();
        c.stats.refined_suffixes += big_total;
        h *= 2;
        cur = nxt;
    }
    cudaEventRecord(c.pev[3], c.stream);
    CAPSSA_CUDA(c, cudaEventSynchronize(c.pev[3]));
    float t01 = 0, t12 = 0, t23 = 0;
    cudaEventElapsedTime(&t01, c.pev[0], c.pev[1]);
    cudaEventElapsedTime(&t12, c.pev[1], c.pev[2]);
    cudaEventElapsedTime(&t23, c.pev[2], c.pev[3]);
    c.stats.keys_ms = t01;
    c.stats.sort_ms = t12;
    c.stats.refine_ms = t23;
    double pass_ms = 0;
    for (int i = 0; i < passes && i < 16; i++) {
        float ms = 0;
        cudaEventElapsedTime(&ms, c.kev[2 * i], c.kev[2 * i + 1]);
        pass_ms += ms;
    }
    c.stats.sort_pass_ms = pass_ms;
    if (profile_on())
        std::fprintf(stderr,
                     "capssa profile  n %llu k %d b %d: keys %.3f ms, sort %.3f ms (%d passes, "
                     "%.3f ms in pass kernels), refine %.3f ms (%u rounds)\n",
                     (unsigned long long)n, geo.k, geo.b, t01, t12, passes, pass_ms, t23,
                     c.stats.refine_rounds);
    *sa_out = sa;
    *pk_out = P;
    return CAPSSA_OK;
}

template <typename S>
capssa_status bounded_pass(Ctx &c, const EngineArgs &a, uint32_t *sa) {
    using namespace eng;
    const uint64_t n = a.n;
    const uint32_t nn = (uint32_t)n;
    uint8_t *flags = (uint8_t *)ws_get(c, WS_OUT2, (size_t)n + 64);
    uint32_t *hv = (uint32_t *)ws_get(c, WS_MISC, (size_t)n * 8 + 64);
    uint32_t *inr = (uint32_t *)ws_get(c, WS_MISC2, (size_t)n * 8 + 64);
    uint64_t *k1 = (uint64_t *)ws_get(c, WS_KEYS_A, (size_t)n * 8);
    uint64_t *k2 = (uint64_t *)ws_get(c, WS_KEYS_B, (size_t)n * 8);
    uint32_t *v1 = (uint32_t *)ws_get(c, WS_MISC3, (size_t)n * 8 + 64);
    if (!flags || !hv || !inr || !k1 || !k2 || !v1) return set_err(c, CAPSSA_ENOMEM, "bounded pass");
    uint32_t *v2 = v1 + n;
    capssa_status s = ctx_run_flags(c, a.text, a.sym_bytes, a.lim, a.max_ctx, sa, n, flags);
    if (s != CAPSSA_OK) return s;
    unsigned g = grid_for(n, 256);
    run_head_value_kernel<<<g, 256, 0, c.stream>>>(flags, nn, hv, inr);
    CAPSSA_LAUNCHED(c);
    uint32_t last_in = 0;
    CAPSSA_CUDA(c, cudaMemcpyAsync(c.h_scratch, inr + (n - 1), 4, cudaMemcpyDeviceToHost, c.stream));
    s = scan_u32(c, hv, hv, n, true, true);  // run id = max head index so far
    if (s != CAPSSA_OK) return s;
    CAPSSA_CUDA(c, cudaStreamSynchronize(c.stream));
    last_in = *(uint32_t *)c.h_scratch;
    s = scan_u32(c, inr, inr, n, false, false);  // compacted index
    if (s != CAPSSA_OK) return s;
    CAPSSA_CUDA(c, cudaMemcpyAsync(c.h_scratch, inr + (n - 1), 4, cudaMemcpyDeviceToHost, c.stream));
    CAPSSA_CUDA(c, cudaStreamSynchronize(c.stream));
    const uint32_t total = *(uint32_t *)c.h_scratch + last_in;
    if (total == 0) return CAPSSA_OK;
    run_compact_kernel<<<g, 256, 0, c.stream>>>(flags, nn, sa, hv, inr, a.lim, a.lim.longer_first,
                                                k1, v1);
    CAPSSA_LAUNCHED(c);
    bool tb = false;
    s = radix::sort_pairs(c, k1, v1, k2, v2, total, 0, 32 + bits_for(n), false, 0, &tb);
    if (s != CAPSSA_OK) return s;
    const uint64_t *sk = tb ? k2 : k1;
    const uint32_t *sv = tb ? v2 : v1;
    uint64_t *rk = tb ? k1 : k2;
    uint32_t *rv = (uint32_t *)hv;  // run ids were consumed by the compaction
    unsigned gt = grid_for(total, 256);
    run_swap_kernel<<<gt, 256, 0, c.stream>>>(sk, sv, total, rk, rv);
    CAPSSA_LAUNCHED(c);
    uint64_t *rk2 = tb ? k2 : k1;
    uint32_t *rv2 = (uint32_t *)inr;
    s = radix::sort_pairs(c, rk, rv, rk2, rv2, total, 0, bits_for(n), false, 0, &tb);
    if (s != CAPSSA_OK) return s;
    run_writeback_kernel<<<gt, 256, 0, c.stream>>>(tb ? rk2 : rk, tb ? rv2 : rv, total, sa, nn);
    CAPSSA_LAUNCHED(c);
    return CAPSSA_OK;
}

// Records the device time from its construction to its destruction as
// stats.finish_ms (the output ordering and copies of a build).
struct FinishTimer {
    Ctx &c;
    explicit FinishTimer(Ctx &cc) : c(cc) { cudaEventRecord(c.pev[4], c.stream); }
    ~FinishTimer() {
        cudaEventRecord(c.pev[5], c.stream);
        if (cudaEventSynchronize(c.pev[5]) == cudaSuccess) {
            float ms = 0;
            cudaEventElapsedTime(&ms, c.pev[4], c.pev[5]);
            c.stats.finish_ms = ms;
        }
    }
};

// Sample-sort partition plan over the sorted suffixes `sorted` (m entries):
// samples as the reference draws them (evenly spaced midpoints of every
// chunk of the input order, each chunk sorted), pivots, then the partition
// of every suffix by splitter search or by the learned CDF model with
// neighbour fixup.  Outputs: a.part_pivots / a.part_sizes (host) and the
// partition statistics.
template <typename S>
capssa_status partition_phase(Ctx &c, const EngineArgs &a, const eng::Packed &P,
                              const uint32_t *sa_full, const uint32_t *sorted, uint64_t m) {
    using namespace eng;
    const uint64_t n = a.n;
    const int lf = a.lim.longer_first;
    const uint32_t p = a.part_p;
    if (p == 0 || m == 0) return CAPSSA_OK;
    if (p > 24576) return set_err(c, CAPSSA_EUNSUPPORTED, "more than 24,576 subproblems");
    const uint32_t chunk = (uint32_t)((m + p - 1) / p);
    double ln_m = std::log((double)m);
    if (ln_m < 1.0) ln_m = 1.0;
    uint64_t total = (uint64_t)p * (uint64_t)std::ceil(4.0 * ln_m);
    total = std::min<uint64_t>(std::max<uint64_t>(total, p), m);
    const uint32_t per = (uint32_t)((total + p - 1) / p);
    // scratch: chunk-major keys/values (ping-pong), buckets, head runs, keys
    const size_t m8 = (size_t)m * 8 + 64, m4 = (size_t)m * 4 + 64, n4 = (size_t)n * 4 + 64;
    char *w = (char *)ws_get(c, WS_PART, 2 * m8 + 3 * m4 + 2 * n4);
    uint32_t *isa = (uint32_t *)ws_get(c, WS_RANK, (size_t)n * 4 + 64);
    if (!w || !isa) return set_err(c, CAPSSA_ENOMEM, "partition workspace");
    uint64_t *ka = (uint64_t *)w, *kb = (uint64_t *)(w + m8);
    uint32_t *va = (uint32_t *)(w + 2 * m8), *vb = (uint32_t *)(w + 2 * m8 + m4);
    uint32_t *bucket_of = (uint32_t *)(w + 2 * m8 + 2 * m4);
    uint32_t *head = (uint32_t *)(w + 2 * m8 + 3 * m4);
    uint32_t *hkey = (uint32_t *)(w + 2 * m8 + 3 * m4 + n4);
    const bool subset = a.positions != nullptr;
    KernelTimes kt(profile_on());
    kt.start(c.stream);
    // full text: every key below is an SA index or its tie-run head, so no
    // position-indexed array is built; subsets: the caller's isa is in place
    // 0. comparison keys (run heads of the comparator's ties)
    const bool ties = a.lim.segmented && !lf;
    if (ties) {
        tie_head_kernel<<<grid_for(n, 256), 256, 0, c.stream>>>(
            sa_full, (uint32_t)n, (const uint8_t *)a.text, a.sym_bytes, a.lim, a.max_ctx, head);
        CAPSSA_LAUNCHED(c);
        capssa_status s0 = scan_u32(c, head, head, n, /*max_op=*/true, /*inclusive=*/true);
        if (s0 != CAPSSA_OK) return s0;
    }
    if (subset) {
        head_key_kernel<<<grid_for(n, 256), 256, 0, c.stream>>>(sa_full, (uint32_t)n,
                                                                ties ? head : nullptr, lf, hkey);
        CAPSSA_LAUNCHED(c);
    }
    kt.mark(c.stream, "isa+heads");
    // 1. every chunk's positions in sorted order
    const int cbits = bits_for(p > 1 ? p - 1 : 1);
    bool in_b = false;
    capssa_status s;
    if (!subset) {
        chunk_key_kernel<<<grid_for(m, 256), 256, 0, c.stream>>>(sa_full, (uint32_t)m, chunk,
                                                                 ka);
        CAPSSA_LAUNCHED(c);
        s = radix::sort_keys(c, ka, kb, (uint32_t)m, 32, 32 + cbits, &in_b);
    } else {
        const int rbits = bits_for(n + 1);
        if (a.pos_bytes == 4)
            chunk_key_subset_kernel<uint32_t><<<grid_for(m, 256), 256, 0, c.stream>>>(
                (const uint32_t *)a.positions, m, n, chunk, isa, lf, rbits, ka, va);
        else
            chunk_key_subset_kernel<uint64_t><<<grid_for(m, 256), 256, 0, c.stream>>>(
                (const uint64_t *)a.positions, m, n, chunk, isa, lf, rbits, ka, va);
        CAPSSA_LAUNCHED(c);
        s = radix::sort_pairs(c, ka, va, kb, vb, (uint32_t)m, 0, rbits + cbits, false, 0, &in_b);
    }
    if (s != CAPSSA_OK) return s;
    kt.mark(c.stream, "chunks");
    // full text: SA indices in the low halves of the sorted records
    const uint32_t *chunked = subset ? (in_b ? vb : va) : nullptr;
    const uint64_t *chunked_rec = subset ? nullptr : (in_b ? kb : ka);
    // 2. samples and their rank keys, sorted; pivots
    std::vector<uint32_t> soff(p + 1, 0);
    for (uint32_t i = 0; i < p; i++) {
        const uint64_t start = (uint64_t)i * chunk;
        const uint64_t len = start >= m ? 0 : std::min<uint64_t>(chunk, m - start);
        soff[i + 1] = soff[i] + (uint32_t)std::min<uint64_t>(per, len);
    }
    const uint32_t ns = soff[p];
    const uint32_t n_piv = (p > 1 && ns > 0) ? p - 1 : 0;
    const size_t nsb = (size_t)ns + 64;
    char *sw = (char *)ws_get(c, WS_SAMPLE, (p + 1) * 4 + 16 + nsb * 8 * 2 + nsb * 4 * 2 +
                                                (size_t)p * 16 + 256 + (size_t)65536 * 12 +
                                                cdf::kParams * 6 + 64);
    if (!sw) return set_err(c, CAPSSA_ENOMEM, "sample workspace");
    uint32_t *d_soff = (uint32_t *)sw;
    uint64_t *sk_a = (uint64_t *)(sw + ((((size_t)p + 1) * 4 + 15) & ~(size_t)15));
    uint64_t *sk_b = sk_a + nsb;
    uint32_t *sp_a = (uint32_t *)(sk_b + nsb), *sp_b = sp_a + nsb;
    uint32_t *piv_pos = sp_b + nsb;
    uint32_t *piv_key = piv_pos + p;
    unsigned long long *sizes =
        (unsigned long long *)(((uintptr_t)(piv_key + p) + 15) & ~(uintptr_t)15);
    unsigned long long *pstats = sizes + p;  // probes, mispredictions
    uint64_t *tx = (uint64_t *)(pstats + 4);
    float *tt = (float *)(tx + 65536);
    float *params = tt + 65536;
    __nv_bfloat16 *wbf = (__nv_bfloat16 *)(params + cdf::kParams + 3);
    CAPSSA_CUDA(c, cudaMemcpyAsync(d_soff, soff.data(), (p + 1) * 4, cudaMemcpyHostToDevice,
                                   c.stream));
    sample_kernel<<<grid_for((uint64_t)p * per, 256), 256, 0, c.stream>>>(
        chunked, chunked_rec, m, chunk, p, per, d_soff, n, subset ? isa : nullptr, lf, sk_a, sp_a);
    CAPSSA_LAUNCHED(c);
    bool s_in_b = false;
    s = radix::sort_pairs(c, sk_a, sp_a, sk_b, sp_b, ns, 0, bits_for(n + 1), false, 0, &s_in_b);
    if (s != CAPSSA_OK) return s;
    const uint32_t *sorted_samples = s_in_b ? sp_b : sp_a;
    if (n_piv) {
        pivot_kernel<<<grid_for(n_piv, 256), 256, 0, c.stream>>>(
            sorted_samples, ns, p, hkey, subset ? nullptr : sa_full,
            !subset && ties ? head : nullptr, piv_pos, piv_key);
        CAPSSA_LAUNCHED(c);
    }
    // 3. learned CDF model on the sample (learned mode)
    const bool learned = a.part_mode == CAPSSA_PARTITION_LEARNED && n_piv > 0;
    if (learned) {
        const uint32_t tn = std::min<uint32_t>(ns, 65536);
        const uint32_t stride = (ns + tn - 1) / tn;
        const uint32_t tn_eff = (ns + stride - 1) / stride;
        train_set_kernel<<<grid_for(tn_eff, 256), 256, 0, c.stream>>>(
            sorted_samples, ns, stride, tn_eff, P, subset ? nullptr : sa_full, tx, tt);
        CAPSSA_LAUNCHED(c);
        cudaEvent_t t0, t1;
        cudaEventCreate(&t0);
        cudaEventCreate(&t1);
        cudaEventRecord(t0, c.stream);
        float loss = 0.0f;
        s = cdf::train(c, tx, tt, tn_eff, 300, params, wbf, &loss);
        cudaEventRecord(t1, c.stream);
        cudaEventSynchronize(t1);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, t0, t1);
        cudaEventDestroy(t0);
        cudaEventDestroy(t1);
        if (s != CAPSSA_OK) return s;
        c.stats.train_ms = ms;
        c.stats.model_loss = loss;
        c.stats.train_samples = tn_eff;
    }
    // 4. partition of every suffix
    CAPSSA_CUDA(c, cudaMemsetAsync(sizes, 0, (size_t)p * 8 + 32, c.stream));
    const size_t smem = (size_t)n_piv * 4 + (size_t)p * 4 + (learned ? cdf::kParams * 2 + 16 : 0);
    const unsigned grid = std::min<unsigned>(grid_for(m, 256), (unsigned)c.sm_count * 4);
    if (learned)
        cudaFuncSetAttribute(partition_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
    else
        cudaFuncSetAttribute(partition_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
    kt.mark(c.stream, "samples+pivots+model");
    cudaEvent_t q0, q1;
    cudaEventCreate(&q0);
    cudaEventCreate(&q1);
    cudaEventRecord(q0, c.stream);
    // the full text in SA order, or the sorted subset
    const uint32_t *items = subset ? sorted : nullptr;
    const uint32_t *psa = subset ? nullptr : sa_full;
    const uint32_t *phead = !subset && ties ? head : nullptr;
    if (learned)
        partition_kernel<true><<<grid, 256, smem, c.stream>>>(items, (uint32_t)m, P, hkey, psa,
                                                              phead, piv_key, n_piv, p, wbf,
                                                              bucket_of, sizes, pstats);
    else
        partition_kernel<false><<<grid, 256, smem, c.stream>>>(items, (uint32_t)m, P, hkey, psa,
                                                               phead, piv_key, n_piv, p, wbf,
                                                               bucket_of, sizes, pstats);
    CAPSSA_LAUNCHED(c);
    cudaEventRecord(q1, c.stream);
    int *bad = c.d_flags + 1;
    CAPSSA_CUDA(c, cudaMemsetAsync(bad, 0, 4, c.stream));
    partition_check_kernel<<<grid_for(m, 256), 256, 0, c.stream>>>(bucket_of, nullptr,
                                                                   (uint32_t)m, bad);
    CAPSSA_LAUNCHED(c);
    std::vector<unsigned long long> h_sizes((size_t)p + 4);
    std::vector<uint32_t> h_piv(n_piv + 1);
    CAPSSA_CUDA(c, cudaMemcpyAsync(h_sizes.data(), sizes, ((size_t)p + 4) * 8,
                                   cudaMemcpyDeviceToHost, c.stream));
    if (n_piv)
        CAPSSA_CUDA(c, cudaMemcpyAsync(h_piv.data(), piv_pos, (size_t)n_piv * 4,
                                       cudaMemcpyDeviceToHost, c.stream));
    int h_bad = 0;
    CAPSSA_CUDA(c, cudaMemcpyAsync(&h_bad, bad, 4, cudaMemcpyDeviceToHost, c.stream));
    kt.mark(c.stream, "partition+check");
    kt.print();
    CAPSSA_CUDA(c, cudaStreamSynchronize(c.stream));
    float pms = 0.0f;
    cudaEventElapsedTime(&pms, q0, q1);
    cudaEventDestroy(q0);
    cudaEventDestroy(q1);
    if (h_bad) return set_err(c, CAPSSA_ECUDA, "partition disagrees with the sorted order");
    c.stats.partition_ms = pms;
    c.stats.partitions = p;
    c.stats.partition_probes = h_sizes[p];
    c.stats.mispredicted = h_sizes[p + 1];
    uint64_t mx = 0;
    for (uint32_t j = 0; j < p; j++) mx = std::max<uint64_t>(mx, h_sizes[j]);
    c.stats.max_partition = mx;
    if (a.part_sizes)
        for (uint32_t j = 0; j < p; j++) a.part_sizes[j] = h_sizes[j];
    if (a.part_pivots)
        for (uint32_t j = 0; j < n_piv; j++) a.part_pivots[j] = h_piv[j];
    return CAPSSA_OK;
}

// Plan outputs and statistics of a partition-first sort: pivots, bucket
// sizes, comparisons per suffix and mispredictions (learned model).
inline capssa_status pf_report(Ctx &c, const EngineArgs &a, const PfRun &pf) {
    const uint32_t p = pf.p;
    std::vector<unsigned long long> h_sizes((size_t)p + 2);
    std::vector<uint32_t> h_piv(p);
    CAPSSA_CUDA(c, cudaMemcpyAsync(h_sizes.data(), pf.d_sizes, ((size_t)p + 2) * 8,
                                   cudaMemcpyDeviceToHost, c.stream));
    CAPSSA_CUDA(c, cudaMemcpyAsync(h_piv.data(), pf.d_pivots, (size_t)(p - 1) * 4,
                                   cudaMemcpyDeviceToHost, c.stream));
    CAPSSA_CUDA(c, cudaStreamSynchronize(c.stream));
    c.stats.partitions = p;
    c.stats.partition_probes = h_sizes[p];
    c.stats.mispredicted = h_sizes[p + 1];
    uint64_t mx = 0;
    for (uint32_t j = 0; j < p; j++) mx = std::max<uint64_t>(mx, h_sizes[j]);
    c.stats.max_partition = mx;
    if (a.part_sizes)
        for (uint32_t j = 0; j < p; j++) a.part_sizes[j] = h_sizes[j];
    if (a.part_pivots)
        for (uint32_t j = 0; j + 1 < p; j++) a.part_pivots[j] = h_piv[j];
    return CAPSSA_OK;
}

// Subsets far smaller than the text (m * kSparseRatio <= n) are sorted on
// their own: the distinct chosen positions become records of their own and
// go through the same radix sort and refinement, so the work is O(m) plus
// one n / 8-byte bitmap.  Repeated positions, deep ties (a group needing
// rank doubling) or any other case leave *res null and the caller sorts the
// whole text instead.  On success *res holds the m positions in order (the
// empty suffix n first under ShorterFirst, last under LongerFirst).
constexpr uint64_t kSparseRatio = 8;

template <typename S>
capssa_status sparse_subset(Ctx &c, const EngineArgs &a, const uint32_t **res) {
    using namespace eng;
    *res = nullptr;
    const uint64_t n = a.n, m = a.m;
    const int lf = a.lim.longer_first;
    const uint64_t nw = n / 32 + 1;
    uint32_t *bits = const_cast<uint32_t *>(a.keep_bits);
    unsigned long long n_empty = 0;
    if (!bits) {
        bits = (uint32_t *)ws_get(c, WS_KEEP, nw * 4 + 64);
        if (!bits) return set_err(c, CAPSSA_ENOMEM, "subset bitmap");
        int *fl = c.d_flags + 1;  // [0] beyond the end, [1] repeated
        unsigned long long *cnt = (unsigned long long *)(c.d_flags + 4);
        CAPSSA_CUDA(c, cudaMemsetAsync(fl, 0, 12 + 8, c.stream));
        CAPSSA_CUDA(c, cudaMemsetAsync(bits, 0, nw * 4, c.stream));
        const unsigned gb = std::min<unsigned>(grid_for(m, 256), (unsigned)c.sm_count * 8);
        if (a.pos_bytes == 4)
            subset_bits_kernel<uint32_t><<<gb, 256, 0, c.stream>>>((const uint32_t *)a.positions, m,
                                                                   n, bits, fl, cnt);
        else
            subset_bits_kernel<uint64_t><<<gb, 256, 0, c.stream>>>((const uint64_t *)a.positions, m,
                                                                   n, bits, fl, cnt);
        CAPSSA_LAUNCHED(c);
        int *h = (int *)c.h_scratch;
        unsigned long long *h_cnt = (unsigned long long *)c.h_scratch + 2;
        CAPSSA_CUDA(c, cudaMemcpyAsync(h, fl, 8, cudaMemcpyDeviceToHost, c.stream));
        CAPSSA_CUDA(c, cudaMemcpyAsync(h_cnt, cnt, 8, cudaMemcpyDeviceToHost, c.stream));
        CAPSSA_CUDA(c, cudaStreamSynchronize(c.stream));
        if (h[0]) return set_err(c, CAPSSA_EINVAL, "a position lies beyond the end of the text");
        if (h[1] || *h_cnt > 1) return CAPSSA_OK;  // repeated positions: the whole-text path
        n_empty = *h_cnt;
    }
    const uint64_t count = m - n_empty;  // chosen positions below n
    if (count == 0) return CAPSSA_OK;
    // the chosen positions, ascending (a stable sort then keeps every tie
    // class in ascending position, as the whole-text path does)
    uint32_t *wc = (uint32_t *)ws_get(c, WS_MISC, nw * 4 + 64);
    uint32_t *pos = (uint32_t *)ws_get(c, WS_MISC2, count * 4 + 64);
    if (!wc || !pos) return set_err(c, CAPSSA_ENOMEM, "subset positions");
    bits_popc_kernel<<<grid_for(nw, 256), 256, 0, c.stream>>>(bits, nw, wc);
    CAPSSA_LAUNCHED(c);
    capssa_status s = scan_u32(c, wc, wc, nw, /*max_op=*/false, /*inclusive=*/true);
    if (s != CAPSSA_OK) return s;
    bits_expand_kernel<<<grid_for(nw, 256), 256, 0, c.stream>>>(bits, nw, wc, pos);
    CAPSSA_LAUNCHED(c);
    SparseRun sp;
    sp.pos = pos;
    sp.m = count;
    uint32_t *sa = nullptr;
    Packed P{};
    s = core_sort<S>(c, a, &sa, &P, nullptr, &sp);
    if (s != CAPSSA_OK || sp.fell_back) return s;
    uint32_t *sv = (uint32_t *)ws_get(c, WS_MISC3, (size_t)m * 8 + 64);
    if (!sv) return set_err(c, CAPSSA_ENOMEM, "subset workspace");
    const uint64_t off = (n_empty && !lf) ? 1 : 0;
    CAPSSA_CUDA(c, cudaMemcpyAsync(sv + off, sa, count * 4, cudaMemcpyDeviceToDevice, c.stream));
    if (n_empty) {
        uint32_t *hv = (uint32_t *)c.h_scratch;
        *hv = (uint32_t)n;
        CAPSSA_CUDA(c, cudaMemcpyAsync(sv + (lf ? m - 1 : 0), hv, 4, cudaMemcpyHostToDevice,
                                       c.stream));
        CAPSSA_CUDA(c, cudaStreamSynchronize(c.stream));  // the pinned word is reused
    }
    c.stats.sparse_subset = 1;
    *res = sv;
    return CAPSSA_OK;
}

template <typename S>
capssa_status engine_build_t(Ctx &c, const EngineArgs &a) {
    using namespace eng;
    const uint64_t n = a.n;
    const int lf = a.lim.longer_first;
    const bool subset = a.positions != nullptr || a.keep_bits != nullptr;
    const uint64_t m = subset ? a.m : n;
    c.stats.n_suffixes = m;
    if (n > 0xFFFFFFFEull) return set_err(c, CAPSSA_EUNSUPPORTED, "texts of 2^32-1 or more symbols");
    if (m > 0xFFFFFFFFull) return set_err(c, CAPSSA_EUNSUPPORTED, "more than 2^32-1 positions");
    if (m == 0) return CAPSSA_OK;
    const bool bounded = a.max_ctx != CAPSSA_UNBOUNDED && a.max_ctx < n;

    uint32_t *sa = nullptr;
    eng::Packed P{};
    // a small subset sorted on its own
    const uint32_t *sparse_res = nullptr;
    if (subset && !a.part_p && !bounded && n > 0 && m * kSparseRatio <= n) {
        capssa_status s = sparse_subset<S>(c, a, &sparse_res);
        if (s != CAPSSA_OK) return s;
    }
    // the sample sort with its partition ahead of the sort (whole texts,
    // unbounded context, at least two buckets)
    bool part_done = false;
    if (n > 0 && !subset && !bounded && a.part_p >= 2 && a.part_first && a.part_p <= 8192) {
        PfRun pf;
        pf.p = a.part_p;
        pf.learned = a.part_mode == CAPSSA_PARTITION_LEARNED;
        pf.bisect = a.part_mode == CAPSSA_PARTITION_BISECT;
        capssa_status s = core_sort<S>(c, a, &sa, &P, &pf);
        if (s != CAPSSA_OK) return s;
        if (!pf.fell_back) {
            s = pf_report(c, a, pf);
            if (s != CAPSSA_OK) return s;
            part_done = true;
        }
    }
    if (n > 0 && !part_done && !sparse_res) {
        capssa_status s = core_sort<S>(c, a, &sa, &P);
        if (s != CAPSSA_OK) return s;
        if (bounded) {
            s = bounded_pass<S>(c, a, sa);
            if (s != CAPSSA_OK) return s;
        }
    }
    if (!subset && a.part_p && !part_done) {
        capssa_status s = partition_phase<S>(c, a, P, sa, sa, n);
        if (s != CAPSSA_OK) return s;
    }
    FinishTimer ft(c);
    // the reference's order inside the comparator's tie classes (only
    // SegmentedText under ShorterFirst has any); `key` marks the classes when
    // the full order's group heads line up with the output
    auto tie_pass = [&](const uint32_t *key) -> capssa_status {
        if (!a.tie_ref || !a.lim.segmented || lf || a.part_p || a.seg_major || a.keep_bits)
            return CAPSSA_OK;
        TieArgs t{};
        t.text = a.text;
        t.sym_bytes = a.sym_bytes;
        t.lim = a.lim;
        t.max_ctx = a.max_ctx;
        t.out = a.out_sa;
        t.out_bytes = a.out_bytes;
        t.m = m;
        t.key = key;
        t.positions = a.positions;
        t.pos_bytes = a.pos_bytes;
        cudaEventRecord(c.pev[6], c.stream);
        capssa_status s0 = reference_tie_order(c, t);
        if (s0 != CAPSSA_OK) return s0;
        cudaEventRecord(c.pev[7], c.stream);
        CAPSSA_CUDA(c, cudaEventSynchronize(c.pev[7]));
        float ms = 0;
        cudaEventElapsedTime(&ms, c.pev[6], c.pev[7]);
        c.stats.tie_order_ms = ms;
        return CAPSSA_OK;
    };
    if (!subset) {
        if (a.out_bytes == 4) {
            if (sa != a.out_sa)
                CAPSSA_CUDA(c, cudaMemcpyAsync(a.out_sa, sa, n * 4, cudaMemcpyDeviceToDevice,
                                               c.stream));
        } else {
            widen_kernel<uint64_t><<<grid_for(n, 256), 256, 0,
                                     c.stream>>>(sa, (uint64_t *)a.out_sa, n);
            CAPSSA_LAUNCHED(c);
        }
        if (a.out_lcp) {
            capssa_status s = lcp_array_sa(c, a.text, a.sym_bytes, n, a.lim, a.max_ctx, sa, n,
                                           a.out_lcp, a.out_bytes);
            if (s != CAPSSA_OK) return s;
        }
        // last: it reuses the sort's buffers (reordering inside a class
        // leaves the LCP array as it is); the refinement's final group heads
        // mark the classes of an unbounded sort
        return tie_pass(bounded ? nullptr : (const uint32_t *)c.bufs[WS_GROUPS_B]);
    }
    // subset: order the requested positions by their index in the full SA
    uint32_t *sv = (uint32_t *)ws_get(c, WS_MISC3, (size_t)m * 8 + 64);
    if (!sv) return set_err(c, CAPSSA_ENOMEM, "subset workspace");
    uint32_t *sv_b = sv + m;
    const unsigned gm = grid_for(m, 256);
    const uint32_t *res = sparse_res;
    if (a.keep_bits && a.part_p) return set_err(c, CAPSSA_EINVAL, "no partition plan for a kept-bit set");
    if (!res && !a.part_p && n > 0) {
        // distinct positions: mark them in a bitmap (L2-sized: n / 8 bytes)
        // and compact the full order, instead of sorting them by rank
        uint32_t *bits = (uint32_t *)ws_get(c, WS_KEYS_A, (size_t)n * 8);
        if (!bits) return set_err(c, CAPSSA_ENOMEM, "subset workspace");
        unsigned long long n_empty = 0;
        bool distinct = true;
        if (a.keep_bits) {
            bits = const_cast<uint32_t *>(a.keep_bits);
        } else {
            int *fl = c.d_flags + 1;  // [0] beyond the end, [1] repeated
            unsigned long long *cnt = (unsigned long long *)(c.d_flags + 4);
            CAPSSA_CUDA(c, cudaMemsetAsync(fl, 0, 12 + 8, c.stream));
            CAPSSA_CUDA(c, cudaMemsetAsync(bits, 0, ((size_t)n / 32 + 1) * 4, c.stream));
            const unsigned gb = std::min<unsigned>(grid_for(m, 256), (unsigned)c.sm_count * 8);
            if (a.pos_bytes == 4)
                subset_bits_kernel<uint32_t><<<gb, 256, 0, c.stream>>>(
                    (const uint32_t *)a.positions, m, n, bits, fl, cnt);
            else
                subset_bits_kernel<uint64_t><<<gb, 256, 0, c.stream>>>(
                    (const uint64_t *)a.positions, m, n, bits, fl, cnt);
            CAPSSA_LAUNCHED(c);
            int *h = (int *)c.h_scratch;
            unsigned long long *h_cnt = (unsigned long long *)c.h_scratch + 2;
            CAPSSA_CUDA(c, cudaMemcpyAsync(h, fl, 8, cudaMemcpyDeviceToHost, c.stream));
            CAPSSA_CUDA(c, cudaMemcpyAsync(h_cnt, cnt, 8, cudaMemcpyDeviceToHost, c.stream));
            CAPSSA_CUDA(c, cudaStreamSynchronize(c.stream));
            if (h[0]) return set_err(c, CAPSSA_EINVAL, "a position lies beyond the end of the text");
            n_empty = *h_cnt;
            distinct = !h[1];
        }
        if (distinct && n_empty <= 1) {
            // one pass: the requested suffixes of the full order, in order,
            // straight into the output (widened on the way) unless an LCP
            // array is wanted too; the empty suffix n sorts first
            // (ShorterFirst) or last
            const uint32_t off = (n_empty && !lf) ? 1u : 0u;
            const bool direct = !a.out_lcp;
            void *dst = direct ? a.out_sa : (void *)sv;
            const int db = direct ? a.out_bytes : 4;
            capssa_status s0 = select_bits(c, sa, n, bits, off, dst, db);
            if (s0 != CAPSSA_OK) return s0;
            if (n_empty) {
                uint64_t *hv = (uint64_t *)c.h_scratch;
                *hv = n;  // little-endian: the low 4 bytes are the u32 value
                CAPSSA_CUDA(c, cudaMemcpyAsync((char *)dst + (lf ? m - 1 : 0) * (uint64_t)db, hv,
                                               db, cudaMemcpyHostToDevice, c.stream));
                CAPSSA_CUDA(c, cudaStreamSynchronize(c.stream));  // the pinned word is reused
            }
            if (direct) return tie_pass(nullptr);
            res = sv;
        }
    }
    if (!res) {
        uint32_t *isa = (uint32_t *)ws_get(c, WS_RANK, (size_t)n * 4 + 64);
        uint64_t *sk_a = (uint64_t *)ws_get(c, WS_MISC, (size_t)m * 8 + 64);
        uint64_t *sk_b = (uint64_t *)ws_get(c, WS_MISC2, (size_t)m * 8 + 64);
        if (!isa || !sk_a || !sk_b) return set_err(c, CAPSSA_ENOMEM, "subset workspace");
        if (n > 0) {
            isa_kernel<<<grid_for(n, 256), 256, 0, c.stream>>>(
                sa, (uint32_t)n, isa);
            CAPSSA_LAUNCHED(c);
        }
        int *bad = c.d_flags + 1;
        CAPSSA_CUDA(c, cudaMemsetAsync(bad, 0, 4, c.stream));
        if (a.pos_bytes == 4)
            subset_isa_key_kernel<uint32_t><<<gm, 256, 0, c.stream>>>(
                (const uint32_t *)a.positions, m, n, isa, lf, sk_a, sv, bad);
        else
            subset_isa_key_kernel<uint64_t><<<gm, 256, 0, c.stream>>>(
                (const uint64_t *)a.positions, m, n, isa, lf, sk_a, sv, bad);
        CAPSSA_LAUNCHED(c);
        int *h_bad = (int *)c.h_scratch;
        CAPSSA_CUDA(c, cudaMemcpyAsync(h_bad, bad, 4, cudaMemcpyDeviceToHost, c.stream));
        CAPSSA_CUDA(c, cudaStreamSynchronize(c.stream));
        if (*h_bad) return set_err(c, CAPSSA_EINVAL, "a position lies beyond the end of the text");
        bool in_b = false;
        capssa_status s = radix::sort_pairs(c, sk_a, sv, sk_b, sv_b, (uint32_t)m, 0, bits_for(n + 1),
                                            false, 0, &in_b);
        if (s != CAPSSA_OK) return s;
        res = in_b ? sv_b : sv;
    }
    capssa_status s = CAPSSA_OK;
    if (a.part_p) {
        s = partition_phase<S>(c, a, P, sa, res, m);
        if (s != CAPSSA_OK) return s;
    }
    if (a.out_bytes == 4) {
        CAPSSA_CUDA(c, cudaMemcpyAsync(a.out_sa, res, m * 4, cudaMemcpyDeviceToDevice, c.stream));
    } else {
        widen_kernel<uint64_t><<<gm, 256, 0, c.stream>>>(res, (uint64_t *)a.out_sa, m);
        CAPSSA_LAUNCHED(c);
    }
    if (a.out_lcp) {
        s = lcp_array_sa(c, a.text, a.sym_bytes, n, a.lim, a.max_ctx, res, m, a.out_lcp,
                         a.out_bytes);
        if (s != CAPSSA_OK) return s;
    }
    return tie_pass(nullptr);
}

}  // namespace
}  // namespace capssa
