// common.cuh — shared types of the GB300 suffix-array library.
//
// The library keeps every per-suffix array in 32-bit positions internally
// (texts up to 2^32-2 symbols), 64-bit packed prefix keys, and converts to
// the caller's index width only at the boundary.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <cstdio>
#include <cstdlib>

#include <string>
#include <vector>

#include "../../include/capssa.h"

namespace capssa {

// Device-side error codes written to Ctx::d_flags[0] (first error wins).
enum DevError : int {
    DEV_OK = 0,
    DEV_LOOKBACK_TIMEOUT = 1,  // a decoupled look-back spin hit its limit
    DEV_OVERFLOW = 2,          // a work list outgrew its capacity
};

// Spin limit for look-back waits: ~2^22 polls with a 64 ns backoff is far
// longer than any predecessor tile takes, and bounded.
constexpr uint32_t kSpinLimit = 1u << 22;

constexpr uint32_t kNoPos = 0xFFFFFFFFu;

// LimitProvider on the device: PlainText (lim = n - p) or SegmentedText
// with the reference's coarse boundary directory (src/limits.rs:194-236,
// 305-328).
struct DevLimits {
    uint64_t n;
    const uint64_t *ends;  // device, n_ends entries
    uint64_t n_ends;
    const uint32_t *dir;   // device, n_dir entries or nullptr
    uint64_t n_dir;
    uint32_t block_shift;
    int segmented;
    int longer_first;
};

__device__ __forceinline__ uint64_t first_end_after(const uint64_t *ends, uint64_t lo,
                                                    uint64_t hi, uint64_t p) {
    while (lo < hi) {
        uint64_t mid = lo + ((hi - lo) >> 1);
        if (__ldg(ends + mid) <= p)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

// Index of the segment holding position p (p < n; PlainText: 0).
__device__ __forceinline__ uint64_t dev_seg_at(const DevLimits &L, uint64_t p) {
    if (!L.segmented) return 0;
    if (L.dir) {
        uint64_t block = p >> L.block_shift;
        uint64_t lo = __ldg(L.dir + block);
        uint64_t hi = __ldg(L.dir + block + 1);
        if (hi < lo + 1) hi = lo + 1;
        if (hi > L.n_ends) hi = L.n_ends;
        return first_end_after(L.ends, lo, hi, p);
    }
    return first_end_after(L.ends, 0, L.n_ends, p);
}

// SegmentedText::lim_at / PlainText::lim_at (src/limits.rs:144-148, 305-328).
__device__ __forceinline__ uint64_t dev_lim_at(const DevLimits &L, uint64_t p) {
    if (!L.segmented) return L.n - p;
    if (L.dir && p < L.n) {
        uint64_t block = p >> L.block_shift;
        uint64_t lo = __ldg(L.dir + block);
        uint64_t hi = __ldg(L.dir + block + 1);
        if (hi < lo + 1) hi = lo + 1;
        if (hi > L.n_ends) hi = L.n_ends;
        uint64_t i = first_end_after(L.ends, lo, hi, p);
        return __ldg(L.ends + i) - p;
    }
    uint64_t i = first_end_after(L.ends, 0, L.n_ends, p);
    if (i < L.n_ends) return __ldg(L.ends + i) - p;
    return L.n - p;
}

// Lanes of the (full) warp whose BITS-bit label equals this lane's: one
// ballot per label bit, intersected.  Cheaper than the general 32-bit
// match instruction for the 8-bit digits of the radix passes.
template <int BITS>
__device__ __forceinline__ unsigned warp_match_bits(uint32_t label) {
    unsigned m = 0xffffffffu;
#pragma unroll
    for (int b = 0; b < BITS; b++) {
        const bool set = (label >> b) & 1u;
        const unsigned bal = __ballot_sync(0xffffffffu, set);
        m &= set ? bal : ~bal;
    }
    return m;
}

// Stable warp multisplit of one item per lane into per-warp digit counters
// `wh` (shared memory): returns this lane's rank among the items of its
// digit that the warp has seen so far (earlier calls, then lower lanes).
// The highest lane of each digit adds the digit's count with one shared
// atomic; a warp's atomics on one address complete in issue order, so
// successive calls need no barrier between them and pipeline.
__device__ __forceinline__ uint32_t warp_rank_digit(uint32_t *wh, uint32_t d, unsigned peers,
                                                    unsigned lt_mask, int lane) {
    const int leader = 31 - __clz(peers);
    uint32_t old = 0;
    if (lane == leader) old = atomicAdd(&wh[d], (uint32_t)__popc(peers));
    old = __shfl_sync(0xffffffffu, old, leader);
    return old + __popc(peers & lt_mask);
}

// Grow-only device buffers owned by a context, addressed by slot.
enum Slot : int {
    WS_TEXT = 0, WS_ENDS, WS_DIR, WS_POS_IN, WS_OUT, WS_OUT2,
    WS_KEYS_A, WS_KEYS_B, WS_VALS_A, WS_VALS_B,
    WS_RANK, WS_KEY2, WS_GROUPS_A, WS_GROUPS_B, WS_COUNTERS,
    WS_RADIX_STATUS, WS_RADIX_HIST, WS_SCAN, WS_CODES, WS_MISC, WS_MISC2, WS_MISC3,
    WS_PACKED, WS_CDF, WS_PART, WS_SAMPLE, WS_KEEP, WS_RUNS, WS_NSLOTS
};

struct Ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    void *bufs[WS_NSLOTS] = {};
    size_t sizes[WS_NSLOTS] = {};
    int *d_flags = nullptr;         // device error flag(s)
    uint64_t *h_scratch = nullptr;  // pinned host scratch (small readbacks)
    std::string err;
    capssa_stats stats{};
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEvent_t pev[8] = {};        // phase boundaries of one suffix sort
    cudaEvent_t kev[2 * 16] = {};   // around each radix pass of the initial sort
    int sm_count = 0;
    // radix autotuner: chosen records per thread by [packed records?][log2 n]
    // (0 = not tuned yet), and its timing events
    int radix_shape[2][33] = {};
    cudaEvent_t tune_ev[2] = {};
    // the last sort produced segment-major order (every segment contiguous)
    bool seg_major_done = false;
    uint64_t *h_emit = nullptr;     // pinned double buffer of the emit stream
    uint64_t launches = 0;
    // side streams: the independent kernels of one refinement round run
    // concurrently, forked from and joined back to `stream` by events
    static constexpr int kSide = 4;
    cudaStream_t side[kSide] = {};
    cudaEvent_t fork_ev = nullptr;
    cudaEvent_t join_ev[kSide] = {};
};

// Returns a device buffer of at least `bytes` for `slot` (nullptr on OOM).
void *ws_get(Ctx &c, int slot, size_t bytes);

// Error helpers.
capssa_status set_err(Ctx &c, capssa_status s, const std::string &msg);
capssa_status cuda_err(Ctx &c, cudaError_t e, const char *where);

#define CAPSSA_CUDA(c, expr)                                        \
    do {                                                            \
        cudaError_t _e = (expr);                                    \
        if (_e != cudaSuccess) return ::capssa::cuda_err((c), _e, #expr); \
    } while (0)

#define CAPSSA_LAUNCHED(c)                                          \
    do {                                                            \
        (c).launches++;                                             \
        cudaError_t _e = cudaGetLastError();                        \
        if (_e != cudaSuccess) return ::capssa::cuda_err((c), _e, "kernel launch"); \
    } while (0)

// Device flag check: returns CAPSSA_ETIMEOUT / CAPSSA_ENOMEM after a sync.
capssa_status check_dev_flags(Ctx &c);

inline unsigned grid_for(uint64_t n, unsigned block, unsigned cap = 1u << 30) {
    uint64_t g = (n + block - 1) / block;
    if (g == 0) g = 1;
    if (g > cap) g = cap;
    return (unsigned)g;
}

// CAPSSA_PROFILE in the environment turns on per-phase / per-round lines on
// stderr, like the reference's CAPS_SA_PROFILE profile_log
// (src/ext_mem.rs:42-51).
inline bool profile_on() {
    static const bool on = std::getenv("CAPSSA_PROFILE") != nullptr;
    return on;
}

// Per-kernel device times of one phase (a refinement round, the tie
// order), printed on one line when CAPSSA_PROFILE is set (events only then).
struct KernelTimes {
    static constexpr int kMax = 12;
    cudaEvent_t ev[kMax + 1] = {};
    const char *name[kMax] = {};
    int used = 0;
    bool on = false;
    explicit KernelTimes(bool enable) : on(enable) {
        if (on)
            for (auto &e : ev) cudaEventCreate(&e);
    }
    ~KernelTimes() {
        if (on)
            for (auto &e : ev) cudaEventDestroy(e);
    }
    void start(cudaStream_t s) {
        used = 0;
        if (on) cudaEventRecord(ev[0], s);
    }
    void mark(cudaStream_t s, const char *what) {
        if (!on || used >= kMax) return;
        name[used] = what;
        cudaEventRecord(ev[++used], s);
    }
    void print() {
        if (!on || !used) return;
        cudaEventSynchronize(ev[used]);
        std::fprintf(stderr, "capssa profile    kernels:");
        for (int i = 0; i < used; i++) {
            float ms = 0;
            cudaEventElapsedTime(&ms, ev[i], ev[i + 1]);
            std::fprintf(stderr, " %s %.3f ms", name[i], ms);
        }
        std::fprintf(stderr, "\n");
    }
};

}  // namespace capssa
