// radix.cu — onesweep LSD radix sort of (u64 key, u32 value) pairs.
//
// GB300 counterpart of the `sort_unstable_by_key` inside seed_subarray
// (src/pack.rs:271) and of every global reordering the suffix sort needs.
// The sort is stable, so equal keys keep input order.
//
// Per 8-bit digit pass one kernel reads each (key, value) once and writes it
// once (24 B per pair of HBM traffic): a block claims the next tile through
// an atomic counter, ranks its keys by digit in shared memory with a
// stable warp-level multisplit (ballots + shared atomics), publishes its per-digit counts
// and learns its global offsets by decoupled look-back over the tiles
// before it, then writes each digit run contiguously.  One up-front kernel
// builds the histograms of every pass from a single read of the keys;
// passes whose digit is constant are skipped.
//
// Every look-back wait is bounded (kSpinLimit polls); on expiry the kernel
// records DEV_LOOKBACK_TIMEOUT and the host call fails with CAPSSA_ETIMEOUT.
#include <algorithm>

#include "common.cuh"
#include "radix.cuh"

namespace capssa {
namespace radix {

constexpr int kMinBlocks = 3;  // resident blocks per SM the register budget is sized for
constexpr int kRadix = 256;
constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr unsigned long long kFlagA = 1ull << 62;
constexpr unsigned long long kFlagP = 2ull << 62;
constexpr unsigned long long kValMask = (1ull << 62) - 1;

static_assert(kThreads == kRadix, "one thread per digit in the per-tile phase");

__global__ void __launch_bounds__(kThreads) hist_kernel(const uint64_t *__restrict__ keys,
                                                        uint32_t n, int begin_bit,
                                                        int n_passes,
                                                        uint32_t *__restrict__ counts) {
    __shared__ uint32_t sh[kMaxPasses * kRadix];
    for (int i = threadIdx.x; i < kMaxPasses * kRadix; i += blockDim.x) sh[i] = 0;
    __syncthreads();
    // whole warps step together (the digit match needs all 32 lanes);
    // lanes past the end carry label 256, which no counter has
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t gwarp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t wstride = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t base = gwarp * 32; base < n; base += wstride * 32) {
        const uint64_t idx = base + lane;
        const bool valid = idx < n;
        const uint64_t k = valid ? keys[idx] : 0;
        for (int p = 0; p < n_passes; p++) {
            const uint32_t d = valid ? (uint32_t)(k >> (begin_bit + 8 * p)) & 255u : 256u;
            const unsigned peers = warp_match_bits<9>(d);
            if (valid && lane == (uint32_t)(31 - __clz(peers)))
                atomicAdd(&sh[p * kRadix + d], (uint32_t)__popc(peers));
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n_passes * kRadix; i += blockDim.x)
        if (sh[i]) atomicAdd(&counts[i], sh[i]);
}

__device__ __forceinline__ unsigned long long ld_volatile_u64(const unsigned long long *p) {
    return *(const volatile unsigned long long *)p;
}
__device__ __forceinline__ void st_volatile_u64(unsigned long long *p, unsigned long long v) {
    *(volatile unsigned long long *)p = v;
}

// Decoupled look-back for digit dg of `tile`: the sum of the counts of
// every earlier tile, from their published aggregates (A) back to the
// nearest inclusive prefix (P).  kLookBatch predecessors are read per round trip;
// a predecessor that has published nothing yet is polled again (bounded by
// kSpinLimit polls, then DEV_LOOKBACK_TIMEOUT).
constexpr int kLookBatch = 4;

__device__ __forceinline__ uint64_t lookback(const unsigned long long *status, uint32_t tile,
                                             uint32_t dg, int *err) {
    uint64_t excl = 0;
    int64_t t = (int64_t)tile - 1;
    uint32_t spins = 0;
    while (t >= 0) {
        unsigned long long sv[kLookBatch];
#pragma unroll
        for (int q = 0; q < kLookBatch; q++)
            sv[q] = t - q >= 0 ? ld_volatile_u64(status + (size_t)(t - q) * kRadix + dg) : kFlagP;
        int used = 0;
        bool found = false, stalled = false;
#pragma unroll
        for (int q = 0; q < kLookBatch; q++) {
            if (!found && !stalled) {
                const unsigned long long flag = sv[q] & ~kValMask;
                if (flag == 0) {
                    stalled = true;
                } else {
                    excl += sv[q] & kValMask;
                    used++;
                    if (flag == kFlagP) found = true;
                }
            }
        }
        if (found) break;
        t -= used;
        if (stalled) {
            if (++spins > kSpinLimit) {
                atomicCAS(err, DEV_OK, DEV_LOOKBACK_TIMEOUT);
                break;
            }
            __nanosleep(32);
        }
    }
    return excl;
}

// MODE: kPairs (values read), kGenVals (value = val_base + index), kKeysOnly.
constexpr int kPairs = 0, kGenVals = 1, kKeysOnly = 2;

// IT records per thread (the tile is 256 * IT records): a template
// parameter so that the tuner below can pick the shape per workload.
template <int MODE, int IT>
__global__ void __launch_bounds__(kThreads, kMinBlocks)
    onesweep_kernel(const uint64_t *__restrict__ keys_in, const uint32_t *__restrict__ vals_in,
                    uint64_t *__restrict__ keys_out, uint32_t *__restrict__ vals_out,
                    uint32_t n, int shift, const uint32_t *__restrict__ digit_offsets,
                    unsigned long long *__restrict__ status, uint32_t *__restrict__ tile_counter,
                    int *__restrict__ err, uint32_t val_base) {
    extern __shared__ __align__(16) unsigned char smem[];
    constexpr bool kVals = MODE != kKeysOnly;
    constexpr int TILE = kThreads * IT;
    uint64_t *s_keys = reinterpret_cast<uint64_t *>(smem);
    uint32_t *s_vals = reinterpret_cast<uint32_t *>(s_keys + TILE);
    uint32_t *s_whist = s_vals + (kVals ? TILE : 0);  // kWarps * kRadix
    uint32_t *s_lstart = s_whist + kWarps * kRadix;  // kRadix
    uint32_t *s_gbase = s_lstart + kRadix;           // kRadix
    uint32_t *s_scan = s_gbase + kRadix;             // kWarps
    __shared__ uint32_t s_tile;

    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    if (tid == 0) s_tile = atomicAdd(tile_counter, 1u);
    for (int i = tid; i < kWarps * kRadix; i += kThreads) s_whist[i] = 0;
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t base = tile * (uint32_t)TILE;
    const uint32_t valid = (n - base) < (uint32_t)TILE ? (n - base) : (uint32_t)TILE;

    uint64_t k[IT];
    uint32_t v[IT];
    uint32_t d[IT];
    uint32_t r[IT];
    const uint32_t wbase = base + warp * 32 * IT;
#pragma unroll
    for (int j = 0; j < IT; j++) {
        uint32_t idx = wbase + j * 32 + lane;
        if (idx < n) {
            k[j] = keys_in[idx];
            if (MODE == kGenVals) v[j] = val_base + idx;
            if (MODE == kPairs) v[j] = vals_in[idx];
        } else {
            k[j] = ~0ull;  // past the end: digit 255, ranked after every valid key
            v[j] = 0;
        }
        d[j] = (uint32_t)(k[j] >> shift) & 255u;
    }
    // warp-level multisplit: rank of each item among equal digits of this warp
    uint32_t *wh = s_whist + warp * kRadix;
    const unsigned lt_mask = (1u << lane) - 1u;
#pragma unroll
    for (int j = 0; j < IT; j++) {
        const unsigned peers = warp_match_bits<8>(d[j]);
        r[j] = warp_rank_digit(wh, d[j], peers, lt_mask, lane);
    }
    __syncthreads();

    // thread `tid` owns digit `tid`: warp prefixes, tile total, look-back
    const uint32_t dg = (uint32_t)tid;
    uint32_t total = 0;
#pragma unroll
    for (int w = 0; w < kWarps; w++) {
        uint32_t c = s_whist[w * kRadix + dg];
        s_whist[w * kRadix + dg] = total;
        total += c;
    }
    uint32_t counted = total;
    if (dg == 255) counted -= (uint32_t)TILE - valid;  // drop the padding items
    unsigned long long *st = status + (size_t)tile * kRadix + dg;
    uint64_t excl = 0;
    if (tile == 0) {
        st_volatile_u64(st, kFlagP | counted);
    } else {
        st_volatile_u64(st, kFlagA | counted);
        excl = lookback(status, tile, dg, err);
        st_volatile_u64(st, kFlagP | (excl + counted));
    }
    s_gbase[dg] = digit_offsets[dg] + (uint32_t)excl;

    // block exclusive scan of the per-digit totals -> local start of each digit
    uint32_t x = total;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_scan[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < kWarps ? s_scan[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < kWarps) s_scan[lane] = w;
    }
    __syncthreads();
    const uint32_t lstart = x - total + (warp > 0 ? s_scan[warp - 1] : 0);
    s_lstart[dg] = lstart;
    // from here s_gbase holds global start - local start: one lookup per
    // record in the write-out
    s_gbase[dg] -= lstart;
    __syncthreads();

#pragma unroll
    for (int j = 0; j < IT; j++) {
        uint32_t pos = s_lstart[d[j]] + wh[d[j]] + r[j];
        s_keys[pos] = k[j];
        if (kVals) s_vals[pos] = v[j];
    }
    __syncthreads();
    for (uint32_t i = tid; i < valid; i += kThreads) {
        uint64_t key = s_keys[i];
        uint32_t dd = (uint32_t)(key >> shift) & 255u;
        uint32_t out = s_gbase[dd] + i;
        if (out < n) {  // only false after a timed-out look-back (flagged)
            keys_out[out] = key;
            if (kVals) vals_out[out] = s_vals[i];
        }
    }
}

__global__ void iota_kernel(uint32_t *out, uint32_t n, uint32_t base) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[i] = base + i;
}

static size_t pass_smem(bool vals, int items) {
    const size_t tile = (size_t)kThreads * items;
    return tile * 8 + (vals ? tile * 4 : 0) + (size_t)kWarps * kRadix * 4 +
           (size_t)kRadix * 4 * 2 + (size_t)kWarps * 4;
}

// Tile shapes the tuner tries, per mode (records per thread).
constexpr int kKeyShapes[3] = {16, 20, 24};
constexpr int kPairShapes[2] = {12, 16};

template <int MODE, int IT>
void launch_shape(Ctx &c, const uint64_t *ki, const uint32_t *vi, uint64_t *ko, uint32_t *vo,
                  uint32_t n, int shift, const uint32_t *offsets, unsigned long long *status,
                  uint32_t *tile_counter, uint32_t val_base) {
    const size_t sm = pass_smem(MODE != kKeysOnly, IT);
    // function attributes are per device: set on the context's device each time
    cudaFuncSetAttribute(onesweep_kernel<MODE, IT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sm);
    const unsigned tiles = (n + kThreads * IT - 1) / (kThreads * IT);
    onesweep_kernel<MODE, IT><<<tiles, kThreads, sm, c.stream>>>(
        ki, vi, ko, vo, n, shift, offsets, status, tile_counter, c.d_flags, val_base);
}

void launch_pass(Ctx &c, int mode, int items, const uint64_t *ki, const uint32_t *vi,
                 uint64_t *ko, uint32_t *vo, uint32_t n, int shift, const uint32_t *offsets,
                 unsigned long long *status, uint32_t *tile_counter, uint32_t val_base) {
#define CAPSSA_SHAPE(M, I)                                                                    \
    if (mode == M && items == I)                                                              \
        return launch_shape<M, I>(c, ki, vi, ko, vo, n, shift, offsets, status, tile_counter, \
                                  val_base);
    CAPSSA_SHAPE(kKeysOnly, 16) CAPSSA_SHAPE(kKeysOnly, 20) CAPSSA_SHAPE(kKeysOnly, 24)
    CAPSSA_SHAPE(kPairs, 12) CAPSSA_SHAPE(kPairs, 16)
    CAPSSA_SHAPE(kGenVals, 12) CAPSSA_SHAPE(kGenVals, 16)
#undef CAPSSA_SHAPE
}

uint32_t *hist_buffer(Ctx &c) {
    return (uint32_t *)ws_get(c, WS_RADIX_HIST, (kMaxPasses + 1) * kRadix * 4 + 64);
}

namespace {

capssa_status sort_impl(Ctx &c, uint64_t *keys_a, uint32_t *vals_a, uint64_t *keys_b,
                        uint32_t *vals_b, uint32_t n, int begin_bit, int end_bit, bool gen_vals,
                        uint32_t val_base, bool *result_in_b, int *passes_run, bool hist_ready) {
    const bool keys_only = vals_a == nullptr;
    *result_in_b = false;
    if (passes_run) *passes_run = 0;
    if (n == 0) return CAPSSA_OK;
    int n_passes = (end_bit - begin_bit + 7) / 8;
    if (n_passes > kMaxPasses) return set_err(c, CAPSSA_EINVAL, "radix: too many passes");
    if (n_passes <= 0) {
        if (gen_vals) {
            iota_kernel<<<grid_for(n, 256, 4096), 256, 0, c.stream>>>(vals_a, n, val_base);
            CAPSSA_LAUNCHED(c);
        }
        return CAPSSA_OK;
    }
    uint32_t *counts = hist_buffer(c);
    // status words for the smallest tile any shape uses
    const uint32_t min_tile = (uint32_t)kThreads * 12;
    uint32_t n_tiles = (n + min_tile - 1) / min_tile;
    unsigned long long *status = (unsigned long long *)ws_get(
        c, WS_RADIX_STATUS, (size_t)n_tiles * kRadix * sizeof(unsigned long long));
    if (!counts || !status) return set_err(c, CAPSSA_ENOMEM, "radix workspace");
    uint32_t *offsets = counts + kMaxPasses * kRadix;  // 256 entries
    uint32_t *tile_counter = offsets + kRadix;

    if (!hist_ready) {
        CAPSSA_CUDA(c, cudaMemsetAsync(counts, 0, kMaxPasses * kRadix * 4, c.stream));
        hist_kernel<<<std::min<unsigned>(grid_for(n, kThreads), (unsigned)c.sm_count * 8),
                      kThreads, 0, c.stream>>>(keys_a, n, begin_bit, n_passes, counts);
        CAPSSA_LAUNCHED(c);
    }
    uint32_t *h = (uint32_t *)c.h_scratch;  // pinned, >= 8 * 256 * 4 bytes
    CAPSSA_CUDA(c, cudaMemcpyAsync(h, counts, n_passes * kRadix * 4, cudaMemcpyDeviceToHost,
                                   c.stream));
    CAPSSA_CUDA(c, cudaStreamSynchronize(c.stream));

    // per-pass exclusive offsets live in the pinned scratch after the counts
    uint32_t *h_off = h + kMaxPasses * kRadix;
    bool in_b = false;
    bool vals_pending = gen_vals;
    for (int p = 0; p < n_passes; p++) {
        uint32_t *cp = h + p * kRadix;
        bool trivial = false;
        for (int i = 0; i < kRadix; i++)
            if (cp[i] == n) trivial = true;
        if (trivial) continue;
        uint32_t acc = 0;
        for (int i = 0; i < kRadix; i++) {
            h_off[p * kRadix + i] = acc;
            acc += cp[i];
        }
        CAPSSA_CUDA(c, cudaMemcpyAsync(offsets, h_off + p * kRadix, kRadix * 4,
                                       cudaMemcpyHostToDevice, c.stream));
        const uint64_t *ki = in_b ? keys_b : keys_a;
        const uint32_t *vi = in_b ? vals_b : vals_a;
        uint64_t *ko = in_b ? keys_a : keys_b;
        uint32_t *vo = in_b ? vals_a : vals_b;
        const int mode = keys_only ? kKeysOnly : (vals_pending ? kGenVals : kPairs);
        const int cls = mode == kKeysOnly ? 1 : 0;
        int lg = 0;
        while ((1u << (lg + 1)) <= n && lg < 31) lg++;
        int &shape = c.radix_shape[cls][lg];
        if (shape == 0) {
            // autotuner: the first large pass of this kind and size class runs
            // every candidate shape on the same input (each writes the same
            // correct output) and keeps the fastest; small sorts take the
            // default
            const int *cand = cls ? kKeyShapes : kPairShapes;
            const int nc = cls ? 3 : 2;
            shape = cls ? 24 : 16;
            if (n >= (1u << 22) && c.tune_ev[0]) {
                float best = 1e30f;
                for (int q = 0; q < nc; q++) {
                    CAPSSA_CUDA(c, cudaMemsetAsync(status, 0, (size_t)n_tiles * kRadix * 8, c.stream));
                    CAPSSA_CUDA(c, cudaMemsetAsync(tile_counter, 0, 4, c.stream));
                    cudaEventRecord(c.tune_ev[0], c.stream);
                    launch_pass(c, mode, cand[q], ki, vi, ko, vo, n, begin_bit + 8 * p, offsets,
                                status, tile_counter, val_base);
                    CAPSSA_LAUNCHED(c);
                    cudaEventRecord(c.tune_ev[1], c.stream);
                    CAPSSA_CUDA(c, cudaEventSynchronize(c.tune_ev[1]));
                    float ms = 0.0f;
                    cudaEventElapsedTime(&ms, c.tune_ev[0], c.tune_ev[1]);
                    if (ms < best) {
                        best = ms;
                        shape = cand[q];
                    }
                }
            }
        }
        // status words of this shape's tiles only (the buffer is sized for the
        // smallest tile any shape uses)
        const uint64_t tile_recs = (uint64_t)kThreads * (uint64_t)shape;
        const uint64_t pass_tiles = ((uint64_t)n + tile_recs - 1) / tile_recs;
        CAPSSA_CUDA(c, cudaMemsetAsync(status, 0, (size_t)pass_tiles * kRadix * 8, c.stream));
        CAPSSA_CUDA(c, cudaMemsetAsync(tile_counter, 0, 4, c.stream));
        const bool timed = passes_run && (*passes_run) < 16;
        if (timed) cudaEventRecord(c.kev[2 * (*passes_run)], c.stream);
        c.stats.radix_items = (uint32_t)shape;
        launch_pass(c, mode, shape, ki, vi, ko, vo, n, begin_bit + 8 * p, offsets, status,
                    tile_counter, val_base);
        CAPSSA_LAUNCHED(c);
        if (timed) cudaEventRecord(c.kev[2 * (*passes_run) + 1], c.stream);
        if (passes_run) (*passes_run)++;
        vals_pending = false;
        in_b = !in_b;
        // the host-side offsets buffer is reused by the next pass only after
        // this copy has been consumed, which stream order guarantees because
        // each pass reads its own slice of h_off.
    }
    if (vals_pending && !keys_only) {
        uint32_t *dst = in_b ? vals_b : vals_a;
        iota_kernel<<<grid_for(n, 256, 4096), 256, 0, c.stream>>>(dst, n, val_base);
        CAPSSA_LAUNCHED(c);
    }
    *result_in_b = in_b;
    return CAPSSA_OK;
}

}  // namespace

capssa_status sort_pairs(Ctx &c, uint64_t *keys_a, uint32_t *vals_a, uint64_t *keys_b,
                         uint32_t *vals_b, uint32_t n, int begin_bit, int end_bit,
                         bool gen_vals, uint32_t val_base, bool *result_in_b,
                         int *passes_run, bool hist_ready) {
    if (!vals_a || !vals_b) return set_err(c, CAPSSA_EINVAL, "radix: null values");
    return sort_impl(c, keys_a, vals_a, keys_b, vals_b, n, begin_bit, end_bit, gen_vals,
                     val_base, result_in_b, passes_run, hist_ready);
}

capssa_status sort_keys(Ctx &c, uint64_t *keys_a, uint64_t *keys_b, uint32_t n, int begin_bit,
                        int end_bit, bool *result_in_b, int *passes_run, bool hist_ready) {
    return sort_impl(c, keys_a, nullptr, keys_b, nullptr, n, begin_bit, end_bit, false, 0,
                     result_in_b, passes_run, hist_ready);
}

}  // namespace radix
}  // namespace capssa
