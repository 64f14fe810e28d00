// scan.cu — single-pass device-wide scan (sum or max) of u32 values with
// decoupled look-back.  Each block claims the next tile through an atomic
// counter, so every tile it waits on has already started; every wait is
// bounded and reports DEV_LOOKBACK_TIMEOUT on expiry.
#include "common.cuh"
#include "scan.cuh"

namespace capssa {

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;
constexpr unsigned long long kA = 1ull << 62, kP = 2ull << 62, kMask = (1ull << 62) - 1;

template <bool MAX>
__device__ __forceinline__ uint32_t op(uint32_t a, uint32_t b) {
    return MAX ? (a > b ? a : b) : a + b;
}

template <bool MAX, bool INCLUSIVE>
__global__ void __launch_bounds__(kScanThreads)
    scan_kernel(const uint32_t *__restrict__ in, uint32_t *__restrict__ out, uint64_t n,
                unsigned long long *__restrict__ status, uint32_t *__restrict__ counter,
                int *__restrict__ err) {
    __shared__ uint32_t s_tile;
    __shared__ uint32_t s_warp[kScanThreads / 32];
    __shared__ uint32_t s_prefix;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) s_tile = atomicAdd(counter, 1u);
    __syncthreads();
    const uint64_t tile = s_tile;
    const uint64_t base = tile * kScanTile + (uint64_t)tid * kScanItems;
    uint32_t v[kScanItems];
    uint32_t agg = 0u;
#pragma unroll
    for (int j = 0; j < kScanItems; j++) {
        uint64_t i = base + j;
        v[j] = i < n ? in[i] : 0u;
        agg = op<MAX>(agg, v[j]);
    }
    // block inclusive scan of per-thread aggregates
    uint32_t x = agg;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x = op<MAX>(x, y);
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < kScanThreads / 32 ? s_warp[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w = op<MAX>(w, y);
        }
        if (lane < kScanThreads / 32) s_warp[lane] = w;
    }
    __syncthreads();
    // exclusive prefix of this thread's items inside the tile
    uint32_t within_excl;
    {
        uint32_t prev_in_warp = __shfl_up_sync(0xffffffffu, x, 1);
        if (lane == 0) prev_in_warp = 0;
        within_excl = op<MAX>(warp > 0 ? s_warp[warp - 1] : 0u, prev_in_warp);
    }
    const uint32_t tile_total = s_warp[kScanThreads / 32 - 1];
    if (tid == 0) {
        uint64_t excl = 0;
        unsigned long long *st = status + tile;
        if (tile == 0) {
            *(volatile unsigned long long *)st = kP | tile_total;
        } else {
            *(volatile unsigned long long *)st = kA | tile_total;
            int64_t t = (int64_t)tile - 1;
            uint32_t spins = 0;
            uint32_t acc = 0;
            while (t >= 0) {
                unsigned long long s = *(volatile unsigned long long *)(status + t);
                unsigned long long f = s & ~kMask;
                if (f == 0) {
                    if (++spins > kSpinLimit) {
                        atomicCAS(err, DEV_OK, DEV_LOOKBACK_TIMEOUT);
                        break;
                    }
                    __nanosleep(64);
                    continue;
                }
                acc = op<MAX>(acc, (uint32_t)(s & kMask));
                if (f == kP) break;
                t--;
            }
            excl = acc;
            *(volatile unsigned long long *)st = kP | op<MAX>((uint32_t)excl, tile_total);
        }
        s_prefix = (uint32_t)excl;
    }
    __syncthreads();
    uint32_t run = op<MAX>(s_prefix, within_excl);
#pragma unroll
    for (int j = 0; j < kScanItems; j++) {
        uint64_t i = base + j;
        uint32_t nx = op<MAX>(run, v[j]);
        if (i < n) out[i] = INCLUSIVE ? nx : run;
        run = nx;
    }
}

// Stream compaction in one pass: the entries of sa whose bit in `bits` is
// set, in order, written to out[off ..] as OT (widened from u32 when OT is
// u64); the tile counts are chained by the same bounded look-back as the
// scan.
template <typename OT>
__global__ void __launch_bounds__(kScanThreads)
    select_kernel(const uint32_t *__restrict__ sa, uint64_t n, const uint32_t *__restrict__ bits,
                  uint64_t off, OT *__restrict__ out, unsigned long long *__restrict__ status,
                  uint32_t *__restrict__ counter, int *__restrict__ err) {
    __shared__ uint32_t s_tile;
    __shared__ uint32_t s_warp[kScanThreads / 32];
    __shared__ uint32_t s_prefix;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) s_tile = atomicAdd(counter, 1u);
    __syncthreads();
    const uint64_t tile = s_tile;
    const uint64_t base = tile * kScanTile + (uint64_t)tid * kScanItems;
    uint32_t v[kScanItems];
    uint32_t keep = 0u, agg = 0u;  // keep: bit j set when item j is selected
#pragma unroll
    for (int j = 0; j < kScanItems; j++) {
        const uint64_t i = base + j;
        v[j] = i < n ? sa[i] : 0u;
        const uint32_t f = i < n ? (__ldg(bits + (v[j] >> 5)) >> (v[j] & 31)) & 1u : 0u;
        keep |= f << j;
        agg += f;
    }
    uint32_t x = agg;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < kScanThreads / 32 ? s_warp[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < kScanThreads / 32) s_warp[lane] = w;
    }
    __syncthreads();
    const uint32_t within_excl = (warp > 0 ? s_warp[warp - 1] : 0u) + x - agg;
    const uint32_t tile_total = s_warp[kScanThreads / 32 - 1];
    if (tid == 0) {
        uint64_t excl = 0;
        unsigned long long *st = status + tile;
        if (tile == 0) {
            *(volatile unsigned long long *)st = kP | tile_total;
        } else {
            *(volatile unsigned long long *)st = kA | tile_total;
            int64_t t = (int64_t)tile - 1;
            uint32_t spins = 0;
            while (t >= 0) {
                unsigned long long s = *(volatile unsigned long long *)(status + t);
                unsigned long long f = s & ~kMask;
                if (f == 0) {
                    if (++spins > kSpinLimit) {
                        atomicCAS(err, DEV_OK, DEV_LOOKBACK_TIMEOUT);
                        break;
                    }
                    __nanosleep(64);
                    continue;
                }
                excl += s & kMask;
                if (f == kP) break;
                t--;
            }
            *(volatile unsigned long long *)st = kP | (excl + tile_total);
        }
        s_prefix = (uint32_t)excl;
    }
    __syncthreads();
    uint64_t o = off + (uint64_t)s_prefix + within_excl;
#pragma unroll
    for (int j = 0; j < kScanItems; j++)
        if ((keep >> j) & 1u) out[o++] = (OT)v[j];
}

}  // namespace

capssa_status select_bits(Ctx &c, const uint32_t *sa, uint64_t n, const uint32_t *bits,
                          uint64_t off, void *out, int out_bytes) {
    if (n == 0) return CAPSSA_OK;
    uint64_t tiles = (n + kScanTile - 1) / kScanTile;
    unsigned long long *status =
        (unsigned long long *)ws_get(c, WS_SCAN, tiles * 8 + 64);
    if (!status) return set_err(c, CAPSSA_ENOMEM, "select workspace");
    uint32_t *counter = (uint32_t *)(status + tiles);
    CAPSSA_CUDA(c, cudaMemsetAsync(status, 0, tiles * 8 + 64, c.stream));
    if (out_bytes == 8)
        select_kernel<uint64_t><<<(unsigned)tiles, kScanThreads, 0, c.stream>>>(
            sa, n, bits, off, (uint64_t *)out, status, counter, c.d_flags);
    else
        select_kernel<uint32_t><<<(unsigned)tiles, kScanThreads, 0, c.stream>>>(
            sa, n, bits, off, (uint32_t *)out, status, counter, c.d_flags);
    CAPSSA_LAUNCHED(c);
    return CAPSSA_OK;
}

capssa_status scan_u32(Ctx &c, const uint32_t *in, uint32_t *out, uint64_t n, bool max_op,
                       bool inclusive) {
    if (n == 0) return CAPSSA_OK;
    uint64_t tiles = (n + kScanTile - 1) / kScanTile;
    unsigned long long *status =
        (unsigned long long *)ws_get(c, WS_SCAN, tiles * 8 + 64);
    if (!status) return set_err(c, CAPSSA_ENOMEM, "scan workspace");
    uint32_t *counter = (uint32_t *)(status + tiles);
    CAPSSA_CUDA(c, cudaMemsetAsync(status, 0, tiles * 8 + 64, c.stream));
    if (max_op && inclusive)
        scan_kernel<true, true><<<(unsigned)tiles, kScanThreads, 0, c.stream>>>(in, out, n, status,
                                                                               counter, c.d_flags);
    else if (max_op)
        scan_kernel<true, false><<<(unsigned)tiles, kScanThreads, 0, c.stream>>>(
            in, out, n, status, counter, c.d_flags);
    else if (inclusive)
        scan_kernel<false, true><<<(unsigned)tiles, kScanThreads, 0, c.stream>>>(
            in, out, n, status, counter, c.d_flags);
    else
        scan_kernel<false, false><<<(unsigned)tiles, kScanThreads, 0, c.stream>>>(
            in, out, n, status, counter, c.d_flags);
    CAPSSA_LAUNCHED(c);
    return CAPSSA_OK;
}

}  // namespace capssa
