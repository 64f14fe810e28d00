// scan.cu — single-pass device-wide scan (sum or max) of u32 values with
// decoupled look-back.  Each block claims the next tile through an atomic
// counter, so every tile it waits on has already started; every wait is
// bounded and reports DEV_LOOKBACK_TIMEOUT on expiry.
#include "common.cuh"
#include "scan.cuh"

namespace capssa {

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr int kScanTile = kScanThreads * kScanItems;
constexpr unsigned long long kA = 1ull << 62, kP = 2ull << 62, kMask = (1ull << 62) - 1;

template <bool MAX>
__device__ __forceinline__ uint32_t op(uint32_t a, uint32_t b) {
    return MAX ? (a > b ? a : b) : a + b;
}

// Exclusive prefix (in place) of the kScanItems * 8 (step, warp) totals of
// a tile, run by warp 0, each lane owning kPer consecutive entries; returns
// the tile total on every lane.
template <bool MAX>
__device__ __forceinline__ uint32_t tile_prefix(uint32_t *tot) {
    constexpr int kPer = kScanItems * (kScanThreads / 32) / 32;
    const int lane = threadIdx.x & 31;
    uint32_t c[kPer], sum = 0u;
#pragma unroll
    for (int q = 0; q < kPer; q++) {
        c[q] = tot[kPer * lane + q];
        sum = op<MAX>(sum, c[q]);
    }
    uint32_t w = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t z = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w = op<MAX>(w, z);
    }
    const uint32_t total = __shfl_sync(0xffffffffu, w, 31);
    uint32_t run = __shfl_up_sync(0xffffffffu, w, 1);  // before this lane's entries
    if (lane == 0) run = 0u;
#pragma unroll
    for (int q = 0; q < kPer; q++) {
        tot[kPer * lane + q] = run;
        run = op<MAX>(run, c[q]);
    }
    return total;
}

// Decoupled look-back by one whole warp: publishes the tile's aggregate,
// then reads 32 predecessors' status words per round trip, combines those
// up to the nearest inclusive prefix (waiting while any of them is not yet
// published, bounded), and publishes this tile's inclusive prefix.  Returns
// the tile's exclusive prefix on every lane.  (A single thread walking the
// predecessors one at a time waited one L2 round trip per predecessor.)
template <bool MAX>
__device__ __forceinline__ uint32_t warp_lookback(unsigned long long *status, uint64_t tile,
                                                  uint32_t tile_total, int *err) {
    const int lane = threadIdx.x & 31;
    if (lane == 0)
        *(volatile unsigned long long *)(status + tile) = (tile == 0 ? kP : kA) | tile_total;
    if (tile == 0) return 0u;
    uint32_t acc = 0u;
    int64_t top = (int64_t)tile - 1;  // lane l reads tile top - l
    uint32_t spins = 0;
    const unsigned long long before_first = kP;  // before tile 0: inclusive, 0
    for (;;) {
        const int64_t t = top - lane;
        unsigned long long sv = before_first;
        if (t >= 0) sv = *(volatile unsigned long long *)(status + t);
        const unsigned long long fl = sv & ~kMask;
        const unsigned pm = __ballot_sync(0xffffffffu, fl == kP);
        const unsigned bad = __ballot_sync(0xffffffffu, fl == 0);
        const int first_p = pm ? __ffs((int)pm) - 1 : 31;  // lanes 0..first_p count
        const unsigned need = first_p == 31 ? 0xffffffffu : (2u << first_p) - 1u;
        if (bad & need) {
            if (++spins > kSpinLimit) {
                if (lane == 0) atomicCAS(err, DEV_OK, DEV_LOOKBACK_TIMEOUT);
                break;
            }
            __nanosleep(32);
            continue;
        }
        uint32_t v = lane <= first_p ? (uint32_t)(sv & kMask) : 0u;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = op<MAX>(v, __shfl_xor_sync(0xffffffffu, v, o));
        acc = op<MAX>(acc, v);
        if (pm) break;
        top -= 32;
    }
    if (lane == 0) *(volatile unsigned long long *)(status + tile) = kP | op<MAX>(acc, tile_total);
    return acc;
}

template <bool MAX, bool INCLUSIVE>
__global__ void __launch_bounds__(kScanThreads)
    scan_kernel(const uint32_t *__restrict__ in, uint32_t *__restrict__ out, uint64_t n,
                unsigned long long *__restrict__ status, uint32_t *__restrict__ counter,
                int *__restrict__ err) {
    constexpr int kWarps = kScanThreads / 32;
    static_assert(kScanItems * kWarps % 32 == 0, "whole (step, warp) totals per lane of warp 0");
    __shared__ uint32_t s_tile;
    // each (step, warp)'s total; then the exclusive prefix in entry order
    __shared__ uint32_t s_tot[kScanItems * kWarps];
    __shared__ uint32_t s_prefix;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) s_tile = atomicAdd(counter, 1u);
    __syncthreads();
    const uint64_t tile = s_tile;
    const uint64_t base = tile * kScanTile;
    // step j covers entries base + j * 256 .. + 255, one per thread: a warp
    // reads and writes 32 consecutive words; x[j] = its inclusive warp prefix
    uint32_t v[kScanItems], x[kScanItems];
#pragma unroll
    for (int j = 0; j < kScanItems; j++) {
        const uint64_t i = base + (uint64_t)j * kScanThreads + tid;
        v[j] = i < n ? __ldg(in + i) : 0u;
        uint32_t y = v[j];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t z = __shfl_up_sync(0xffffffffu, y, o);
            if (lane >= o) y = op<MAX>(y, z);
        }
        x[j] = y;
        if (lane == 31) s_tot[j * kWarps + warp] = y;
    }
    __syncthreads();
    if (warp == 0) {
        const uint32_t tile_total = tile_prefix<MAX>(s_tot);
        const uint32_t acc = warp_lookback<MAX>(status, tile, tile_total, err);
        if (lane == 0) s_prefix = acc;
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kScanItems; j++) {
        const uint64_t i = base + (uint64_t)j * kScanThreads + tid;
        const uint32_t pre = op<MAX>(s_prefix, s_tot[j * kWarps + warp]);
        uint32_t incl = op<MAX>(pre, x[j]);
        uint32_t excl = __shfl_up_sync(0xffffffffu, incl, 1);
        if (lane == 0) excl = pre;
        if (i < n) out[i] = INCLUSIVE ? incl : excl;
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
    constexpr int kWarps = kScanThreads / 32;
    static_assert(kScanItems * kWarps % 32 == 0, "whole (step, warp) counts per lane of warp 0");
    __shared__ uint32_t s_tile;
    // kept entries per (step, warp); then their exclusive prefix in entry order
    __shared__ uint32_t s_cnt[kScanItems * kWarps];
    __shared__ uint32_t s_prefix;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) s_tile = atomicAdd(counter, 1u);
    __syncthreads();
    const uint64_t tile = s_tile;
    const uint64_t base = tile * kScanTile;
    // step j covers entries base + j * 256 .. + 255, one per thread: loads and
    // stores of a warp are contiguous
    uint32_t v[kScanItems], ball[kScanItems];
#pragma unroll
    for (int j = 0; j < kScanItems; j++) {
        const uint64_t i = base + (uint64_t)j * kScanThreads + tid;
        v[j] = i < n ? __ldg(sa + i) : 0u;
        const bool f = i < n && ((__ldg(bits + (v[j] >> 5)) >> (v[j] & 31)) & 1u);
        ball[j] = __ballot_sync(0xffffffffu, f);
        if (lane == 0) s_cnt[j * kWarps + warp] = __popc(ball[j]);
    }
    __syncthreads();
    if (warp == 0) {
        const uint32_t tile_total = tile_prefix<false>(s_cnt);
        const uint32_t acc = warp_lookback<false>(status, tile, tile_total, err);
        if (lane == 0) s_prefix = acc;
    }
    __syncthreads();
    const uint64_t o0 = off + (uint64_t)s_prefix;
    const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
    for (int j = 0; j < kScanItems; j++)
        if ((ball[j] >> lane) & 1u)
            out[o0 + s_cnt[j * kWarps + warp] + __popc(ball[j] & lt)] = (OT)v[j];
}


// ---------------------------------------------------------------- scatter

// dst[idx[i]] = val(i) for a destination far beyond L2.  Done directly, a
// random 4-byte scatter over the whole array runs at the rate DRAM serves
// partial sectors (about 26 G writes/s: 20 ms for 2^29 entries).  Instead
// the (index, value) pairs are first distributed to at most 256 windows of
// 2^wb destination entries (8 MB or more) and then applied window by window,
// so every destination line is assembled in L2 and written back whole.  The
// distribution is a counting sort of 4096-pair tiles: per-tile window counts,
// one exclusive scan of them in window-major order, then each tile writes its
// pairs, grouped by window in shared memory, after its slot in every window.
// Tiles run in index order, so the tiles in flight write next to each other in
// every window (a handful of pages, not the whole pair array: blocks that
// each owned a long chunk were TLB-bound, 12 ms at 2^29).
constexpr int kWinMin = 21;
constexpr int kWinMax = 256;
constexpr int kWinPer = 16;  // pairs per thread and tile
constexpr int kWinTile = 256 * kWinPer;

__device__ __forceinline__ uint32_t pair_val(const uint32_t *vals, uint32_t i) {
    return vals ? __ldg(vals + i) : i;
}

__global__ void scatter_direct_kernel(const uint32_t *__restrict__ idx,
                                      const uint32_t *__restrict__ vals, uint32_t m,
                                      uint32_t *__restrict__ dst) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x)
        dst[idx[i]] = pair_val(vals, i);
}

// hist[w * gridDim.x + t] = pairs of tile t in window w.
__global__ void __launch_bounds__(256)
    win_count_kernel(const uint32_t *__restrict__ idx, uint32_t m, int wb,
                     uint32_t *__restrict__ hist) {
    __shared__ uint32_t h[kWinMax];
    h[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t base = blockIdx.x * (uint32_t)kWinTile;
#pragma unroll
    for (int j = 0; j < kWinPer; j++) {
        const uint32_t i = base + j * 256 + threadIdx.x;
        if (i < m) atomicAdd(&h[__ldg(idx + i) >> wb], 1u);
    }
    __syncthreads();
    hist[(size_t)threadIdx.x * gridDim.x + blockIdx.x] = h[threadIdx.x];
}

// Exclusive block-wide prefix of one u32 per thread (256 threads).
__device__ __forceinline__ uint32_t block_excl_256(uint32_t v) {
    __shared__ uint32_t s_w[8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_w[warp] = x;
    __syncthreads();
    uint32_t before = 0;
    for (int w = 0; w < warp; w++) before += s_w[w];
    return before + x - v;
}

// (index << 32 | value) pairs of tile t into their windows, after the tile's
// slot0[w * gridDim.x + t] in each; staged in shared memory in window order
// so that consecutive threads write consecutive slots.
__global__ void __launch_bounds__(256)
    win_scatter_kernel(const uint32_t *__restrict__ idx, const uint32_t *__restrict__ vals,
                       uint32_t m, int wb, const uint32_t *__restrict__ slot0,
                       uint64_t *__restrict__ pairs) {
    __shared__ uint64_t st[kWinTile];
    __shared__ uint32_t s_cnt[kWinMax], s_start[kWinMax], s_slot[kWinMax];
    s_cnt[threadIdx.x] = 0;
    s_slot[threadIdx.x] = slot0[(size_t)threadIdx.x * gridDim.x + blockIdx.x];
    __syncthreads();
    const uint32_t base = blockIdx.x * (uint32_t)kWinTile;
    const uint32_t valid = m - base < (uint32_t)kWinTile ? m - base : (uint32_t)kWinTile;
    uint64_t e[kWinPer];
    uint32_t r[kWinPer];
#pragma unroll
    for (int j = 0; j < kWinPer; j++) {
        const uint32_t l = j * 256 + threadIdx.x;
        if (l < valid) {
            const uint32_t p = __ldg(idx + base + l);
            e[j] = ((uint64_t)p << 32) | pair_val(vals, base + l);
            r[j] = atomicAdd(&s_cnt[p >> wb], 1u);
        }
    }
    __syncthreads();
    s_start[threadIdx.x] = block_excl_256(s_cnt[threadIdx.x]);
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kWinPer; j++) {
        const uint32_t l = j * 256 + threadIdx.x;
        if (l < valid) st[s_start[(uint32_t)(e[j] >> 32) >> wb] + r[j]] = e[j];
    }
    __syncthreads();
    for (uint32_t l = threadIdx.x; l < valid; l += 256) {
        const uint64_t x = st[l];
        const uint32_t w = (uint32_t)(x >> 32) >> wb;
        pairs[s_slot[w] + (l - s_start[w])] = x;
    }
}

// dst[index] = value, streaming the pairs window by window.
__global__ void win_apply_kernel(const uint64_t *__restrict__ pairs, uint32_t m,
                                 uint32_t *__restrict__ dst) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
        const uint64_t e = __ldg(pairs + i);
        dst[e >> 32] = (uint32_t)e;
    }
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


size_t scatter_hist_words(uint64_t m) {
    return (size_t)kWinMax * ((m + kWinTile - 1) / kWinTile) + 64;
}

capssa_status scatter_u32(Ctx &c, const uint32_t *idx, const uint32_t *vals, uint64_t m,
                          uint32_t *dst, uint64_t n_dst, uint64_t *pairs, uint32_t *hist) {
    if (m == 0) return CAPSSA_OK;
    if (m > 0xFFFFFFFFull || n_dst > 0x100000000ull)
        return set_err(c, CAPSSA_EUNSUPPORTED, "scatter beyond 2^32 entries");
    const uint32_t mm = (uint32_t)m;
    if (n_dst <= (1ull << 24) || !pairs || !hist) {  // the destination fits L2
        scatter_direct_kernel<<<grid_for(m, 256), 256, 0, c.stream>>>(idx, vals, mm, dst);
        CAPSSA_LAUNCHED(c);
        return CAPSSA_OK;
    }
    int wb = kWinMin;
    while ((uint64_t)kWinMax << wb < n_dst) wb++;
    const uint32_t tiles = (uint32_t)((m + kWinTile - 1) / kWinTile);
    win_count_kernel<<<tiles, 256, 0, c.stream>>>(idx, mm, wb, hist);
    CAPSSA_LAUNCHED(c);
    capssa_status s = scan_u32(c, hist, hist, (uint64_t)kWinMax * tiles, false, false);
    if (s != CAPSSA_OK) return s;
    win_scatter_kernel<<<tiles, 256, 0, c.stream>>>(idx, vals, mm, wb, hist, pairs);
    CAPSSA_LAUNCHED(c);
    win_apply_kernel<<<grid_for(m, 256), 256, 0, c.stream>>>(pairs, mm, dst);
    CAPSSA_LAUNCHED(c);
    return CAPSSA_OK;
}

}  // namespace capssa
