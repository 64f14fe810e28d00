// bucket.cu — shared-memory sort of key buckets and bucket boundaries
// (see bucket.cuh).
#include <algorithm>
#include <vector>

#include "bucket.cuh"
#include "radix.cuh"

namespace capssa {
namespace bucket {

namespace {

constexpr int kThreads = 512;
constexpr int kItems = kCap / kThreads;  // 16
constexpr int kWarps = kThreads / 32;
constexpr size_t kSmem = (size_t)kCap * 8 * 2 + (size_t)kCap * 4 * 2 + (size_t)kWarps * 256 * 4 +
                         256 * 4 + 64;

// One block sorts one bucket at a time.  The bucket is split into kWarps
// contiguous warp chunks (a multiple of 32 records each); every 8-bit pass
// ranks each warp's records by digit with ballots and shared atomics (a
// stable multisplit), scans the per-warp digit counts and scatters into the
// other shared buffer.  The first pass reads its records straight from
// global memory, passes whose digit is constant over the bucket are
// skipped, and the result is written back once, coalesced.
__global__ void __launch_bounds__(kThreads, 1)
    bucket_sort_kernel(uint64_t *__restrict__ keys, uint32_t *__restrict__ vals,
                       const uint32_t *__restrict__ start, uint32_t nbuckets, int low_bits) {
    extern __shared__ __align__(16) unsigned char smem[];
    uint64_t *k0 = reinterpret_cast<uint64_t *>(smem);
    uint64_t *k1 = k0 + kCap;
    uint32_t *v0 = reinterpret_cast<uint32_t *>(k1 + kCap);
    uint32_t *v1 = v0 + kCap;
    uint32_t *whist = v1 + kCap;        // kWarps x 256
    uint32_t *dstart = whist + kWarps * 256;
    __shared__ uint32_t s_scan[kThreads / 32];
    __shared__ int s_skip[2];  // by pass parity: a pass never resets the flag being read
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const unsigned lt_mask = (1u << lane) - 1u;

    for (uint32_t b = blockIdx.x; b < nbuckets; b += gridDim.x) {
        const uint32_t s = start[b], len = start[b + 1] - s;
        if (len <= 1 || len > kCap) continue;  // block-uniform
        // warp chunks: `chunk` records each (multiple of 32), `iters` rows of 32
        const uint32_t chunk = ((len + kWarps - 1) / kWarps + 31) & ~31u;
        const int iters = (int)(chunk >> 5);
        const uint32_t wbase = warp * chunk;
        // padding lanes (index >= len) rank last in digit 255 of the last warp
        const uint32_t pad = (uint32_t)(kWarps * chunk) - len;
        uint64_t *ks = k0, *kd = k1;
        uint32_t *vs = v0, *vd = v1;
        bool first = true;
        for (int shift = 0; shift < low_bits; shift += 8) {
            const int par = (shift >> 3) & 1;
            for (int i = tid; i < kWarps * 256; i += kThreads) whist[i] = 0;
            if (tid == 0) s_skip[par] = 0;
            uint64_t kk[kItems];
            uint32_t vv[kItems], d[kItems], r[kItems];
#pragma unroll
            for (int j = 0; j < kItems; j++) {
                if (j < iters) {
                    const uint32_t e = wbase + j * 32 + lane;
                    const bool valid = e < len;
                    if (first) {
                        kk[j] = valid ? keys[s + e] : ~0ull;
                        vv[j] = valid ? vals[s + e] : 0u;
                    } else {
                        kk[j] = valid ? ks[e] : ~0ull;
                        vv[j] = valid ? vs[e] : 0u;
                    }
                    d[j] = valid ? (uint32_t)(kk[j] >> shift) & 255u : 255u;
                }
            }
            __syncthreads();
            uint32_t *wh = whist + warp * 256;
#pragma unroll
            for (int j = 0; j < kItems; j++)
                if (j < iters) r[j] = warp_rank_digit(wh, d[j], warp_match_bits<8>(d[j]), lt_mask, lane);
            __syncthreads();
            uint32_t total = 0;
            if (tid < 256) {
#pragma unroll
                for (int w = 0; w < kWarps; w++) {
                    uint32_t c = whist[w * 256 + tid];
                    whist[w * 256 + tid] = total;
                    total += c;
                }
                uint32_t counted = tid == 255 ? total - pad : total;
                if (counted == len) s_skip[par] = 1;
            }
            // exclusive scan of the digit totals over threads 0..255
            uint32_t x = total;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            if (lane == 31) s_scan[warp] = x;
            __syncthreads();
            if (tid < 256) {
                uint32_t before = 0;
                for (int w = 0; w < warp; w++) before += s_scan[w];
                dstart[tid] = before + x - total;
            }
            __syncthreads();
            if (s_skip[par]) {
                // one digit for the whole bucket: order unchanged
                if (first) {
#pragma unroll
                    for (int j = 0; j < kItems; j++) {
                        const uint32_t e = wbase + j * 32 + lane;
                        if (j < iters && e < len) {
                            ks[e] = kk[j];
                            vs[e] = vv[j];
                        }
                    }
                    first = false;
                    __syncthreads();
                }
                continue;
            }
            first = false;
#pragma unroll
            for (int j = 0; j < kItems; j++) {
                if (j < iters) {
                    const uint32_t pos = dstart[d[j]] + wh[d[j]] + r[j];
                    if (pos < len) {
                        kd[pos] = kk[j];
                        vd[pos] = vv[j];
                    }
                }
            }
            __syncthreads();
            uint64_t *tk = ks;
            ks = kd;
            kd = tk;
            uint32_t *tv = vs;
            vs = vd;
            vd = tv;
        }
        if (!first) {
            for (uint32_t i = tid; i < len; i += kThreads) {
                keys[s + i] = ks[i];
                vals[s + i] = vs[i];
            }
        }
        __syncthreads();
    }
}

__global__ void starts_kernel(const uint64_t *__restrict__ keys, uint32_t n, int shift,
                              uint32_t *__restrict__ start) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t b = (uint32_t)(keys[i] >> shift) & (kBuckets - 1);
        int64_t prev = i == 0 ? -1 : (int64_t)((uint32_t)(keys[i - 1] >> shift) & (kBuckets - 1));
        for (int64_t v = prev + 1; v <= (int64_t)b; v++) start[v] = i;
        if (i == n - 1)
            for (uint32_t v = b + 1; v <= kBuckets; v++) start[v] = n;
    }
}

// Oversize buckets: (ordinal, low key bits) composites for one global sort.
__global__ void gather_over_kernel(const uint64_t *__restrict__ keys,
                                   const uint32_t *__restrict__ vals,
                                   const uint32_t *__restrict__ ostart,  // bucket start per ordinal
                                   const uint32_t *__restrict__ toff,    // tmp offset per ordinal (+1)
                                   uint32_t nover, uint32_t total, int low_bits,
                                   uint64_t *__restrict__ tk, uint32_t *__restrict__ tv) {
    const uint64_t low_mask = low_bits >= 64 ? ~0ull : ((1ull << low_bits) - 1);
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += gridDim.x * blockDim.x) {
        uint32_t lo = 0, hi = nover;  // last ordinal with toff <= t
        while (hi - lo > 1) {
            uint32_t mid = (lo + hi) >> 1;
            if (toff[mid] <= t)
                lo = mid;
            else
                hi = mid;
        }
        uint32_t src = ostart[lo] + (t - toff[lo]);
        tk[t] = ((uint64_t)lo << low_bits) | (keys[src] & low_mask);
        tv[t] = vals[src];
    }
}

__global__ void scatter_over_kernel(const uint64_t *__restrict__ tk,
                                    const uint32_t *__restrict__ tv,
                                    const uint32_t *__restrict__ ostart,
                                    const uint32_t *__restrict__ toff, const uint32_t *__restrict__ obkt,
                                    uint32_t total, int low_bits, int shift,
                                    uint64_t *__restrict__ keys, uint32_t *__restrict__ vals) {
    const uint64_t low_mask = low_bits >= 64 ? ~0ull : ((1ull << low_bits) - 1);
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += gridDim.x * blockDim.x) {
        uint64_t k = tk[t];
        uint32_t ord = (uint32_t)(k >> low_bits);
        uint32_t dst = ostart[ord] + (t - toff[ord]);
        keys[dst] = ((uint64_t)obkt[ord] << shift) | (k & low_mask);
        vals[dst] = tv[t];
    }
}

}  // namespace

capssa_status bucket_starts(Ctx &c, const uint64_t *keys, uint32_t n, int shift,
                            uint32_t *d_start) {
    if (n == 0) return CAPSSA_OK;
    starts_kernel<<<grid_for(n, 256), 256, 0, c.stream>>>(keys, n, shift, d_start);
    CAPSSA_LAUNCHED(c);
    return CAPSSA_OK;
}

capssa_status sort_buckets(Ctx &c, uint64_t *keys, uint32_t *vals, uint64_t *t1k, uint32_t *t1v,
                           uint64_t *t2k, uint32_t *t2v, uint32_t n, const uint32_t *d_start,
                           const uint32_t *h_start, int low_bits) {
    (void)n;
    // per-device attribute: set on every call (cheap)
    cudaFuncSetAttribute(bucket_sort_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)kSmem);
    bucket_sort_kernel<<<(unsigned)c.sm_count, kThreads, kSmem, c.stream>>>(keys, vals, d_start,
                                                                           kBuckets, low_bits);
    CAPSSA_LAUNCHED(c);
    // buckets past the shared-memory capacity: one global sort of
    // (ordinal, low bits) composites, then back into place
    std::vector<uint32_t> ostart, obkt, toff;
    uint32_t total = 0;
    for (uint32_t b = 0; b < kBuckets; b++) {
        uint32_t len = h_start[b + 1] - h_start[b];
        if (len > kCap) {
            ostart.push_back(h_start[b]);
            obkt.push_back(b);
            toff.push_back(total);
            total += len;
        }
    }
    if (ostart.empty()) return CAPSSA_OK;
    const uint32_t nover = (uint32_t)ostart.size();
    uint32_t *meta = (uint32_t *)ws_get(c, WS_MISC3, (size_t)nover * 12 + 64);
    if (!meta) return set_err(c, CAPSSA_ENOMEM, "bucket metadata");
    std::vector<uint32_t> h(3 * (size_t)nover);
    std::copy(ostart.begin(), ostart.end(), h.begin());
    std::copy(toff.begin(), toff.end(), h.begin() + nover);
    std::copy(obkt.begin(), obkt.end(), h.begin() + 2 * (size_t)nover);
    CAPSSA_CUDA(c, cudaMemcpyAsync(meta, h.data(), h.size() * 4, cudaMemcpyHostToDevice, c.stream));
    uint32_t *d_ostart = meta, *d_toff = meta + nover, *d_obkt = meta + 2 * nover;
    int ord_bits = 1;
    while ((1u << ord_bits) < nover) ord_bits++;
    gather_over_kernel<<<grid_for(total, 256), 256, 0, c.stream>>>(
        keys, vals, d_ostart, d_toff, nover, total, low_bits, t1k, t1v);
    CAPSSA_LAUNCHED(c);
    bool in_b = false;
    capssa_status s = radix::sort_pairs(c, t1k, t1v, t2k, t2v, total, 0, low_bits + ord_bits,
                                        false, 0, &in_b);
    if (s != CAPSSA_OK) return s;
    scatter_over_kernel<<<grid_for(total, 256), 256, 0, c.stream>>>(
        in_b ? t2k : t1k, in_b ? t2v : t1v, d_ostart, d_toff, d_obkt, total, low_bits, low_bits,
        keys, vals);
    CAPSSA_LAUNCHED(c);
    CAPSSA_CUDA(c, cudaStreamSynchronize(c.stream));  // host vectors go out of scope
    return CAPSSA_OK;
}

}  // namespace bucket
}  // namespace capssa
