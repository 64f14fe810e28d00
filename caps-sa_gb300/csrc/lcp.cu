// lcp.cu — LCP-based kernels: LCP arrays, batched LcpDispatch::lcp /
// suffix_cmp_with, the bounded-context run flags, and the merge-path
// version of the reference's LCP-enhanced two-way merge.
#include <algorithm>

#include "lcp.cuh"

namespace capssa {

namespace {

constexpr int kWarpBlock = 256;  // 8 warps per block, one pair per warp

__device__ __forceinline__ int dev_boundary_order(const DevLimits &L, uint64_t pa, uint64_t la,
                                                  uint64_t pb, uint64_t lb) {
    if (!L.longer_first) return (la > lb) - (la < lb);
    if (lb != la) return (lb > la) - (lb < la);
    return (pa > pb) - (pa < pb);
}

// Thread-level LcpDispatch::lcp restricted to lim symbols.
__device__ __forceinline__ uint64_t thread_sym_lcp(const void *text, int sym, uint64_t p,
                                                   uint64_t q, uint64_t lim) {
    const uint64_t k = (uint64_t)sym;
    return thread_lcp_bytes((const uint8_t *)text, p * k, q * k, lim * k) / k;
}

// LcpDispatch::suffix_cmp_with (src/lcp.rs:184-201), one thread.
__device__ int thread_suffix_cmp(const void *text, int sym, const DevLimits &L, uint64_t p,
                                 uint64_t q, uint64_t max_ctx) {
    uint64_t lp = dev_lim_at(L, p), lq = dev_lim_at(L, q);
    uint64_t lim = lp < lq ? lp : lq;
    if (max_ctx < lim) lim = max_ctx;
    uint64_t common = thread_sym_lcp(text, sym, p, q, lim);
    if (common < lim) {
        uint64_t a = sym_at(text, sym, p + common), b = sym_at(text, sym, q + common);
        return (a > b) - (a < b);
    }
    return dev_boundary_order(L, p, lp, q, lq);
}

template <typename OT>
__global__ void __launch_bounds__(kWarpBlock)
    lcp_array_kernel(const void *__restrict__ text, int sym, DevLimits L, uint64_t max_ctx,
                     const uint32_t *__restrict__ sa, uint64_t m, OT *__restrict__ out) {
    const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const uint32_t lane = threadIdx.x & 31;
    for (uint64_t i = warp; i < m; i += nwarps) {
        uint64_t r = 0;
        if (i > 0) {
            uint64_t a = sa[i - 1], b = sa[i];
            uint64_t cap = min(dev_lim_at(L, a), dev_lim_at(L, b));
            if (max_ctx < cap) cap = max_ctx;
            const uint64_t k = (uint64_t)sym;
            r = warp_lcp_bytes((const uint8_t *)text, a * k, b * k, cap * k) / k;
        }
        if (lane == 0) out[i] = (OT)r;
    }
}

__global__ void __launch_bounds__(kWarpBlock)
    lcp_pairs_kernel(const void *__restrict__ text, int sym, uint64_t n,
                     const uint64_t *__restrict__ p, const uint64_t *__restrict__ q,
                     uint64_t count, uint64_t max_ctx, uint64_t *__restrict__ out) {
    const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t i = warp; i < count; i += nwarps) {
        uint64_t r = warp_sym_lcp(text, sym, n, p[i], q[i], max_ctx);
        if ((threadIdx.x & 31) == 0) out[i] = r;
    }
}

__global__ void __launch_bounds__(kWarpBlock)
    suffix_cmp_kernel(const void *__restrict__ text, int sym, DevLimits L,
                      const uint64_t *__restrict__ p, const uint64_t *__restrict__ q,
                      uint64_t count, uint64_t max_ctx, int8_t *__restrict__ out) {
    const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t i = warp; i < count; i += nwarps) {
        uint64_t a = p[i], b = q[i];
        uint64_t la = dev_lim_at(L, a), lb = dev_lim_at(L, b);
        uint64_t lim = la < lb ? la : lb;
        if (max_ctx < lim) lim = max_ctx;
        const uint64_t k = (uint64_t)sym;
        uint64_t common = warp_lcp_bytes((const uint8_t *)text, a * k, b * k, lim * k) / k;
        int r;
        if (common < lim) {
            uint64_t x = sym_at(text, sym, a + common), y = sym_at(text, sym, b + common);
            r = (x > y) - (x < y);
        } else {
            r = dev_boundary_order(L, a, la, b, lb);
        }
        if ((threadIdx.x & 31) == 0) out[i] = (int8_t)r;
    }
}

__global__ void __launch_bounds__(kWarpBlock)
    ctx_run_kernel(const void *__restrict__ text, int sym, DevLimits L, uint64_t C,
                   const uint32_t *__restrict__ sa, uint64_t m, uint8_t *__restrict__ flags) {
    const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t i = warp; i < m; i += nwarps) {
        uint8_t f = 0;
        if (i > 0) {
            uint64_t a = sa[i - 1], b = sa[i];
            uint64_t cap = min(dev_lim_at(L, a), dev_lim_at(L, b));
            if (cap >= C) {
                const uint64_t k = (uint64_t)sym;
                f = warp_lcp_bytes((const uint8_t *)text, a * k, b * k, C * k) / k >= C;
            }
        }
        if ((threadIdx.x & 31) == 0) flags[i] = f;
    }
}

// ------------------------------------------------------------ merge path

constexpr uint64_t kMergeSeg = 128;  // outputs per sequential segment

template <typename IT>
__device__ __forceinline__ bool tied(const void *text, int sym, const DevLimits &L, IT a, IT b,
                                     uint64_t max_ctx) {
    return thread_suffix_cmp(text, sym, L, (uint64_t)a, (uint64_t)b, max_ctx) == 0;
}

// Split of diagonal d: i elements from x, d - i from y, with comparator
// ties counted as "x first".  A split is safe when no comparator tie spans
// it across the two runs; only safe splits start a segment, so every tie
// class is merged inside one sequential segment with the reference's
// alternating tie rule.
template <typename IT>
__global__ void merge_split_kernel(const void *__restrict__ text, int sym, DevLimits L,
                                   const IT *__restrict__ x, uint64_t lx,
                                   const IT *__restrict__ y, uint64_t ly, uint64_t max_ctx,
                                   uint64_t nseg, uint64_t *__restrict__ split,
                                   uint8_t *__restrict__ safe) {
    for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s <= nseg;
         s += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t d = min(s * kMergeSeg, lx + ly);
        uint64_t lo = d > ly ? d - ly : 0, hi = d < lx ? d : lx;
        while (lo < hi) {
            uint64_t mid = (lo + hi) >> 1;
            // does x[mid] come before y[d - 1 - mid]?
            if (thread_suffix_cmp(text, sym, L, x[mid], y[d - 1 - mid], max_ctx) <= 0)
                lo = mid + 1;
            else
                hi = mid;
        }
        uint64_t i = lo, j = d - lo;
        bool ok = true;
        if (s > 0 && s < nseg) {
            if (i > 0 && j < ly && tied(text, sym, L, x[i - 1], y[j], max_ctx)) ok = false;
            if (ok && j > 0 && i < lx && tied(text, sym, L, y[j - 1], x[i], max_ctx)) ok = false;
            if (ok && i > 0 && j > 0 && i < lx && j < ly &&
                tied(text, sym, L, x[i - 1], y[j - 1], max_ctx) &&
                tied(text, sym, L, x[i], y[j], max_ctx))
                ok = false;
        }
        split[s] = i;
        safe[s] = ok ? 1 : 0;
    }
}

// sample_sort::merge body (src/sample_sort.rs:430-500) on one segment, with
// the segment's entry state rebuilt from the element output just before it.
template <typename IT>
__global__ void merge_seg_kernel(const void *__restrict__ text, int sym, DevLimits L,
                                 const IT *__restrict__ x, const IT *__restrict__ lcp_x,
                                 uint64_t lx, const IT *__restrict__ y,
                                 const IT *__restrict__ lcp_y, uint64_t ly, uint64_t max_ctx,
                                 uint64_t nseg, const uint64_t *__restrict__ split,
                                 const uint8_t *__restrict__ safe, IT *__restrict__ z,
                                 IT *__restrict__ lcp_z) {
    for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < nseg;
         s += (uint64_t)gridDim.x * blockDim.x) {
        if (s > 0 && !safe[s]) continue;
        uint64_t e = s + 1;
        while (e < nseg && !safe[e]) e++;
        const uint64_t d0 = min(s * kMergeSeg, lx + ly);
        const uint64_t de = min(e * kMergeSeg, lx + ly);
        uint64_t i0 = split[s], j0 = d0 - i0;
        uint64_t ie = split[e], je = de - ie;
        // A = stream of the last output before this segment (x if none:
        // the reference starts with A = x, B = y)
        bool a_is_x = true;
        uint64_t m = 0;
        if (d0 > 0) {
            if (i0 == 0)
                a_is_x = false;
            else if (j0 == 0)
                a_is_x = true;
            else
                a_is_x = thread_suffix_cmp(text, sym, L, x[i0 - 1], y[j0 - 1], max_ctx) >= 0;
            uint64_t prev = a_is_x ? (uint64_t)x[i0 - 1] : (uint64_t)y[j0 - 1];
            bool b_has = a_is_x ? (j0 < ly) : (i0 < lx);
            if (b_has) {
                uint64_t bf = a_is_x ? (uint64_t)y[j0] : (uint64_t)x[i0];
                uint64_t cap = min(dev_lim_at(L, prev), dev_lim_at(L, bf));
                if (max_ctx < cap) cap = max_ctx;
                m = thread_sym_lcp(text, sym, prev, bf, cap);
            }
        }
        const IT *arr_a = a_is_x ? x : y, *arr_b = a_is_x ? y : x;
        const IT *la_arr = a_is_x ? lcp_x : lcp_y, *lb_arr = a_is_x ? lcp_y : lcp_x;
        uint64_t ia = a_is_x ? i0 : j0, ib = a_is_x ? j0 : i0;
        uint64_t ea = a_is_x ? ie : je, eb = a_is_x ? je : ie;
        uint64_t k = d0;
        bool ca_ok = false, cb_ok = false;
        uint64_t ca_idx = 0, ca_lim = 0, cb_idx = 0, cb_lim = 0;
        while (ia < ea && ib < eb) {
            uint64_t l_a = (uint64_t)la_arr[ia];
            bool out_a;
            uint64_t lcp_out, new_m;
            if (l_a > m) {
                out_a = true;
                lcp_out = l_a;
                new_m = m;
            } else if (l_a < m) {
                out_a = false;
                lcp_out = m;
                new_m = l_a;
            } else {
                uint64_t pa = arr_a[ia], pb = arr_b[ib];
                uint64_t lim_a, lim_b;
                if (ca_ok && ca_idx == ia) {
                    lim_a = ca_lim;
                } else {
                    lim_a = dev_lim_at(L, pa);
                    ca_ok = true;
                    ca_idx = ia;
                    ca_lim = lim_a;
                }
                if (cb_ok && cb_idx == ib) {
                    lim_b = cb_lim;
                } else {
                    lim_b = dev_lim_at(L, pb);
                    cb_ok = true;
                    cb_idx = ib;
                    cb_lim = lim_b;
                }
                uint64_t cap = min(lim_a, lim_b);
                if (max_ctx < cap) cap = max_ctx;
                uint64_t rem = cap > m ? cap - m : 0;
                uint64_t ext = thread_sym_lcp(text, sym, pa + m, pb + m, rem);
                uint64_t total = m + ext;
                bool a_smaller;
                if (total < cap)
                    a_smaller = sym_at(text, sym, pa + total) < sym_at(text, sym, pb + total);
                else
                    a_smaller = dev_boundary_order(L, pa, lim_a, pb, lim_b) < 0;
                out_a = a_smaller;
                lcp_out = m;
                new_m = total;
            }
            if (out_a) {
                z[k] = arr_a[ia];
                lcp_z[k] = (IT)lcp_out;
                ia++;
                ca_ok = false;
            } else {
                z[k] = arr_b[ib];
                lcp_z[k] = (IT)lcp_out;
                ib++;
                cb_ok = false;
                const IT *t;
                t = arr_a; arr_a = arr_b; arr_b = t;
                t = la_arr; la_arr = lb_arr; lb_arr = t;
                uint64_t u;
                u = ia; ia = ib; ib = u;
                u = ea; ea = eb; eb = u;
                bool o = ca_ok; ca_ok = cb_ok; cb_ok = o;
                u = ca_idx; ca_idx = cb_idx; cb_idx = u;
                u = ca_lim; ca_lim = cb_lim; cb_lim = u;
            }
            m = new_m;
            k++;
        }
        // drain (src/sample_sort.rs:614-636): the first drained record of B
        // carries m, the LCP against the last output.  A still holds records
        // only when B had none inside this segment; then nothing was output
        // here and A's own LCP array already relates A's front to the last
        // output (the reference never reaches this case: its B is non-empty).
        for (int side = 0; side < 2; side++) {
            const IT *arr = side == 0 ? arr_a : arr_b;
            const IT *ls = side == 0 ? la_arr : lb_arr;
            uint64_t i = side == 0 ? ia : ib, en = side == 0 ? ea : eb;
            bool first = side == 1;
            while (i < en) {
                z[k] = arr[i];
                lcp_z[k] = first ? (IT)m : ls[i];
                first = false;
                i++;
                k++;
            }
        }
    }
}

unsigned warp_grid(Ctx &c, uint64_t items) {
    uint64_t blocks = (items * 32 + kWarpBlock - 1) / kWarpBlock;
    if (blocks < 1) blocks = 1;
    uint64_t cap = (uint64_t)c.sm_count * 32;
    return (unsigned)std::min<uint64_t>(blocks, cap);
}

}  // namespace

capssa_status lcp_array_sa(Ctx &c, const void *text, int sym_bytes, uint64_t n,
                           const DevLimits &L, uint64_t max_ctx, const uint32_t *sa, uint64_t m,
                           void *out_lcp, int out_bytes) {
    (void)n;
    if (m == 0) return CAPSSA_OK;
    if (out_bytes == 4)
        lcp_array_kernel<uint32_t><<<warp_grid(c, m), kWarpBlock, 0, c.stream>>>(
            text, sym_bytes, L, max_ctx, sa, m, (uint32_t *)out_lcp);
    else
        lcp_array_kernel<uint64_t><<<warp_grid(c, m), kWarpBlock, 0, c.stream>>>(
            text, sym_bytes, L, max_ctx, sa, m, (uint64_t *)out_lcp);
    CAPSSA_LAUNCHED(c);
    return CAPSSA_OK;
}

capssa_status lcp_pairs(Ctx &c, const void *text, int sym_bytes, uint64_t n, const uint64_t *p,
                        const uint64_t *q, uint64_t count, uint64_t max_ctx, uint64_t *out) {
    if (count == 0) return CAPSSA_OK;
    lcp_pairs_kernel<<<warp_grid(c, count), kWarpBlock, 0, c.stream>>>(text, sym_bytes, n, p, q,
                                                                      count, max_ctx, out);
    CAPSSA_LAUNCHED(c);
    return CAPSSA_OK;
}

capssa_status suffix_cmp_pairs(Ctx &c, const void *text, int sym_bytes, const DevLimits &L,
                               const uint64_t *p, const uint64_t *q, uint64_t count,
                               uint64_t max_ctx, int8_t *out) {
    if (count == 0) return CAPSSA_OK;
    suffix_cmp_kernel<<<warp_grid(c, count), kWarpBlock, 0, c.stream>>>(text, sym_bytes, L, p, q,
                                                                       count, max_ctx, out);
    CAPSSA_LAUNCHED(c);
    return CAPSSA_OK;
}

capssa_status ctx_run_flags(Ctx &c, const void *text, int sym_bytes, const DevLimits &L,
                            uint64_t max_ctx, const uint32_t *sa, uint64_t m, uint8_t *flags) {
    if (m == 0) return CAPSSA_OK;
    ctx_run_kernel<<<warp_grid(c, m), kWarpBlock, 0, c.stream>>>(text, sym_bytes, L, max_ctx, sa,
                                                                m, flags);
    CAPSSA_LAUNCHED(c);
    return CAPSSA_OK;
}

capssa_status merge_runs(Ctx &c, const void *text, int sym_bytes, const DevLimits &L,
                         const void *x, const void *lcp_x, uint64_t len_x, const void *y,
                         const void *lcp_y, uint64_t len_y, uint64_t max_ctx, void *z,
                         void *lcp_z, int idx_bytes) {
    const uint64_t total = len_x + len_y;
    if (total == 0) return CAPSSA_OK;
    const size_t ib = (size_t)idx_bytes;
    if (len_x == 0 || len_y == 0) {
        const void *src = len_x ? x : y, *ls = len_x ? lcp_x : lcp_y;
        CAPSSA_CUDA(c, cudaMemcpyAsync(z, src, total * ib, cudaMemcpyDeviceToDevice, c.stream));
        CAPSSA_CUDA(c, cudaMemcpyAsync(lcp_z, ls, total * ib, cudaMemcpyDeviceToDevice, c.stream));
        return CAPSSA_OK;
    }
    const uint64_t nseg = (total + kMergeSeg - 1) / kMergeSeg;
    uint64_t *split = (uint64_t *)ws_get(c, WS_MISC, (nseg + 1) * 9 + 64);
    if (!split) return set_err(c, CAPSSA_ENOMEM, "merge workspace");
    uint8_t *safe = (uint8_t *)(split + nseg + 1);
    unsigned g = grid_for(nseg + 1, 128, (unsigned)c.sm_count * 16);
    if (idx_bytes == 4) {
        merge_split_kernel<uint32_t><<<g, 128, 0, c.stream>>>(
            text, sym_bytes, L, (const uint32_t *)x, len_x, (const uint32_t *)y, len_y, max_ctx,
            nseg, split, safe);
        CAPSSA_LAUNCHED(c);
        merge_seg_kernel<uint32_t><<<g, 128, 0, c.stream>>>(
            text, sym_bytes, L, (const uint32_t *)x, (const uint32_t *)lcp_x, len_x,
            (const uint32_t *)y, (const uint32_t *)lcp_y, len_y, max_ctx, nseg, split, safe,
            (uint32_t *)z, (uint32_t *)lcp_z);
        CAPSSA_LAUNCHED(c);
    } else {
        merge_split_kernel<uint64_t><<<g, 128, 0, c.stream>>>(
            text, sym_bytes, L, (const uint64_t *)x, len_x, (const uint64_t *)y, len_y, max_ctx,
            nseg, split, safe);
        CAPSSA_LAUNCHED(c);
        merge_seg_kernel<uint64_t><<<g, 128, 0, c.stream>>>(
            text, sym_bytes, L, (const uint64_t *)x, (const uint64_t *)lcp_x, len_x,
            (const uint64_t *)y, (const uint64_t *)lcp_y, len_y, max_ctx, nseg, split, safe,
            (uint64_t *)z, (uint64_t *)lcp_z);
        CAPSSA_LAUNCHED(c);
    }
    return CAPSSA_OK;
}

}  // namespace capssa

// ====================================================================
// Allocation-free merge entry point.
//
// Some callers cannot call cudaMalloc at the point where they need a merge:
// a host application that hands all device memory to its own pool allocator
// up front, code running between other work on a stream where an allocation
// (and the device-wide synchronisation cudaMalloc/cudaFree may imply) is not
// acceptable, or a caller without a library context.  For them
// capssa_merge_noalloc_u8_u32 runs the same merge-path kernels as
// capssa_merge_u8_u32, but with every buffer supplied by the caller and the
// merge-path scratch (split points and safety flags) taken from a fixed
// file-scope device array instead of the context workspace.
// ====================================================================

namespace capssa {
namespace {

// Largest merge (len_x + len_y) the static scratch serves: 2^24 records.
constexpr uint64_t kNoAllocMaxRecords = 1ull << 24;
constexpr uint64_t kNoAllocMaxSegs = kNoAllocMaxRecords / kMergeSeg;  // 131072
constexpr size_t kNoAllocSplitBytes = (kNoAllocMaxSegs + 1) * 8;
constexpr size_t kNoAllocSafeOff = (kNoAllocSplitBytes + 255) & ~size_t(255);
constexpr size_t kNoAllocFlagOff = (kNoAllocSafeOff + kNoAllocMaxSegs + 1 + 255) & ~size_t(255);
constexpr size_t kNoAllocScratchBytes = kNoAllocFlagOff + 256;  // about 1.2 MiB

// Held by every GPU that loads the library until the process exits.  Every
// call shares it and it keeps the last call's contents.
static __device__ __align__(256) unsigned char g_noalloc_merge_scratch[kNoAllocScratchBytes];

// Device address of the scratch array in the current context.  The
// host-side symbol is only a stand-in, never a device address, and the
// address belongs to the context that loaded this module: it is looked up
// on every call (after the first call on a device, which loads the module,
// this is a runtime table lookup), so a reset device or another current
// context never sees a stale address.
cudaError_t noalloc_scratch(unsigned char **out) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_merge_scratch);
    if (e != cudaSuccess) return e;
    *out = (unsigned char *)p;
    return cudaSuccess;
}

// Contract checks the reference makes by panicking: positions <= n and
// SegmentedText ends strictly increasing with the last one equal to n.
__global__ void noalloc_check_kernel(const uint32_t *__restrict__ x, uint64_t lx,
                                     const uint32_t *__restrict__ y, uint64_t ly, uint64_t n,
                                     const uint64_t *__restrict__ ends, uint64_t n_ends,
                                     uint32_t *__restrict__ bad) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < lx + ly + n_ends;
         i += stride) {
        bool ok;
        if (i < lx)
            ok = x[i] <= n;
        else if (i < lx + ly)
            ok = y[i - lx] <= n;
        else {
            uint64_t e = i - lx - ly;
            ok = (e == 0 || ends[e - 1] < ends[e]) && (e + 1 < n_ends || ends[e] == n);
        }
        if (!ok) atomicExch(bad, 1u);
    }
}

}  // namespace
}  // namespace capssa

extern "C" capssa_status capssa_merge_noalloc_u8_u32(
    void *cuda_stream, const uint8_t *text, uint64_t n, const uint64_t *ends, uint64_t n_ends,
    int32_t boundary, const uint32_t *x, const uint32_t *lcp_x, uint64_t len_x,
    const uint32_t *y, const uint32_t *lcp_y, uint64_t len_y, uint64_t max_context, uint32_t *z,
    uint32_t *lcp_z) {
    using namespace capssa;
    // refuse oversize merges before any work, without letting the sum wrap
    if (len_x > kNoAllocMaxRecords || len_y > kNoAllocMaxRecords - len_x) return CAPSSA_EINVAL;
    const uint64_t total = len_x + len_y;
    if (total == 0) return CAPSSA_OK;
    if (boundary != CAPSSA_SHORTER_FIRST && boundary != CAPSSA_LONGER_FIRST) return CAPSSA_EINVAL;
    if (!text || !z || !lcp_z || (len_x && (!x || !lcp_x)) || (len_y && (!y || !lcp_y)) ||
        (n_ends && !ends))
        return CAPSSA_EINVAL;
    cudaStream_t stream = (cudaStream_t)cuda_stream;
    // an error the caller left pending is theirs: report it without clearing
    // it, so that every error read after the launches below is this call's
    if (cudaPeekAtLastError() != cudaSuccess) return CAPSSA_ECUDA;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return CAPSSA_ECUDA;
    unsigned char *scratch = nullptr;
    if (noalloc_scratch(&scratch) != cudaSuccess) return CAPSSA_ECUDA;
    uint64_t *split = (uint64_t *)scratch;
    uint8_t *safe = scratch + kNoAllocSafeOff;
    uint32_t *bad = (uint32_t *)(scratch + kNoAllocFlagOff);

    // the flag keeps the previous call's value: clear it first
    if (cudaMemsetAsync(bad, 0, 4, stream) != cudaSuccess) return CAPSSA_ECUDA;
    noalloc_check_kernel<<<256, 256, 0, stream>>>(x, len_x, y, len_y, n, ends, n_ends, bad);
    uint32_t h_bad = 0;
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpyAsync(&h_bad, bad, 4, cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
        cudaStreamSynchronize(stream) != cudaSuccess)
        return CAPSSA_ECUDA;
    if (h_bad) return CAPSSA_EINVAL;

    if (len_x == 0 || len_y == 0) {
        const uint32_t *src = len_x ? x : y, *ls = len_x ? lcp_x : lcp_y;
        if (cudaMemcpyAsync(z, src, total * 4, cudaMemcpyDeviceToDevice, stream) != cudaSuccess ||
            cudaMemcpyAsync(lcp_z, ls, total * 4, cudaMemcpyDeviceToDevice, stream) != cudaSuccess ||
            cudaStreamSynchronize(stream) != cudaSuccess)
            return CAPSSA_ECUDA;
        return CAPSSA_OK;
    }
    DevLimits L{};
    L.n = n;
    L.longer_first = boundary == CAPSSA_LONGER_FIRST;
    if (n_ends) {  // SegmentedText without the coarse directory: binary search over ends
        L.segmented = 1;
        L.ends = ends;
        L.n_ends = n_ends;
    }
    const uint64_t nseg = (total + kMergeSeg - 1) / kMergeSeg;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    unsigned g = grid_for(nseg + 1, 128, (unsigned)(sms > 0 ? sms : 1) * 16);
    merge_split_kernel<uint32_t><<<g, 128, 0, stream>>>(text, 1, L, x, len_x, y, len_y,
                                                        max_context, nseg, split, safe);
    merge_seg_kernel<uint32_t><<<g, 128, 0, stream>>>(text, 1, L, x, lcp_x, len_x, y, lcp_y,
                                                      len_y, max_context, nseg, split, safe, z,
                                                      lcp_z);
    if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(stream) != cudaSuccess)
        return CAPSSA_ECUDA;
    return CAPSSA_OK;
}
