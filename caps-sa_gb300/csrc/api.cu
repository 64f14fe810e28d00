// api.cu — the C ABI (include/capssa.h): contexts, workspace, staging of
// host/device buffers, and the exported entry points.
#include <algorithm>
#include <cmath>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "common.cuh"
#include "cdf.cuh"
#include "engine.cuh"
#include "scan.cuh"
#include "lcp.cuh"
#include "radix.cuh"

namespace capssa {

capssa_status presence_u8(Ctx &c, const uint8_t *text, uint64_t n, uint32_t *present);

void *ws_get(Ctx &c, int slot, size_t bytes) {
    if (bytes == 0) bytes = 64;
    if (c.sizes[slot] >= bytes) return c.bufs[slot];
    if (c.bufs[slot]) {
        cudaStreamSynchronize(c.stream);
        cudaFree(c.bufs[slot]);
        c.bufs[slot] = nullptr;
        c.sizes[slot] = 0;
    }
    // grow with headroom so repeated calls of similar size do not realloc
    size_t want = bytes + bytes / 8 + 256;
    void *p = nullptr;
    if (cudaMalloc(&p, want) != cudaSuccess) {
        cudaGetLastError();
        want = bytes;
        if (cudaMalloc(&p, want) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
    }
    c.bufs[slot] = p;
    c.sizes[slot] = want;
    return p;
}

capssa_status set_err(Ctx &c, capssa_status s, const std::string &msg) {
    if (c.err.empty()) c.err = msg;
    return s;
}

capssa_status cuda_err(Ctx &c, cudaError_t e, const char *where) {
    std::string m = std::string("CUDA error in ") + where + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation) return set_err(c, CAPSSA_ENOMEM, m);
    return set_err(c, CAPSSA_ECUDA, m);
}

capssa_status check_dev_flags(Ctx &c) {
    int h[2] = {0, 0};
    CAPSSA_CUDA(c, cudaMemcpyAsync(h, c.d_flags, 4, cudaMemcpyDeviceToHost, c.stream));
    CAPSSA_CUDA(c, cudaStreamSynchronize(c.stream));
    if (h[0] == DEV_LOOKBACK_TIMEOUT)
        return set_err(c, CAPSSA_ETIMEOUT, "a device-side wait exceeded its limit");
    if (h[0] != DEV_OK) return set_err(c, CAPSSA_ECUDA, "device error flag set");
    return CAPSSA_OK;
}

// Key geometry for b bits per symbol on a text of n symbols.  Symbols past
// log2(n) / H + 3 (H the symbols' entropy) rarely separate random suffixes, so the key keeps only
// as many symbols as fit in the radix passes that this minimum needs (DNA
// at n = 2^28: 17 symbols + a flag = 35 bits, 5 passes), with the position
// packed below it when key and position fit 64 bits.  Otherwise the widest
// key holds kmax symbols (kmax*b + bits(kmax) <= 64) and a length field.
KeyGeom key_geom(int b, uint64_t n, bool plain, double hbits, int top_bits, uint64_t n_k,
                 bool allow_flagless, bool seg_flag) {
    KeyGeom g{};
    g.b = b < 1 ? 1 : b;
    if (n_k == 0 || n_k > n) n_k = n;
    int logn = 0;
    while (logn < 64 && (n_k >> logn) > 1) logn++;
    // log2(n) / H + 3 symbols (H = symbol entropy in bits, <= b): random
    // suffixes then tie in about n / 2^(3H+1) pairs, which the refinement
    // resolves cheaply
    const double h = hbits > 0.25 ? (hbits < g.b ? hbits : (double)g.b) : 0.25;
    const int kmin = (int)std::ceil((double)logn / h - 1e-9) + 3;
    // the position rides below the key when both fit in 64 bits; a plain
    // text then marks its k-1 short suffixes with one flag bit instead of a
    // length field (they are refined from depth 0)
    // position bits below the key: segment-local positions when a segment
    // index rides above it (the index recovers the global position)
    const uint64_t npos = top_bits ? n_k : n;
    int vbits = 1;
    while (vbits < 32 && (1ull << vbits) < npos) vbits++;
    if (plain && top_bits == 0 && kmin * g.b + 1 + vbits <= 64) {
        const int passes = (kmin * g.b + 1 + 7) / 8;
        // without the flag, one symbol less than kmin (random ties 2^H times
        // likelier, still a few percent) when that saves a whole pass
        const int k2 = kmin - 1;
        const int passes2 = (k2 * g.b + 7) / 8;
        if (allow_flagless && k2 >= 2 && passes2 < passes && k2 * g.b + vbits <= 64 &&
            n >= (1ull << 16)) {
            int k = k2;
            while ((k + 1) * g.b <= 8 * passes2 && (k + 1) * g.b <= 63 &&
                   (k + 1) * g.b + vbits <= 64)
                k++;
            g.k = k;
            g.lbits = 0;
            g.flag_len = 2;
            g.total = k * g.b;
            g.vbits = vbits;
            g.flagless = 1;
            return g;
        }
        int k = kmin;
        while ((k + 1) * g.b + 1 <= 8 * passes && (k + 1) * g.b + 1 + vbits <= 64) k++;
        g.k = k;
        g.lbits = 1;
        g.flag_len = 1;
        g.total = k * g.b + 1;
        g.vbits = vbits;
        return g;
    }
    // segment-major ShorterFirst (many texts in one sort): suffixes from
    // different texts never tie, so the few that end inside the key need only
    // an early-end flag (their groups are refined from depth 0), not a length
    // field; with the flag, one symbol less than kmin when that saves a pass
    if (seg_flag && top_bits) {
        int k = kmin;
        int passes = (top_bits + k * g.b + 1 + 7) / 8;
        const int passes2 = (top_bits + (k - 1) * g.b + 1 + 7) / 8;
        if (k - 1 >= 2 && passes2 < passes && top_bits + (k - 1) * g.b + 1 + vbits <= 64) {
            k--;
            passes = passes2;
        }
        if (top_bits + k * g.b + 1 + vbits <= 64) {
            while (top_bits + (k + 1) * g.b + 1 <= 8 * passes &&
                   top_bits + (k + 1) * g.b + 1 + vbits <= 64)
                k++;
            g.k = k;
            g.lbits = 1;
            g.flag_len = 1;
            g.total = k * g.b + 1;
            g.vbits = vbits;
            g.local_pos = 1;
            return g;
        }
    }
    auto lbits_of = [](int k) {
        int lb = 0;
        while ((1 << lb) <= k) lb++;  // bits of 0..k
        return lb;
    };
    // widest key below the top bits (at least one symbol)
    int kmax = 1;
    for (int k = 1; k * g.b <= 63; k++)
        if (top_bits + k * g.b + lbits_of(k) <= 64) kmax = k;
    int k = kmax;
    if (kmin < kmax) {
        int passes = (top_bits + kmin * g.b + lbits_of(kmin) + 7) / 8;
        // widening never gives up a packed position that fits at kmin (the
        // sort then moves 8 bytes a record instead of 12)
        const bool pos_fits = top_bits + kmin * g.b + lbits_of(kmin) + vbits <= 64;
        k = kmin;
        while (k + 1 <= kmax && top_bits + (k + 1) * g.b + lbits_of(k + 1) <= 8 * passes &&
               (!pos_fits || top_bits + (k + 1) * g.b + lbits_of(k + 1) + vbits <= 64))
            k++;
    }
    g.k = k;
    g.lbits = lbits_of(k);
    g.total = g.k * g.b + g.lbits;
    g.flag_len = 0;
    g.vbits = top_bits + g.total + vbits <= 64 ? vbits : 0;
    g.local_pos = top_bits && g.vbits;
    return g;
}

KeyGeom pf_geom(int b, uint64_t n, bool plain, double hbits, int bucket_bits) {
    KeyGeom g{};
    g.b = b < 1 ? 1 : b;
    int logn = 0;
    while (logn < 64 && (n >> logn) > 1) logn++;
    const double h = hbits > 0.25 ? (hbits < g.b ? hbits : (double)g.b) : 0.25;
    // the same target as key_geom (log2(n) / H + 3 symbols), less the
    // symbols of information the bucket index already carries
    const int ktot = (int)std::ceil((double)logn / h - 1e-9) + 3;
    const int kb = (int)std::floor((double)bucket_bits / h + 1e-9);
    int k = std::max(2, ktot - kb);
    int vbits = 1;
    while (vbits < 32 && (1ull << vbits) < n) vbits++;
    auto lb = [&](int kk) {
        if (plain) return 1;
        int x = 0;
        while ((1 << x) <= kk) x++;
        return x;
    };
    auto bits = [&](int kk) { return bucket_bits + kk * g.b + lb(kk); };
    while (k > 1 && (bits(k) + vbits > 64 || k * g.b > 63)) k--;
    if (bits(k) + vbits > 64 || k * g.b > 63) return g;  // g.k == 0
    const int passes = (bits(k) + 7) / 8;
    while ((k + 1) * g.b <= 63 && bits(k + 1) <= 8 * passes && bits(k + 1) + vbits <= 64) k++;
    g.k = k;
    g.lbits = lb(k);
    g.flag_len = plain ? 1 : 0;
    g.total = k * g.b + g.lbits;
    g.vbits = vbits;
    return g;
}

namespace {

bool is_device_ptr(const void *p) {
    if (!p) return false;
    cudaPointerAttributes attr;
    if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged;
}

double ms_since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

// Copy `bytes` from a host or device buffer into workspace slot `slot`
// (plus `pad` zero bytes); returns the device pointer.
capssa_status stage_in(Ctx &c, int slot, const void *src, size_t bytes, size_t pad, void **out) {
    void *d = ws_get(c, slot, bytes + pad);
    if (!d) return set_err(c, CAPSSA_ENOMEM, "staging buffer");
    if (bytes && d != src) {
        bool dev = is_device_ptr(src);
        auto t0 = std::chrono::steady_clock::now();
        CAPSSA_CUDA(c, cudaMemcpyAsync(d, src, bytes,
                                       dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                       c.stream));
        if (!dev) {
            CAPSSA_CUDA(c, cudaStreamSynchronize(c.stream));
            c.stats.h2d_ms += ms_since(t0);
            c.stats.h2d_bytes += bytes;
        }
    }
    if (pad) CAPSSA_CUDA(c, cudaMemsetAsync((char *)d + bytes, 0, pad, c.stream));
    *out = d;
    return CAPSSA_OK;
}

// Device-resident limits: ends validated like SegmentedText::from_ends
// (src/limits.rs:261-282) and the coarse directory of
// BoundaryDirectory::build (src/limits.rs:210-235).
capssa_status stage_limits(Ctx &c, const capssa_limits *lp, uint64_t n, DevLimits *out) {
    DevLimits L{};
    L.n = n;
    if (lp && (lp->boundary != CAPSSA_SHORTER_FIRST && lp->boundary != CAPSSA_LONGER_FIRST))
        return set_err(c, CAPSSA_EINVAL, "unknown boundary order");
    if (lp && lp->kind != CAPSSA_LIMITS_PLAIN && lp->kind != CAPSSA_LIMITS_SEGMENTED)
        return set_err(c, CAPSSA_EINVAL, "unknown limits kind");
    L.longer_first = lp ? (lp->boundary == CAPSSA_LONGER_FIRST) : 0;
    if (!lp || lp->kind == CAPSSA_LIMITS_PLAIN) {
        *out = L;
        return CAPSSA_OK;
    }
    L.segmented = 1;
    const uint64_t ne = lp->n_ends;
    std::vector<uint64_t> h(ne);
    if (ne) {
        if (!lp->ends) return set_err(c, CAPSSA_EINVAL, "segmented limits without ends");
        if (is_device_ptr(lp->ends)) {
            CAPSSA_CUDA(c, cudaMemcpyAsync(h.data(), lp->ends, ne * 8, cudaMemcpyDeviceToHost,
                                           c.stream));
            CAPSSA_CUDA(c, cudaStreamSynchronize(c.stream));
        } else {
            std::memcpy(h.data(), lp->ends, ne * 8);
        }
    }
    for (uint64_t i = 1; i < ne; i++)
        if (!(h[i - 1] < h[i]))
            return set_err(c, CAPSSA_EINVAL, "SegmentedText::from_ends: ends must be strictly increasing");
    if (ne == 0 ? n != 0 : h[ne - 1] != n)
        return set_err(c, CAPSSA_EINVAL, "SegmentedText::from_ends: last end != text length");
    std::vector<uint32_t> dir;
    uint32_t shift = 0;
    if (ne >= 256 && ne <= 0xFFFFFFFFull && n > 0) {
        uint64_t target = std::min<uint64_t>(std::max<uint64_t>(ne * 2, 1), 2000000);
        uint64_t min_block = (n + target - 1) / target;
        uint64_t bs = 1;
        while (bs < min_block) bs <<= 1;
        while ((1ull << shift) < bs) shift++;
        uint64_t nb = (n + bs - 1) / bs;
        dir.resize(nb + 1);
        uint64_t e = 0;
        for (uint64_t b = 0; b <= nb; b++) {
            uint64_t bstart = std::min(b * bs, n);
            while (e < ne && h[e] <= bstart) e++;
            dir[b] = (uint32_t)e;
        }
    }
    void *d_ends = nullptr;
    capssa_status s = stage_in(c, WS_ENDS, h.data(), ne * 8, 64, &d_ends);
    if (s != CAPSSA_OK) return s;
    L.ends = (const uint64_t *)d_ends;
    L.n_ends = ne;
    if (!dir.empty()) {
        void *d_dir = nullptr;
        s = stage_in(c, WS_DIR, dir.data(), dir.size() * 4, 64, &d_dir);
        if (s != CAPSSA_OK) return s;
        L.dir = (const uint32_t *)d_dir;
        L.n_dir = dir.size();
        L.block_shift = shift;
    }
    CAPSSA_CUDA(c, cudaStreamSynchronize(c.stream));  // host vectors go out of scope
    *out = L;
    return CAPSSA_OK;
}

struct CallScope {
    Ctx &c;
    explicit CallScope(Ctx &cc) : c(cc) {
        c.err.clear();
        c.stats = capssa_stats{};
        c.launches = 0;
        cudaSetDevice(c.device);
        cudaMemsetAsync(c.d_flags, 0, 16, c.stream);
        cudaEventRecord(c.ev0, c.stream);
    }
    capssa_status finish(capssa_status s) {
        if (s == CAPSSA_OK) s = check_dev_flags(c);
        cudaEventRecord(c.ev1, c.stream);
        cudaEventSynchronize(c.ev1);
        float ms = 0;
        cudaEventElapsedTime(&ms, c.ev0, c.ev1);
        c.stats.device_ms = ms;
        c.stats.kernel_launches = c.launches;
        cudaError_t e = cudaGetLastError();
        if (s == CAPSSA_OK && e != cudaSuccess) s = cuda_err(c, e, "call");
        return s;
    }
};

// Deliver a device result to a host or device destination.
capssa_status stage_out(Ctx &c, void *dst, const void *dsrc, size_t bytes) {
    if (!bytes || dst == dsrc) return CAPSSA_OK;
    bool dev = is_device_ptr(dst);
    auto t0 = std::chrono::steady_clock::now();
    CAPSSA_CUDA(c, cudaMemcpyAsync(dst, dsrc, bytes,
                                   dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                                   c.stream));
    if (!dev) {
        CAPSSA_CUDA(c, cudaStreamSynchronize(c.stream));
        c.stats.d2h_ms += ms_since(t0);
        c.stats.d2h_bytes += bytes;
    }
    return CAPSSA_OK;
}

template <typename ST>
capssa_status stage_text(Ctx &c, const ST *text, uint64_t n, void **d_text) {
    return stage_in(c, WS_TEXT, text, n * sizeof(ST), 64 + sizeof(ST) * 8, d_text);
}

// The sample sort's partition plan, requested from a build (see
// capssa_sample_sort_plan_*).
struct PartRequest {
    uint32_t p;
    int mode;
    uint64_t *pivots;  // host, p - 1
    uint64_t *sizes;   // host, p
};

// Every builder funnels through here.
template <typename ST>
capssa_status build_common(Ctx &c, const ST *text, uint64_t n, const void *positions,
                           int pos_bytes, uint64_t m, const capssa_limits *lp,
                           const capssa_opts *opts, void *out_sa, int out_bytes, void *out_lcp,
                           const PartRequest *part = nullptr, uint64_t seg_major_len = 0,
                           const uint32_t *keep_bits = nullptr, bool in_memory = false) {
    if (!text && n) return set_err(c, CAPSSA_EINVAL, "null text");
    if (opts && (opts->tie_order < CAPSSA_TIES_POSITION || opts->tie_order > CAPSSA_TIES_REFERENCE))
        return set_err(c, CAPSSA_EINVAL, "unknown tie order");
    const bool chosen = positions || keep_bits;  // a subset, m suffixes
    if (!out_sa && (chosen ? m : n)) return set_err(c, CAPSSA_EINVAL, "null output");
    if (out_bytes == 4 && n > 0xFFFFFFFFull)
        return set_err(c, CAPSSA_EINVAL, "u32 index cannot address this text");
    uint64_t max_ctx = opts ? opts->max_context : CAPSSA_UNBOUNDED;
    DevLimits L{};
    capssa_status s = stage_limits(c, lp, n, &L);
    if (s != CAPSSA_OK) return s;
    void *d_text = nullptr;
    s = stage_text(c, text, n, &d_text);
    if (s != CAPSSA_OK) return s;
    const uint64_t count = chosen ? m : n;
    void *d_pos = nullptr;
    if (positions && m) {
        s = stage_in(c, WS_POS_IN, positions, m * (size_t)pos_bytes, 64, &d_pos);
        if (s != CAPSSA_OK) return s;
    }
    bool out_dev = is_device_ptr(out_sa);
    void *d_out = out_sa;
    if (!out_dev && count) {
        d_out = ws_get(c, WS_OUT, count * (size_t)out_bytes + 64);
        if (!d_out) return set_err(c, CAPSSA_ENOMEM, "output buffer");
    }
    void *d_lcp = nullptr;
    bool lcp_dev = out_lcp && is_device_ptr(out_lcp);
    if (out_lcp) {
        d_lcp = lcp_dev ? out_lcp : ws_get(c, WS_OUT2, count * (size_t)out_bytes + 64);
        if (!d_lcp) return set_err(c, CAPSSA_ENOMEM, "lcp buffer");
    }
    EngineArgs a{};
    a.text = d_text;
    a.sym_bytes = (int)sizeof(ST);
    a.n = n;
    a.lim = L;
    a.max_ctx = max_ctx;
    a.positions = positions ? d_pos : nullptr;
    a.pos_bytes = pos_bytes;
    a.keep_bits = keep_bits;
    a.m = m;
    a.out_sa = d_out;
    a.out_bytes = out_bytes;
    a.out_lcp = d_lcp;
    a.seg_major = seg_major_len ? 1 : 0;
    a.seg_max_len = seg_major_len;
    if (part) {
        a.part_p = part->p;
        a.part_mode = part->mode;
        a.part_pivots = part->pivots;
        a.part_sizes = part->sizes;
        a.part_first = !opts || opts->sampling != CAPSSA_SAMPLING_REFERENCE ? 1 : 0;
    }
    // the merge sort's tie order belongs to the in-memory builders
    a.tie_ref = in_memory && opts && opts->tie_order == CAPSSA_TIES_REFERENCE ? 1 : 0;
    if (positions && m == 0) return CAPSSA_OK;
    s = engine_build(c, a);
    if (s != CAPSSA_OK) return s;
    s = check_dev_flags(c);
    if (s != CAPSSA_OK) return s;
    if (!out_dev) {
        s = stage_out(c, out_sa, d_out, count * (size_t)out_bytes);
        if (s != CAPSSA_OK) return s;
    }
    if (out_lcp && !lcp_dev) {
        s = stage_out(c, out_lcp, d_lcp, count * (size_t)out_bytes);
        if (s != CAPSSA_OK) return s;
    }
    return CAPSSA_OK;
}

// The partition a sample-sort call asked for (AUTO: splitter search).
int part_mode(const capssa_opts *opts) {
    if (opts && (opts->partition == CAPSSA_PARTITION_LEARNED ||
                 opts->partition == CAPSSA_PARTITION_BISECT))
        return opts->partition;
    return CAPSSA_PARTITION_SPLITTERS;
}

// effective_subproblem_count (src/ext_mem.rs:1159-1178)
uint64_t effective_p(uint64_t n, uint64_t requested, int threads) {
    if (n == 0) return 0;
    uint64_t raw;
    if (requested == 0) {
        uint64_t nt = threads > 0 ? (uint64_t)threads
                                  : std::max<uint64_t>(1, std::thread::hardware_concurrency());
        uint64_t from_size = (n + 65535) / 65536;
        raw = std::min<uint64_t>(std::max<uint64_t>(from_size, nt), 8192);
    } else {
        raw = requested;
    }
    return std::min<uint64_t>(std::max<uint64_t>(raw, 1), n);
}

// Streams `count` device positions to `emit` in batches of 4 Mi (32 MiB),
// each batch copied to pinned memory while the previous one is consumed.
capssa_status emit_stream(Ctx &c, const uint64_t *d_sa, uint64_t count, capssa_emit_fn emit,
                          void *user) {
    capssa_status s = CAPSSA_OK;
    const uint64_t batch = 1u << 22;
    if (!c.h_emit) CAPSSA_CUDA(c, cudaMallocHost(&c.h_emit, 2 * batch * 8));
    uint64_t *h = c.h_emit;
    cudaEvent_t done[2];
    cudaEventCreateWithFlags(&done[0], cudaEventDisableTiming);
    cudaEventCreateWithFlags(&done[1], cudaEventDisableTiming);
    auto t0 = std::chrono::steady_clock::now();
    uint64_t nb = (count + batch - 1) / batch;
    auto issue = [&](uint64_t b) {
        uint64_t off = b * batch, len = std::min(batch, count - off);
        cudaMemcpyAsync(h + (b & 1) * batch, d_sa + off, len * 8, cudaMemcpyDeviceToHost, c.stream);
        cudaEventRecord(done[b & 1], c.stream);
    };
    issue(0);
    for (uint64_t b = 0; b < nb && s == CAPSSA_OK; b++) {
        if (b + 1 < nb) issue(b + 1);
        cudaEventSynchronize(done[b & 1]);
        uint64_t off = b * batch, len = std::min(batch, count - off);
        c.stats.d2h_bytes += len * 8;
        if (emit(user, h + (b & 1) * batch, len) != 0)
            s = set_err(c, CAPSSA_EEMIT, "emit callback aborted the build");
    }
    cudaStreamSynchronize(c.stream);
    c.stats.d2h_ms += ms_since(t0);
    cudaEventDestroy(done[0]);
    cudaEventDestroy(done[1]);
    return s;
}

// Sample-sort builders: the suffix order on the device, delivered to the
// caller's emit callback in batches, each batch copied while the previous
// one is being consumed.
template <typename ST>
capssa_status sample_sort_common(Ctx &c, const ST *text, uint64_t n, const uint64_t *positions,
                                 uint64_t m, const capssa_limits *lp, const capssa_opts *opts,
                                 capssa_emit_fn emit, void *user) {
    if (!emit) return set_err(c, CAPSSA_EINVAL, "null emit callback");
    const uint64_t count = positions ? m : n;
    if (count == 0) return CAPSSA_OK;
    uint64_t *d_sa = (uint64_t *)ws_get(c, WS_OUT, count * 8 + 64);
    if (!d_sa) return set_err(c, CAPSSA_ENOMEM, "output buffer");
    PartRequest pr{(uint32_t)effective_p(count, opts ? opts->subproblem_count : 0,
                                         opts ? opts->host_threads : 0),
                   part_mode(opts),
                   nullptr, nullptr};
    capssa_status s =
        build_common<ST>(c, text, n, positions, 8, m, lp, opts, d_sa, 8, nullptr, &pr);
    if (s != CAPSSA_OK) return s;
    return emit_stream(c, d_sa, count, emit, user);
}

// build_ext_mem* (src/ext_mem.rs:279-553): the same suffix order streamed
// to `emit`.  The reference spills partition buckets to temp files to bound
// host RAM; here the whole working set (under 50 bytes per suffix, so under
// 200 GB for the largest supported text) lives in device memory and the
// host holds only the text and the two emit batches, so there is nothing
// to spill and no partition plan to compute.
template <typename ST>
capssa_status ext_mem_common(Ctx &c, const ST *text, uint64_t n, const void *positions,
                             int pos_bytes, uint64_t m, const capssa_limits *lp,
                             const capssa_opts *opts, capssa_emit_fn emit, void *user,
                             const uint32_t *keep_bits = nullptr) {
    if (!emit) return set_err(c, CAPSSA_EINVAL, "null emit callback");
    const uint64_t count = (positions || keep_bits) ? m : n;
    if (count == 0) return CAPSSA_OK;
    uint64_t *d_sa = (uint64_t *)ws_get(c, WS_OUT, count * 8 + 64);
    if (!d_sa) return set_err(c, CAPSSA_ENOMEM, "output buffer");
    capssa_status s = build_common<ST>(c, text, n, positions, pos_bytes, m, lp, opts, d_sa, 8,
                                       nullptr, nullptr, 0, keep_bits);
    if (s != CAPSSA_OK) return s;
    return emit_stream(c, d_sa, count, emit, user);
}

// Segment-major global order -> per-text positions: slot i belongs to the
// text t with offs[t] <= i < offs[t + 1] (empty texts own no slot), and so
// does the position it holds.
template <typename IT>
__global__ void localize_kernel(const uint32_t *__restrict__ sa, uint32_t n,
                                const uint64_t *__restrict__ offs, uint64_t n_texts,
                                IT *__restrict__ out) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint64_t lo = 0, hi = n_texts;  // last t with offs[t] <= i
        while (hi - lo > 1) {
            uint64_t mid = (lo + hi) >> 1;
            if (__ldg(offs + mid) <= i)
                lo = mid;
            else
                hi = mid;
        }
        out[i] = (IT)(sa[i] - __ldg(offs + lo));
    }
}

// Positions kept by the symbol range [lo, hi), one bit each (a warp ballot
// per 32 positions), and their count.
template <typename ST>
__global__ void filter_bits_kernel(const ST *__restrict__ text, uint64_t n, uint64_t lo,
                                   uint64_t hi, uint32_t *__restrict__ bits,
                                   unsigned long long *__restrict__ count) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const uint64_t words = (n + 31) / 32;
    unsigned long long kept = 0;
    for (uint64_t w = warp; w < words; w += nwarps) {
        const uint64_t p = w * 32 + lane;
        bool keep = false;
        if (p < n) {
            const uint64_t v = (uint64_t)text[p];
            keep = v >= lo && v < hi;
        }
        const unsigned b = __ballot_sync(0xffffffffu, keep);
        if (lane == 0) {
            bits[w] = b;
            kept += (unsigned long long)__popc(b);
        }
    }
    if (lane == 0 && kept) atomicAdd(count, kept);
}

template <typename ST>
capssa_status filter_common(Ctx &c, const ST *text, uint64_t n, uint64_t lo, uint64_t hi,
                            const capssa_limits *lp, const capssa_opts *opts, void *out_sa,
                            int out_bytes, uint64_t *m_out, capssa_emit_fn emit = nullptr,
                            void *user = nullptr) {
    if (!m_out) return set_err(c, CAPSSA_EINVAL, "null count output");
    *m_out = 0;
    if (n == 0) return CAPSSA_OK;
    if (!text) return set_err(c, CAPSSA_EINVAL, "null text");
    if (n > 0xFFFFFFFEull) return set_err(c, CAPSSA_EUNSUPPORTED, "texts of 2^32-1 or more symbols");
    void *d_text = nullptr;
    capssa_status s = stage_text(c, text, n, &d_text);
    if (s != CAPSSA_OK) return s;
    // the kept positions as a bitmap (n / 8 bytes); the engine takes the kept
    // suffixes from the full order, no position list is built
    uint32_t *bits = (uint32_t *)ws_get(c, WS_KEEP, (n / 32 + 2) * 4 + 64);
    if (!bits) return set_err(c, CAPSSA_ENOMEM, "filter workspace");
    unsigned long long *cnt = (unsigned long long *)(c.d_flags + 4);
    CAPSSA_CUDA(c, cudaMemsetAsync(cnt, 0, 8, c.stream));
    filter_bits_kernel<ST><<<std::min<unsigned>(grid_for((n + 31) / 32 * 32, 256),
                                                 (unsigned)c.sm_count * 16),
                             256, 0, c.stream>>>((const ST *)d_text, n, lo, hi, bits, cnt);
    CAPSSA_LAUNCHED(c);
    unsigned long long *h_cnt = (unsigned long long *)c.h_scratch;
    CAPSSA_CUDA(c, cudaMemcpyAsync(h_cnt, cnt, 8, cudaMemcpyDeviceToHost, c.stream));
    CAPSSA_CUDA(c, cudaStreamSynchronize(c.stream));
    const uint64_t m = *h_cnt;
    *m_out = m;
    if ((!out_sa && !emit) || m == 0) return CAPSSA_OK;
    if (emit)
        return ext_mem_common<ST>(c, (const ST *)d_text, n, nullptr, 4, m, lp, opts, emit, user,
                                  bits);
    return build_common<ST>(c, (const ST *)d_text, n, nullptr, 4, m, lp, opts, out_sa, out_bytes,
                            nullptr, nullptr, 0, bits);
}

// Many texts: one segmented sort of the concatenation in segment-major
// order (the text index above the key bits), so every text's suffixes come
// out contiguous and in that text's own order (within one text the
// segmented comparator is exactly PlainText's); positions are then made
// local.
template <typename ST>
capssa_status batched_common(Ctx &c, const ST *texts, const uint64_t *offsets, uint64_t n_texts,
                             const capssa_opts *opts, void *out_sa, int out_bytes) {
    if (n_texts == 0) return CAPSSA_OK;
    if (!offsets) return set_err(c, CAPSSA_EINVAL, "null offsets");
    std::vector<uint64_t> off(n_texts + 1);
    if (is_device_ptr(offsets)) {
        CAPSSA_CUDA(c, cudaMemcpy(off.data(), offsets, (n_texts + 1) * 8, cudaMemcpyDeviceToHost));
    } else {
        std::memcpy(off.data(), offsets, (n_texts + 1) * 8);
    }
    if (off[0] != 0) return set_err(c, CAPSSA_EINVAL, "offsets[0] must be 0");
    for (uint64_t t = 0; t < n_texts; t++)
        if (off[t + 1] < off[t]) return set_err(c, CAPSSA_EINVAL, "offsets must not decrease");
    const uint64_t n = off[n_texts];
    if (n == 0) return CAPSSA_OK;
    if (n > 0xFFFFFFFEull) return set_err(c, CAPSSA_EUNSUPPORTED, "texts of 2^32-1 or more symbols");
    std::vector<uint64_t> ends;
    ends.reserve(n_texts);
    uint64_t longest = 0;
    for (uint64_t t = 1; t <= n_texts; t++)
        if (off[t] != off[t - 1]) {
            ends.push_back(off[t]);
            longest = std::max(longest, off[t] - off[t - 1]);
        }
    capssa_limits lp{CAPSSA_LIMITS_SEGMENTED, CAPSSA_SHORTER_FIRST, ends.data(), ends.size()};
    uint32_t *d_sa = (uint32_t *)ws_get(c, WS_OUT2, n * 4 + 64);
    if (!d_sa) return set_err(c, CAPSSA_ENOMEM, "batched output");
    capssa_opts o;
    capssa_opts_default(&o);
    if (opts) o = *opts;
    o.max_context = CAPSSA_UNBOUNDED;
    capssa_status s =
        build_common<ST>(c, texts, n, nullptr, 4, 0, &lp, &o, d_sa, 4, nullptr, nullptr, longest);
    if (s != CAPSSA_OK) return s;
    void *d_off = nullptr;
    s = stage_in(c, WS_MISC3, off.data(), off.size() * 8, 64, &d_off);
    if (s != CAPSSA_OK) return s;
    // the text index and one symbol must share the 64-bit key
    if (!c.seg_major_done)
        return set_err(c, CAPSSA_EUNSUPPORTED, "too many texts for this alphabet width");
    const bool out_dev = is_device_ptr(out_sa);
    void *dst = out_dev ? out_sa : ws_get(c, WS_OUT, n * out_bytes + 64);
    if (!dst) return set_err(c, CAPSSA_ENOMEM, "batched output");
    if (out_bytes == 4)
        localize_kernel<uint32_t><<<grid_for(n, 256), 256, 0, c.stream>>>(
            d_sa, (uint32_t)n, (const uint64_t *)d_off, n_texts, (uint32_t *)dst);
    else
        localize_kernel<uint64_t><<<grid_for(n, 256), 256, 0, c.stream>>>(
            d_sa, (uint32_t)n, (const uint64_t *)d_off, n_texts, (uint64_t *)dst);
    CAPSSA_LAUNCHED(c);
    if (!out_dev) return stage_out(c, out_sa, dst, n * out_bytes);
    return CAPSSA_OK;
}

}  // namespace

// Failure-detection self-test: waits on a status word that nothing sets,
// with the same bounded polling as every look-back, then records
// DEV_LOOKBACK_TIMEOUT (the host call returns CAPSSA_ETIMEOUT).
__global__ void bounded_wait_kernel(const unsigned long long *word, uint32_t polls, int *err) {
    if (threadIdx.x != 0) return;
    for (uint32_t i = 0; i < polls; i++) {
        if (*(const volatile unsigned long long *)word != 0ull) return;
        __nanosleep(64);
    }
    atomicCAS(err, DEV_OK, DEV_LOOKBACK_TIMEOUT);
}

__global__ void pack_keys_kernel(const uint8_t *__restrict__ text, uint64_t n,
                                 const uint8_t *__restrict__ code, uint32_t bits, uint32_t k,
                                 uint32_t alphabet, DevLimits L, const uint64_t *__restrict__ pos,
                                 uint64_t m, uint64_t *__restrict__ keys) {
    // Packer::key_at_bounded (src/pack.rs:187-203)
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t p = pos[i];
        uint64_t lim = dev_lim_at(L, p);
        uint64_t take = k;
        if (lim < take) take = lim;
        if (n - p < take) take = n - p;
        uint64_t bias = L.longer_first ? 0 : 1, pad = L.longer_first ? alphabet : 0;
        uint64_t key = 0;
        for (uint64_t j = 0; j < take; j++) key = (key << bits) | ((uint64_t)code[text[p + j]] + bias);
        for (uint64_t j = take; j < k; j++) key = (key << bits) | pad;
        keys[i] = key;
    }
}

}  // namespace capssa

using namespace capssa;

// ===================================================================== C ABI

extern "C" {

void capssa_opts_default(capssa_opts *o) {
    std::memset(o, 0, sizeof(*o));
    o->max_context = CAPSSA_UNBOUNDED;
}

int capssa_abi_version(void) { return CAPSSA_ABI_VERSION; }

capssa_status capssa_ctx_create(capssa_ctx **out, int device) {
    if (!out) return CAPSSA_EINVAL;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return CAPSSA_ECUDA;
    }
    if (device < 0 || device >= count) return CAPSSA_EINVAL;
    Ctx *c = new (std::nothrow) Ctx();
    if (!c) return CAPSSA_ENOMEM;
    c->device = device;
    if (cudaSetDevice(device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&c->d_flags, 64) != cudaSuccess ||
        cudaMallocHost(&c->h_scratch, 1 << 16) != cudaSuccess ||
        cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess ||
        [&] {
            for (auto &e : c->pev)
                if (cudaEventCreate(&e) != cudaSuccess) return true;
            for (auto &e : c->kev)
                if (cudaEventCreate(&e) != cudaSuccess) return true;
            for (auto &e : c->tune_ev)
                if (cudaEventCreate(&e) != cudaSuccess) return true;
            for (auto &st : c->side)
                if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess)
                    return true;
            if (cudaEventCreateWithFlags(&c->fork_ev, cudaEventDisableTiming) != cudaSuccess)
                return true;
            for (auto &e : c->join_ev)
                if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
                    return true;
            return false;
        }()) {
        cudaGetLastError();
        delete c;
        return CAPSSA_ECUDA;
    }
    c->own_stream = true;
    cudaMemset(c->d_flags, 0, 64);
    cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
    *out = reinterpret_cast<capssa_ctx *>(c);
    return CAPSSA_OK;
}

void capssa_ctx_trim(capssa_ctx *ctx) {
    if (!ctx) return;
    Ctx *c = reinterpret_cast<Ctx *>(ctx);
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    for (int i = 0; i < WS_NSLOTS; i++) {
        if (c->bufs[i]) cudaFree(c->bufs[i]);
        c->bufs[i] = nullptr;
        c->sizes[i] = 0;
    }
    if (c->h_emit) cudaFreeHost(c->h_emit);
    c->h_emit = nullptr;
}

void capssa_ctx_destroy(capssa_ctx *ctx) {
    if (!ctx) return;
    Ctx *c = reinterpret_cast<Ctx *>(ctx);
    capssa_ctx_trim(ctx);
    if (c->d_flags) cudaFree(c->d_flags);
    if (c->h_scratch) cudaFreeHost(c->h_scratch);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    for (auto &e : c->pev)
        if (e) cudaEventDestroy(e);
    for (auto &e : c->kev)
        if (e) cudaEventDestroy(e);
    for (auto &e : c->tune_ev)
        if (e) cudaEventDestroy(e);
    for (auto &st : c->side)
        if (st) cudaStreamDestroy(st);
    if (c->fork_ev) cudaEventDestroy(c->fork_ev);
    for (auto &e : c->join_ev)
        if (e) cudaEventDestroy(e);
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

capssa_status capssa_ctx_set_stream(capssa_ctx *ctx, void *stream) {
    if (!ctx) return CAPSSA_EINVAL;
    Ctx *c = reinterpret_cast<Ctx *>(ctx);
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    if (c->own_stream) cudaStreamDestroy(c->stream);
    if (stream) {
        c->stream = (cudaStream_t)stream;
        c->own_stream = false;
    } else {
        if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess)
            return CAPSSA_ECUDA;
        c->own_stream = true;
    }
    return CAPSSA_OK;
}

const char *capssa_ctx_last_error(const capssa_ctx *ctx) {
    if (!ctx) return "null context";
    return reinterpret_cast<const Ctx *>(ctx)->err.c_str();
}

capssa_status capssa_ctx_stats(const capssa_ctx *ctx, capssa_stats *out) {
    if (!ctx || !out) return CAPSSA_EINVAL;
    *out = reinterpret_cast<const Ctx *>(ctx)->stats;
    return CAPSSA_OK;
}

uint64_t capssa_ctx_workspace_bytes(const capssa_ctx *ctx) {
    if (!ctx) return 0;
    const Ctx *c = reinterpret_cast<const Ctx *>(ctx);
    uint64_t t = 0;
    for (int i = 0; i < WS_NSLOTS; i++) t += c->sizes[i];
    return t;
}

#define CTX_OR_EINVAL(ctx)                                                     \
    if (!ctx) return CAPSSA_EINVAL;                                            \
    Ctx &c = *reinterpret_cast<Ctx *>(ctx);                                    \
    CallScope scope(c);

#define DEFINE_FOR_I(S, ST, I, IT, IB)                                                        \
    capssa_status capssa_build_in_memory_for_filter_##S##_##I(                                \
        capssa_ctx *ctx, const ST *text, uint64_t n, uint64_t lo, uint64_t hi,                \
        const capssa_limits *lp, const capssa_opts *opts, IT *out_sa, uint64_t *m_out) {      \
        CTX_OR_EINVAL(ctx);                                                                   \
        return scope.finish(filter_common<ST>(c, text, n, lo, hi, lp, opts, out_sa, IB,       \
                                              m_out));                                        \
    }                                                                                         \
    capssa_status capssa_build_in_memory_##S##_##I(capssa_ctx *ctx, const ST *text,           \
                                                   uint64_t n, const capssa_limits *lp,       \
                                                   const capssa_opts *opts, IT *out_sa) {     \
        CTX_OR_EINVAL(ctx);                                                                   \
        return scope.finish(build_common<ST>(c, text, n, nullptr, IB, 0, lp, opts, out_sa, IB, \
                                             nullptr, nullptr, 0, nullptr, true));            \
    }                                                                                         \
    capssa_status capssa_build_in_memory_for_positions_##S##_##I(                             \
        capssa_ctx *ctx, const ST *text, uint64_t n, const IT *positions, uint64_t m,         \
        const capssa_limits *lp, const capssa_opts *opts, IT *out_sa) {                       \
        CTX_OR_EINVAL(ctx);                                                                   \
        if (!positions && m) return scope.finish(set_err(c, CAPSSA_EINVAL, "null positions")); \
        return scope.finish(build_common<ST>(c, text, n, positions ? (const void *)positions   \
                                                                   : (const void *)out_sa,    \
                                             IB, m, lp, opts, out_sa, IB, nullptr, nullptr,   \
                                             0, nullptr, true));                              \
    }                                                                                         \
    capssa_status capssa_build_in_memory_lcp_##S##_##I(                                       \
        capssa_ctx *ctx, const ST *text, uint64_t n, const IT *positions, uint64_t m,         \
        const capssa_limits *lp, const capssa_opts *opts, IT *out_sa, IT *out_lcp) {          \
        CTX_OR_EINVAL(ctx);                                                                   \
        if (!out_lcp) return scope.finish(set_err(c, CAPSSA_EINVAL, "null lcp output"));     \
        return scope.finish(build_common<ST>(c, text, n, positions, IB, positions ? m : 0, lp, \
                                             opts, out_sa, IB, out_lcp, nullptr, 0, nullptr,  \
                                             true));                                          \
    }                                                                                         \
    capssa_status capssa_merge_##S##_##I(                                                     \
        capssa_ctx *ctx, const ST *text, uint64_t n, const capssa_limits *lp, const IT *x,    \
        const IT *lcp_x, uint64_t len_x, const IT *y, const IT *lcp_y, uint64_t len_y,        \
        uint64_t max_context, IT *z, IT *lcp_z) {                                             \
        CTX_OR_EINVAL(ctx);                                                                   \
        return scope.finish(merge_common<ST>(c, text, n, lp, x, lcp_x, len_x, y, lcp_y, len_y, \
                                             max_context, z, lcp_z, IB));                     \
    }                                                                                         \
    capssa_status capssa_build_batched_##S##_##I(capssa_ctx *ctx, const ST *texts,            \
                                                 const uint64_t *offsets, uint64_t n_texts,   \
                                                 const capssa_opts *opts, IT *out_sa) {       \
        CTX_OR_EINVAL(ctx);                                                                   \
        return scope.finish(batched_common<ST>(c, texts, offsets, n_texts, opts, out_sa, IB)); \
    }

#define DEFINE_FOR_S(S, ST)                                                                   \
    DEFINE_FOR_I(S, ST, u32, uint32_t, 4)                                                     \
    DEFINE_FOR_I(S, ST, u64, uint64_t, 8)                                                     \
    capssa_status capssa_sample_sort_plan_##S(capssa_ctx *ctx, const ST *text, uint64_t n,    \
                                              const uint64_t *positions, uint64_t m,          \
                                              const capssa_limits *lp,                        \
                                              const capssa_opts *opts, uint64_t *p_out,       \
                                              uint64_t *pivots, uint64_t *sizes) {            \
        CTX_OR_EINVAL(ctx);                                                                   \
        if (positions == nullptr && m) return scope.finish(set_err(c, CAPSSA_EINVAL, "null positions")); \
        return scope.finish(plan_common<ST>(c, text, n, positions, m, lp, opts, p_out, pivots, \
                                            sizes));                                          \
    }                                                                                         \
    capssa_status capssa_build_ext_mem_##S(capssa_ctx *ctx, const ST *text, uint64_t n,       \
                                           const capssa_limits *lp, const capssa_opts *opts,  \
                                           capssa_emit_fn emit, void *user) {                 \
        CTX_OR_EINVAL(ctx);                                                                   \
        return scope.finish(                                                                  \
            ext_mem_common<ST>(c, text, n, nullptr, 8, 0, lp, opts, emit, user));             \
    }                                                                                         \
    capssa_status capssa_build_ext_mem_for_positions_##S(                                     \
        capssa_ctx *ctx, const ST *text, uint64_t n, const uint64_t *positions, uint64_t m,   \
        const capssa_limits *lp, const capssa_opts *opts, capssa_emit_fn emit, void *user) {  \
        CTX_OR_EINVAL(ctx);                                                                   \
        if (!positions && m) return scope.finish(set_err(c, CAPSSA_EINVAL, "null positions")); \
        if (m == 0) return scope.finish(emit ? CAPSSA_OK : set_err(c, CAPSSA_EINVAL, "null emit callback")); \
        return scope.finish(                                                                  \
            ext_mem_common<ST>(c, text, n, positions, 8, m, lp, opts, emit, user));           \
    }                                                                                         \
    capssa_status capssa_build_ext_mem_for_filter_##S(                                        \
        capssa_ctx *ctx, const ST *text, uint64_t n, uint64_t lo, uint64_t hi,                \
        const capssa_limits *lp, const capssa_opts *opts, capssa_emit_fn emit, void *user,    \
        uint64_t *m_out) {                                                                    \
        CTX_OR_EINVAL(ctx);                                                                   \
        if (!emit) return scope.finish(set_err(c, CAPSSA_EINVAL, "null emit callback"));     \
        uint64_t m_local = 0;                                                                 \
        capssa_status st = filter_common<ST>(c, text, n, lo, hi, lp, opts, nullptr, 8,        \
                                             &m_local, emit, user);                           \
        if (m_out) *m_out = m_local;                                                          \
        return scope.finish(st);                                                              \
    }                                                                                         \
    capssa_status capssa_build_in_memory_sample_sort_##S(                                     \
        capssa_ctx *ctx, const ST *text, uint64_t n, const capssa_limits *lp,                 \
        const capssa_opts *opts, capssa_emit_fn emit, void *user) {                           \
        CTX_OR_EINVAL(ctx);                                                                   \
        return scope.finish(sample_sort_common<ST>(c, text, n, nullptr, 0, lp, opts, emit, user)); \
    }                                                                                         \
    capssa_status capssa_build_in_memory_sample_sort_for_positions_##S(                       \
        capssa_ctx *ctx, const ST *text, uint64_t n, const uint64_t *positions, uint64_t m,   \
        const capssa_limits *lp, const capssa_opts *opts, capssa_emit_fn emit, void *user) {  \
        CTX_OR_EINVAL(ctx);                                                                   \
        if (!positions && m) return scope.finish(set_err(c, CAPSSA_EINVAL, "null positions")); \
        if (m == 0) return scope.finish(CAPSSA_OK);                                           \
        return scope.finish(                                                                  \
            sample_sort_common<ST>(c, text, n, positions, m, lp, opts, emit, user));          \
    }                                                                                         \
    capssa_status capssa_lcp_##S(capssa_ctx *ctx, const ST *text, uint64_t n,                 \
                                 const uint64_t *p, const uint64_t *q, uint64_t count,        \
                                 uint64_t max_context, uint64_t *out) {                       \
        CTX_OR_EINVAL(ctx);                                                                   \
        return scope.finish(pairs_common<ST>(c, text, n, nullptr, p, q, count, max_context,   \
                                             out, nullptr));                                  \
    }                                                                                         \
    capssa_status capssa_suffix_cmp_##S(capssa_ctx *ctx, const ST *text, uint64_t n,          \
                                        const capssa_limits *lp, const uint64_t *p,           \
                                        const uint64_t *q, uint64_t count,                    \
                                        uint64_t max_context, int8_t *out) {                  \
        CTX_OR_EINVAL(ctx);                                                                   \
        return scope.finish(                                                                  \
            pairs_common<ST>(c, text, n, lp, p, q, count, max_context, nullptr, out));        \
    }

}  // extern "C"

namespace capssa {
namespace {

// True when every position (idx_bytes wide, host or device) is <= n.
bool positions_within(Ctx &c, const void *pos, uint64_t count, int idx_bytes, uint64_t n) {
    if (!count) return true;
    std::vector<uint8_t> h(count * idx_bytes);
    const void *src = pos;
    if (is_device_ptr(pos)) {
        if (cudaMemcpyAsync(h.data(), pos, h.size(), cudaMemcpyDeviceToHost, c.stream) !=
                cudaSuccess ||
            cudaStreamSynchronize(c.stream) != cudaSuccess)
            return false;
        src = h.data();
    }
    for (uint64_t i = 0; i < count; i++) {
        uint64_t v = idx_bytes == 4 ? ((const uint32_t *)src)[i] : ((const uint64_t *)src)[i];
        if (v > n) return false;
    }
    return true;
}

template <typename ST>
capssa_status merge_common(Ctx &c, const ST *text, uint64_t n, const capssa_limits *lp,
                           const void *x, const void *lcp_x, uint64_t len_x, const void *y,
                           const void *lcp_y, uint64_t len_y, uint64_t max_ctx, void *z,
                           void *lcp_z, int ib) {
    const uint64_t total = len_x + len_y;
    if (total == 0) return CAPSSA_OK;
    if ((len_x && (!x || !lcp_x)) || (len_y && (!y || !lcp_y)) || !z || !lcp_z)
        return set_err(c, CAPSSA_EINVAL, "null merge buffer");
    if (!positions_within(c, x, len_x, ib, n) || !positions_within(c, y, len_y, ib, n))
        return set_err(c, CAPSSA_EINVAL, "a run position lies beyond the end of the text");
    DevLimits L{};
    capssa_status s = stage_limits(c, lp, n, &L);
    if (s != CAPSSA_OK) return s;
    void *d_text = nullptr;
    s = stage_text(c, text, n, &d_text);
    if (s != CAPSSA_OK) return s;
    void *dx = nullptr, *dlx = nullptr, *dy = nullptr, *dly = nullptr;
    if ((s = stage_in(c, WS_KEYS_A, x, len_x * ib, 64, &dx)) != CAPSSA_OK) return s;
    if ((s = stage_in(c, WS_KEYS_B, lcp_x, len_x * ib, 64, &dlx)) != CAPSSA_OK) return s;
    if ((s = stage_in(c, WS_VALS_A, y, len_y * ib, 64, &dy)) != CAPSSA_OK) return s;
    if ((s = stage_in(c, WS_VALS_B, lcp_y, len_y * ib, 64, &dly)) != CAPSSA_OK) return s;
    void *dz = ws_get(c, WS_OUT, total * ib + 64), *dlz = ws_get(c, WS_OUT2, total * ib + 64);
    if (!dz || !dlz) return set_err(c, CAPSSA_ENOMEM, "merge output");
    s = merge_runs(c, d_text, (int)sizeof(ST), L, dx, dlx, len_x, dy, dly, len_y, max_ctx, dz,
                   dlz, ib);
    if (s != CAPSSA_OK) return s;
    if ((s = stage_out(c, z, dz, total * ib)) != CAPSSA_OK) return s;
    return stage_out(c, lcp_z, dlz, total * ib);
}

template <typename ST>
capssa_status pairs_common(Ctx &c, const ST *text, uint64_t n, const capssa_limits *lp,
                           const uint64_t *p, const uint64_t *q, uint64_t count, uint64_t max_ctx,
                           uint64_t *out_lcp, int8_t *out_cmp) {
    if (count == 0) return CAPSSA_OK;
    if (!p || !q || (!out_lcp && !out_cmp)) return set_err(c, CAPSSA_EINVAL, "null pair buffer");
    std::vector<uint64_t> hp(count), hq(count);
    const uint64_t *pp = p, *qq = q;
    if (is_device_ptr(p)) {
        CAPSSA_CUDA(c, cudaMemcpy(hp.data(), p, count * 8, cudaMemcpyDeviceToHost));
        pp = hp.data();
    }
    if (is_device_ptr(q)) {
        CAPSSA_CUDA(c, cudaMemcpy(hq.data(), q, count * 8, cudaMemcpyDeviceToHost));
        qq = hq.data();
    }
    for (uint64_t i = 0; i < count; i++)
        if (pp[i] > n || qq[i] > n) return set_err(c, CAPSSA_EINVAL, "position beyond the text");
    DevLimits L{};
    capssa_status s = stage_limits(c, lp, n, &L);
    if (s != CAPSSA_OK) return s;
    void *d_text = nullptr;
    if ((s = stage_text(c, text, n, &d_text)) != CAPSSA_OK) return s;
    void *dp = nullptr, *dq = nullptr;
    if ((s = stage_in(c, WS_KEYS_A, pp, count * 8, 64, &dp)) != CAPSSA_OK) return s;
    if ((s = stage_in(c, WS_KEYS_B, qq, count * 8, 64, &dq)) != CAPSSA_OK) return s;
    if (out_lcp) {
        uint64_t *d = (uint64_t *)ws_get(c, WS_OUT, count * 8 + 64);
        if (!d) return set_err(c, CAPSSA_ENOMEM, "lcp output");
        s = lcp_pairs(c, d_text, (int)sizeof(ST), n, (const uint64_t *)dp, (const uint64_t *)dq,
                      count, max_ctx, d);
        if (s != CAPSSA_OK) return s;
        return stage_out(c, out_lcp, d, count * 8);
    }
    int8_t *d = (int8_t *)ws_get(c, WS_OUT, count + 64);
    if (!d) return set_err(c, CAPSSA_ENOMEM, "cmp output");
    s = suffix_cmp_pairs(c, d_text, (int)sizeof(ST), L, (const uint64_t *)dp, (const uint64_t *)dq,
                         count, max_ctx, d);
    if (s != CAPSSA_OK) return s;
    return stage_out(c, out_cmp, d, count);
}

}  // namespace
}  // namespace capssa

extern "C" {
}  // extern "C"

namespace capssa {
namespace {

// capssa_sample_sort_plan_*: p, and with output arrays the pivots and the
// partition sizes of the sample sort's plan.
template <typename ST>
capssa_status plan_common(Ctx &c, const ST *text, uint64_t n, const uint64_t *positions,
                          uint64_t m, const capssa_limits *lp, const capssa_opts *opts,
                          uint64_t *p_out, uint64_t *pivots, uint64_t *sizes) {
    const uint64_t count = positions ? m : n;
    const uint64_t p =
        effective_p(count, opts ? opts->subproblem_count : 0, opts ? opts->host_threads : 0);
    if (p_out) *p_out = p;
    if (!pivots || !sizes || count == 0) return CAPSSA_OK;
    if (p > 0xFFFFFFFFull) return set_err(c, CAPSSA_EUNSUPPORTED, "more than 2^32-1 subproblems");
    uint64_t *d_sa = (uint64_t *)ws_get(c, WS_OUT, count * 8 + 64);
    if (!d_sa) return set_err(c, CAPSSA_ENOMEM, "output buffer");
    PartRequest pr{(uint32_t)p,
                   part_mode(opts),
                   pivots, sizes};
    return build_common<ST>(c, text, n, positions, 8, m, lp, opts, d_sa, 8, nullptr, &pr);
}

}  // namespace
}  // namespace capssa

extern "C" {

DEFINE_FOR_S(u8, uint8_t)
DEFINE_FOR_S(u16, uint16_t)
DEFINE_FOR_S(u32, uint32_t)

capssa_status capssa_selftest_bounded_wait(capssa_ctx *ctx, uint32_t polls) {
    CTX_OR_EINVAL(ctx);
    if (polls == 0 || polls > (1u << 20))
        return scope.finish(set_err(c, CAPSSA_EINVAL, "polls must be 1..2^20"));
    unsigned long long *word = (unsigned long long *)ws_get(c, WS_MISC, 64);
    if (!word) return scope.finish(set_err(c, CAPSSA_ENOMEM, "self-test word"));
    if (cudaMemsetAsync(word, 0, 64, c.stream) != cudaSuccess)
        return scope.finish(set_err(c, CAPSSA_ECUDA, "self-test word clear"));
    bounded_wait_kernel<<<1, 32, 0, c.stream>>>(word, polls, c.d_flags);
    c.launches++;
    return scope.finish(CAPSSA_OK);
}

capssa_status capssa_cdf_grad(capssa_ctx *ctx, const float *params, const uint64_t *prefixes,
                              const float *targets, uint64_t n, float *grad, float *loss) {
    CTX_OR_EINVAL(ctx);
    if (!params || !grad || !loss || (n && (!prefixes || !targets)))
        return scope.finish(set_err(c, CAPSSA_EINVAL, "null model buffer"));
    if (n > 0xFFFFFFFFull) return scope.finish(set_err(c, CAPSSA_EUNSUPPORTED, "2^32 samples"));
    void *dp = nullptr, *dx = nullptr, *dt = nullptr;
    capssa_status s = stage_in(c, WS_MISC, params, cdf::kParams * 4, 64, &dp);
    if (s == CAPSSA_OK) s = stage_in(c, WS_MISC2, prefixes, n * 8, 64, &dx);
    if (s == CAPSSA_OK) s = stage_in(c, WS_MISC3, targets, n * 4, 64, &dt);
    if (s != CAPSSA_OK) return scope.finish(s);
    float *dg = (float *)ws_get(c, WS_OUT2, (cdf::kParams + 1) * 4 + 64);
    if (!dg) return scope.finish(set_err(c, CAPSSA_ENOMEM, "gradient buffer"));
    if (cudaMemsetAsync(dg, 0, (cdf::kParams + 1) * 4, c.stream) != cudaSuccess)
        return scope.finish(set_err(c, CAPSSA_ECUDA, "gradient clear"));
    s = cdf::grad(c, (const float *)dp, (const uint64_t *)dx, (const float *)dt, (uint32_t)n, dg,
                  dg + cdf::kParams);
    if (s == CAPSSA_OK) s = stage_out(c, grad, dg, cdf::kParams * 4);
    float lsum = 0.0f;
    if (s == CAPSSA_OK) s = stage_out(c, &lsum, dg + cdf::kParams, 4);
    if (s == CAPSSA_OK) *loss = n ? lsum / (float)n : 0.0f;
    return scope.finish(s);
}

capssa_status capssa_cdf_infer(capssa_ctx *ctx, const float *params, const uint64_t *prefixes,
                               uint64_t n, float *out) {
    CTX_OR_EINVAL(ctx);
    if (!params || (n && (!prefixes || !out)))
        return scope.finish(set_err(c, CAPSSA_EINVAL, "null model buffer"));
    if (n > 0xFFFFFFFFull) return scope.finish(set_err(c, CAPSSA_EUNSUPPORTED, "2^32 samples"));
    void *dp = nullptr, *dx = nullptr;
    capssa_status s = stage_in(c, WS_MISC, params, cdf::kParams * 4, 64, &dp);
    if (s == CAPSSA_OK) s = stage_in(c, WS_MISC2, prefixes, n * 8, 64, &dx);
    if (s != CAPSSA_OK) return scope.finish(s);
    float *dy = (float *)ws_get(c, WS_OUT2, n * 4 + 64);
    if (!dy) return scope.finish(set_err(c, CAPSSA_ENOMEM, "model output"));
    s = cdf::infer(c, (const float *)dp, (const uint64_t *)dx, (uint32_t)n, dy);
    if (s == CAPSSA_OK) s = stage_out(c, out, dy, n * 4);
    return scope.finish(s);
}

capssa_status capssa_cdf_train(capssa_ctx *ctx, const uint64_t *prefixes, const float *targets,
                               uint64_t n, int32_t steps, float *params, float *loss) {
    CTX_OR_EINVAL(ctx);
    if (!params || !loss || (n && (!prefixes || !targets)) || steps < 0)
        return scope.finish(set_err(c, CAPSSA_EINVAL, "bad model training arguments"));
    if (n > 0xFFFFFFFFull) return scope.finish(set_err(c, CAPSSA_EUNSUPPORTED, "2^32 samples"));
    void *dx = nullptr, *dt = nullptr;
    capssa_status s = stage_in(c, WS_MISC2, prefixes, n * 8, 64, &dx);
    if (s == CAPSSA_OK) s = stage_in(c, WS_MISC3, targets, n * 4, 64, &dt);
    if (s != CAPSSA_OK) return scope.finish(s);
    float *dp = (float *)ws_get(c, WS_OUT2, cdf::kParams * 6 + 64);
    if (!dp) return scope.finish(set_err(c, CAPSSA_ENOMEM, "model buffer"));
    float fl = 0.0f;
    s = cdf::train(c, (const uint64_t *)dx, (const float *)dt, (uint32_t)n, steps, dp,
                   (__nv_bfloat16 *)(dp + cdf::kParams + 3), &fl);
    if (s == CAPSSA_OK) s = stage_out(c, params, dp, cdf::kParams * 4);
    if (s == CAPSSA_OK) *loss = fl;
    return scope.finish(s);
}

// Packer::new + seed_params (src/pack.rs:103-176, 217-234): the byte
// presence scan runs on the device, the 256-entry map on the host.
capssa_status capssa_pack_params_u8(capssa_ctx *ctx, const uint8_t *text, uint64_t n,
                                    int32_t policy, uint64_t max_extra_bytes, capssa_packer *out,
                                    int32_t *available) {
    CTX_OR_EINVAL(ctx);
    if (!out || !available || (!text && n)) return scope.finish(set_err(c, CAPSSA_EINVAL, "null argument"));
    *available = 0;
    std::memset(out, 0, sizeof(*out));
    if (policy == CAPSSA_SEED_DISABLED) return scope.finish(CAPSSA_OK);
    bool present[256] = {};
    if (n) {
        void *d_text = nullptr;
        capssa_status s = stage_text(c, text, n, &d_text);
        if (s != CAPSSA_OK) return scope.finish(s);
        uint32_t *d_present = (uint32_t *)ws_get(c, WS_CODES, 256 * 4 + 64);
        if (!d_present) return scope.finish(set_err(c, CAPSSA_ENOMEM, "presence table"));
        cudaMemsetAsync(d_present, 0, 256 * 4, c.stream);
        s = presence_u8(c, (const uint8_t *)d_text, n, d_present);
        if (s != CAPSSA_OK) return scope.finish(s);
        uint32_t h[256];
        cudaMemcpyAsync(h, d_present, 1024, cudaMemcpyDeviceToHost, c.stream);
        cudaStreamSynchronize(c.stream);
        for (int i = 0; i < 256; i++) present[i] = h[i] != 0;
    }
    uint32_t next = 0;
    bool identity = true;
    for (int b = 0; b < 256; b++) {
        out->code[b] = (uint8_t)next;
        if (present[b]) {
            if ((int)next != b) identity = false;
            next++;
        }
    }
    uint32_t bits = next <= 1 ? 1 : next <= 3 ? 2 : next <= 15 ? 4 : 8;
    if (!identity) {
        if (policy != CAPSSA_SEED_REMAP || n > max_extra_bytes) return scope.finish(CAPSSA_OK);
    } else {
        for (int b = 0; b < 256; b++) out->code[b] = (uint8_t)b;
    }
    if (!((uint64_t)next < (1ull << bits))) return scope.finish(CAPSSA_OK);  // has_sentinel
    out->bits = bits;
    out->k = 64 / bits;
    out->alphabet = next;
    out->identity = identity ? 1 : 0;
    *available = 1;
    return scope.finish(CAPSSA_OK);
}

capssa_status capssa_pack_keys_u8(capssa_ctx *ctx, const uint8_t *text, uint64_t n,
                                  const capssa_packer *pk, const capssa_limits *lp,
                                  const uint64_t *positions, uint64_t m, uint64_t *keys) {
    CTX_OR_EINVAL(ctx);
    if (!pk || (!positions && m) || (!keys && m)) return scope.finish(set_err(c, CAPSSA_EINVAL, "null argument"));
    if (m == 0) return scope.finish(CAPSSA_OK);
    if (pk->bits == 0 || pk->k == 0) return scope.finish(set_err(c, CAPSSA_EINVAL, "invalid packer"));
    if (!positions_within(c, positions, m, 8, n))
        return scope.finish(set_err(c, CAPSSA_EINVAL, "a position lies beyond the end of the text"));
    DevLimits L{};
    capssa_status s = stage_limits(c, lp, n, &L);
    if (s != CAPSSA_OK) return scope.finish(s);
    void *d_text = nullptr, *d_pos = nullptr, *d_code = nullptr;
    if ((s = stage_text(c, text, n, &d_text)) != CAPSSA_OK) return scope.finish(s);
    if ((s = stage_in(c, WS_POS_IN, positions, m * 8, 64, &d_pos)) != CAPSSA_OK) return scope.finish(s);
    if ((s = stage_in(c, WS_CODES, pk->code, 256, 64, &d_code)) != CAPSSA_OK) return scope.finish(s);
    uint64_t *d_keys = (uint64_t *)ws_get(c, WS_OUT, m * 8 + 64);
    if (!d_keys) return scope.finish(set_err(c, CAPSSA_ENOMEM, "key output"));
    pack_keys_kernel<<<grid_for(m, 256), 256, 0, c.stream>>>(
        (const uint8_t *)d_text, n, (const uint8_t *)d_code, pk->bits, pk->k, pk->alphabet, L,
        (const uint64_t *)d_pos, m, d_keys);
    c.launches++;
    if (cudaGetLastError() != cudaSuccess) return scope.finish(set_err(c, CAPSSA_ECUDA, "pack launch"));
    return scope.finish(stage_out(c, keys, d_keys, m * 8));
}

// seed_subarray (src/pack.rs:241-321): the positions in suffix order and
// the exact adjacent LCP array under the provider's limits.
capssa_status capssa_seed_subarray_u8_u32(capssa_ctx *ctx, const uint8_t *text, uint64_t n,
                                          const capssa_packer *pk, const capssa_limits *lp,
                                          uint32_t *sa, uint32_t *lcp, uint64_t m) {
    CTX_OR_EINVAL(ctx);
    if (!pk) return scope.finish(set_err(c, CAPSSA_EINVAL, "null packer"));
    capssa_opts o;
    capssa_opts_default(&o);
    return scope.finish(build_common<uint8_t>(c, text, n, sa, 4, m, lp, &o, sa, 4, lcp));
}

capssa_status capssa_seed_subarray_u8_u64(capssa_ctx *ctx, const uint8_t *text, uint64_t n,
                                          const capssa_packer *pk, const capssa_limits *lp,
                                          uint64_t *sa, uint64_t *lcp, uint64_t m) {
    CTX_OR_EINVAL(ctx);
    if (!pk) return scope.finish(set_err(c, CAPSSA_EINVAL, "null packer"));
    capssa_opts o;
    capssa_opts_default(&o);
    return scope.finish(build_common<uint8_t>(c, text, n, sa, 8, m, lp, &o, sa, 8, lcp));
}

}  // extern "C"

namespace capssa {
__global__ void presence_u8_kernel(const uint8_t *__restrict__ text, uint64_t n,
                                   uint32_t *__restrict__ present) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t s = text[i];
        if (__ldcg(present + s) == 0) present[s] = 1;
    }
}
capssa_status presence_u8(Ctx &c, const uint8_t *text, uint64_t n, uint32_t *present) {
    presence_u8_kernel<<<std::min<unsigned>(grid_for(n, 256), c.sm_count * 8), 256, 0, c.stream>>>(
        text, n, present);
    CAPSSA_LAUNCHED(c);
    return CAPSSA_OK;
}
}  // namespace capssa

// ------------------------------------------------------------ on-disk formats

namespace capssa {
namespace {

// SaLcp<I> bucket records (src/ext_bucket.rs:65-108): (pos, lcp) pairs, the
// device's little-endian words being the record's byte order.
template <typename IT>
__global__ void sa_lcp_records_kernel(const IT *__restrict__ sa, const IT *__restrict__ lcp,
                                      uint64_t n, IT *__restrict__ rec) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        rec[2 * i] = sa[i];
        rec[2 * i + 1] = lcp[i];
    }
}

template <typename IT>
capssa_status sa_lcp_records(Ctx &c, const IT *sa, const IT *lcp, uint64_t n, void *out) {
    if (n == 0) return CAPSSA_OK;
    if (!sa || !lcp || !out) return set_err(c, CAPSSA_EINVAL, "null buffer");
    void *d_sa = nullptr, *d_lcp = nullptr;
    capssa_status s = stage_in(c, WS_MISC, sa, n * sizeof(IT), 64, &d_sa);
    if (s == CAPSSA_OK) s = stage_in(c, WS_MISC2, lcp, n * sizeof(IT), 64, &d_lcp);
    if (s != CAPSSA_OK) return s;
    const bool out_dev = is_device_ptr(out);
    void *d_rec = out_dev ? out : ws_get(c, WS_OUT, 2 * n * sizeof(IT) + 64);
    if (!d_rec) return set_err(c, CAPSSA_ENOMEM, "record buffer");
    sa_lcp_records_kernel<IT><<<grid_for(n, 256, 152 * 64), 256, 0, c.stream>>>(
        (const IT *)d_sa, (const IT *)d_lcp, n, (IT *)d_rec);
    CAPSSA_LAUNCHED(c);
    if (!out_dev) return stage_out(c, out, d_rec, 2 * n * sizeof(IT));
    return CAPSSA_OK;
}

// Little-endian bytes of `len` values, `width` bytes each, appended to f.
int write_le(FILE *f, const uint64_t *v, uint64_t len, int width) {
    unsigned char buf[8 * 4096];
    while (len) {
        const uint64_t take = len < 4096 ? len : 4096;
        for (uint64_t i = 0; i < take; i++) {
            if (width == 4 && v[i] > 0xFFFFFFFFull) return 1;
            for (int b = 0; b < width; b++) buf[i * width + b] = (unsigned char)(v[i] >> (8 * b));
        }
        if (std::fwrite(buf, (size_t)width, (size_t)take, f) != take) return 1;
        v += take;
        len -= take;
    }
    return 0;
}

}  // namespace
}  // namespace capssa

extern "C" {

// examples/rustar_segmented_bench.rs:236-245: state = 0x6c62272e07bb0142_
// 62b821756295c58d; per position p: state ^= p, state *= 2^88 + 0x13b
// (mod 2^128), state ^= p << 64.
void capssa_checksum128_init(capssa_checksum128 *c) {
    if (!c) return;
    c->count = 0;
    c->hi = 0x6c62272e07bb0142ull;
    c->lo = 0x62b821756295c58dull;
}

void capssa_checksum128_update(capssa_checksum128 *c, const uint64_t *positions, uint64_t len) {
    if (!c || (!positions && len)) return;
    unsigned __int128 x = ((unsigned __int128)c->hi << 64) | c->lo;
    const unsigned __int128 prime = ((unsigned __int128)1 << 88) | 0x13b;
    for (uint64_t i = 0; i < len; i++) {
        const uint64_t p = positions[i];
        x ^= p;
        x *= prime;
        x ^= (unsigned __int128)p << 64;
    }
    c->count += len;
    c->lo = (uint64_t)x;
    c->hi = (uint64_t)(x >> 64);
}

int capssa_emit_checksum128(void *user, const uint64_t *positions, uint64_t len) {
    if (!user) return 1;
    capssa_checksum128_update((capssa_checksum128 *)user, positions, len);
    return 0;
}

int capssa_emit_file_u64(void *user, const uint64_t *positions, uint64_t len) {
    if (!user || (!positions && len)) return 1;
    return write_le((FILE *)user, positions, len, 8);
}

int capssa_emit_file_u32(void *user, const uint64_t *positions, uint64_t len) {
    if (!user || (!positions && len)) return 1;
    return write_le((FILE *)user, positions, len, 4);
}

capssa_status capssa_sa_lcp_records_u32(capssa_ctx *ctx, const uint32_t *sa, const uint32_t *lcp,
                                        uint64_t n, void *out_records) {
    CTX_OR_EINVAL(ctx);
    return scope.finish(sa_lcp_records<uint32_t>(c, sa, lcp, n, out_records));
}

capssa_status capssa_sa_lcp_records_u64(capssa_ctx *ctx, const uint64_t *sa, const uint64_t *lcp,
                                        uint64_t n, void *out_records) {
    CTX_OR_EINVAL(ctx);
    return scope.finish(sa_lcp_records<uint64_t>(c, sa, lcp, n, out_records));
}

}  // extern "C"
