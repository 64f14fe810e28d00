// ties.cu — the reference's order inside comparator tie classes.
//
// Under SegmentedText with the ShorterFirst boundary order, suffixes that are
// equal up to their (equal) limits compare Equal, and the reference emits
// them in whatever order its merge sort produces: recursive halves at
// mid = len / 2 of the input positions (src/sample_sort.rs:221-266), merged
// by merge_body! (src/sample_sort.rs:430-497), which on Equal outputs from the
// stream it did not output from last.  Inside one merge the members of a
// class therefore alternate between the two halves, beginning with the half
// that did not output the element just before the class (the left half when
// nothing came before it: the right half goes first), and the longer half's
// remaining members follow.  Nodes whose class members all sit in one half
// keep their order.
//
// The engine emits each class in ascending input order.  This pass computes,
// for every class and every merge-tree node with class members in both
// halves (a split node), which half output last before the class:
//   * the predecessor of the class among the node's inputs is the input with
//     the largest suffix-order slot below the class start.  A block walks
//     back from the class start through the slots, and each slot marks the
//     split nodes of the class on its input's root-to-leaf path (first hit =
//     largest slot); nodes the walk did not reach within its budget scan
//     their input range instead;
//   * if the predecessor belongs to another tie class with members in both
//     halves of the node, that class's last output decides: its longer half,
//     or, with equal halves, the half it did not begin with there (a link to
//     that class's own split node, followed afterwards);
// then places every member by composing the alternations from its leaf up to
// the root.  The model was checked against the oracle's merge sort (which
// restates the reference's) on random segmented texts, subsets, repeated
// positions and finite contexts.
#include <algorithm>

#include "common.cuh"
#include "lcp.cuh"
#include "radix.cuh"
#include "scan.cuh"
#include "ties.cuh"

namespace capssa {
namespace {

constexpr int kMaxDepth = 40;            // merge-tree depth for up to 2^32 inputs, with slack
constexpr uint32_t kWalkSlots = 1u << 16;  // slots a class walks back before scanning
constexpr uint32_t kChaseLimit = 1u << 24;  // links followed from one split node
enum : uint32_t { kWalkDone = 0, kWalkExhausted = 1, kWalkBudget = 2 };

inline int bits_upto(uint64_t v) {  // bits to represent 0..v
    int b = 1;
    while (b < 64 && (v >> b) != 0) b++;
    return b;
}

__device__ __forceinline__ uint32_t lower_bound_u32(const uint32_t *__restrict__ a, uint32_t lo,
                                                    uint32_t hi, uint64_t x) {
    while (lo < hi) {
        const uint32_t mid = lo + ((hi - lo) >> 1);
        if ((uint64_t)__ldg(a + mid) < x)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

// tie[r] = 1 when slot r - 1 and r compare Equal; pos32 = the positions.
template <typename OT>
__global__ void tie_flag_kernel(const OT *__restrict__ out, uint32_t m,
                                const uint32_t *__restrict__ key,
                                const uint8_t *__restrict__ text, int sym_bytes, DevLimits L,
                                uint64_t max_ctx, uint32_t *__restrict__ pos32,
                                uint32_t *__restrict__ tie) {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t r0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); r0 < m; r0 += stride) {
        // whole warps step together: a slot's limit is its left neighbour's too
        const uint32_t lane = threadIdx.x & 31, r = r0 + lane;
        const bool in = r < m;
        const uint32_t b = in ? (uint32_t)out[r] : 0u;
        const uint64_t lb = key || !in ? 0ull : dev_lim_at(L, b);
        const uint64_t lup = __shfl_up_sync(0xffffffffu, lb, 1);
        if (!in) continue;
        pos32[r] = b;
        uint32_t t = 0;
        if (r > 0) {
            if (key) {
                t = key[r] == key[r - 1];
            } else {  // suffix_cmp_with Equal: same limit, same symbols up to it (or max_ctx)
                const uint32_t a = (uint32_t)out[r - 1];
                const uint64_t la = lane ? lup : dev_lim_at(L, a);
                if (la == lb) {
                    const uint64_t lim = la < max_ctx ? la : max_ctx;
                    const uint64_t k = (uint64_t)sym_bytes;
                    t = thread_lcp_bytes(text, (uint64_t)a * k, (uint64_t)b * k, lim * k) >=
                        lim * k;
                }
            }
        }
        tie[r] = t;
    }
}

// Member marks (0/1, scanned afterwards): slots tied to a neighbour.
__global__ void member_mark_kernel(const uint32_t *__restrict__ tie, uint32_t m,
                                   uint32_t *__restrict__ mem) {
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < m; r += gridDim.x * blockDim.x)
        mem[r] = (tie[r] || (r + 1 < m && tie[r + 1])) ? 1u : 0u;
}

// The members' slots, in slot order (ms: exclusive scan of the marks).
__global__ void member_list_kernel(const uint32_t *__restrict__ tie, uint32_t m,
                                   const uint32_t *__restrict__ ms, uint32_t *__restrict__ slot) {
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < m; r += gridDim.x * blockDim.x)
        if (tie[r] || (r + 1 < m && tie[r + 1])) slot[ms[r]] = r;
}

// Class-start marks over the member list (a member not tied to its left).
__global__ void start_mark_kernel(const uint32_t *__restrict__ tie, const uint32_t *__restrict__ slot,
                                  uint32_t M, uint32_t *__restrict__ st) {
    for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < M; u += gridDim.x * blockDim.x)
        st[u] = tie[slot[u]] ? 0u : 1u;
}

// cstart / moff per class, (class << 32 | input index) and position per
// member (cs: exclusive scan of the start marks over the member list).
__global__ void class_emit_kernel(const uint32_t *__restrict__ tie,
                                  const uint32_t *__restrict__ slot, uint32_t M,
                                  const uint32_t *__restrict__ cs,
                                  const uint32_t *__restrict__ idxf,
                                  const uint32_t *__restrict__ pos32,
                                  uint32_t *__restrict__ cstart, uint32_t *__restrict__ moff,
                                  uint64_t *__restrict__ mkey, uint32_t *__restrict__ melem) {
    for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < M; u += gridDim.x * blockDim.x) {
        const uint32_t r = slot[u];
        const bool st = !tie[r];
        const uint32_t ord = st ? cs[u] : cs[u] - 1;
        if (st) {
            cstart[ord] = r;
            moff[ord] = u;
        }
        mkey[u] = ((uint64_t)ord << 32) | idxf[r];
        melem[u] = pos32[r];
    }
}

struct Classes {
    uint32_t C, M;               // classes, members
    uint64_t N;                  // merge-tree inputs
    const uint32_t *cstart;      // first slot of each class (ascending)
    const uint32_t *moff;        // first member of each class
    const uint64_t *mkey;        // (class << 32 | input index), by class then input index
    const uint32_t *midx;        // input index of each member
    __device__ __forceinline__ uint32_t size(uint32_t c) const {
        return (c + 1 < C ? __ldg(moff + c + 1) : M) - __ldg(moff + c);
    }
};

__global__ void member_idx_kernel(const uint64_t *__restrict__ mkey, uint32_t M,
                                  uint32_t *__restrict__ midx) {
    for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < M; u += gridDim.x * blockDim.x)
        midx[u] = (uint32_t)mkey[u];
}

// Split node of consecutive members u, u + 1 (id u - class): their lowest
// common merge-tree node.
__global__ void split_info_kernel(Classes K, uint32_t *__restrict__ slo, uint32_t *__restrict__ shi,
                                  uint32_t *__restrict__ scls, uint32_t *__restrict__ pred) {
    for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < K.M; u += gridDim.x * blockDim.x) {
        const uint32_t c = (uint32_t)(K.mkey[u] >> 32);
        if (u + 1 >= K.moff[c] + K.size(c)) continue;  // the class's last member
        const uint64_t x = K.midx[u], y = K.midx[u + 1];
        uint64_t lo = 0, hi = K.N;
        for (int d = 0; d < kMaxDepth; d++) {
            const uint64_t mid = lo + (hi - lo) / 2;
            if (y < mid)
                hi = mid;
            else if (x >= mid)
                lo = mid;
            else
                break;
        }
        const uint32_t t = u - c;
        slo[t] = (uint32_t)lo;
        shi[t] = (uint32_t)(hi - 1);  // inclusive: hi may be 2^32
        scls[t] = c;
        pred[t] = 0;
    }
}

// One block per class: walk back from the class start; every slot marks the
// split nodes on its input's path (pred = slot + 1, the largest wins).
__global__ void __launch_bounds__(256)
    walk_kernel(Classes K, const uint32_t *__restrict__ idxf, uint32_t *__restrict__ pred,
                uint32_t *__restrict__ cstate, uint32_t *__restrict__ n_budget) {
    __shared__ uint32_t s_found;
    for (uint32_t c = blockIdx.x; c < K.C; c += gridDim.x) {
        const uint32_t s = K.cstart[c], mb = K.moff[c], k = K.size(c);
        if (threadIdx.x == 0) s_found = 0;
        __syncthreads();
        uint32_t walked = 0, state = kWalkDone;
        for (;;) {
            if (walked >= s) {
                state = kWalkExhausted;
                break;
            }
            if (walked >= kWalkSlots) {
                state = kWalkBudget;
                break;
            }
            const uint32_t top = s - walked;  // slots [top - 256, top)
            if (threadIdx.x < top) {
                const uint32_t q = top - 1 - threadIdx.x;
                const uint64_t j = idxf[q];
                uint32_t a = mb, b = mb + k;
                uint64_t lo = 0, hi = K.N;
                for (int d = 0; d < kMaxDepth && b - a >= 2; d++) {
                    const uint64_t mid = lo + (hi - lo) / 2;
                    const uint32_t cm = lower_bound_u32(K.midx, a, b, mid);
                    if (a < cm && cm < b) {
                        const uint32_t old = atomicMax(&pred[cm - 1 - c], q + 1);
                        if (old == 0) atomicAdd(&s_found, 1u);
                    }
                    if (j < mid) {
                        b = cm;
                        hi = mid;
                    } else {
                        a = cm;
                        lo = mid;
                    }
                }
            }
            walked += 256;
            __syncthreads();
            const bool done = s_found == k - 1;
            __syncthreads();
            if (done) break;
        }
        if (threadIdx.x == 0) {
            cstate[c] = state;
            if (state == kWalkBudget) atomicAdd(n_budget, 1u);
        }
        __syncthreads();
    }
}

// Split nodes the walk did not reach: one warp scans the node's inputs for
// the largest slot below the class start.
__global__ void brute_kernel(Classes K, uint32_t S, const uint32_t *__restrict__ slo,
                             const uint32_t *__restrict__ shi, const uint32_t *__restrict__ scls,
                             const uint32_t *__restrict__ cstate,
                             const uint32_t *__restrict__ slot_of, uint32_t *__restrict__ pred) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    for (uint32_t t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < S; t += warps) {
        const uint32_t c = scls[t];
        if (pred[t] != 0 || cstate[c] != kWalkBudget) continue;
        const uint32_t s = K.cstart[c];
        uint32_t best = 0;
        for (uint64_t j = (uint64_t)slo[t] + lane; j <= shi[t]; j += 32) {
            const uint32_t q = __ldg(slot_of + j);
            if (q < s && q + 1 > best) best = q + 1;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) best = max(best, __shfl_xor_sync(0xffffffffu, best, o));
        if (lane == 0) pred[t] = best;
    }
}

// Which half goes first at each split node (start: 0 left, 1 right), or a
// link (dep = split id + 1) to the split node of the preceding class whose
// last output decides.
__global__ void resolve_kernel(Classes K, uint32_t S, const uint32_t *__restrict__ slo,
                               const uint32_t *__restrict__ shi, const uint32_t *__restrict__ pred,
                               const uint32_t *__restrict__ idxf, uint32_t *__restrict__ start,
                               uint32_t *__restrict__ dep) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < S; t += gridDim.x * blockDim.x) {
        const uint64_t lo = slo[t], hi = (uint64_t)shi[t] + 1, mid = lo + (hi - lo) / 2;
        dep[t] = 0;
        if (pred[t] == 0) {  // nothing before the class: the left half was "last"
            start[t] = 1;
            continue;
        }
        const uint32_t q = pred[t] - 1;
        // the tie class holding slot q, if any
        uint32_t c2 = 0;
        {
            uint32_t a = 0, b = K.C;  // first class starting after q
            while (a < b) {
                const uint32_t md = a + ((b - a) >> 1);
                if (K.cstart[md] <= q)
                    a = md + 1;
                else
                    b = md;
            }
            c2 = a;  // classes [0, a) start at or before q
        }
        uint32_t last;
        if (c2 > 0 && q < K.cstart[c2 - 1] + K.size(c2 - 1)) {
            const uint32_t cc = c2 - 1, mb = K.moff[cc], me = mb + K.size(cc);
            const uint32_t a = lower_bound_u32(K.midx, mb, me, lo);
            const uint32_t md = lower_bound_u32(K.midx, a, me, mid);
            const uint32_t b = lower_bound_u32(K.midx, md, me, hi);
            const uint32_t cl = md - a, cr = b - md;
            if (cr == 0)
                last = 0;
            else if (cl == 0)
                last = 1;
            else if (cl != cr)
                last = cl > cr ? 0u : 1u;
            else {  // equal halves: it ended on the half it did not begin with
                dep[t] = (md - 1 - cc) + 1;
                continue;
            }
        } else {
            last = (uint64_t)idxf[q] >= mid ? 1u : 0u;
        }
        start[t] = 1u - last;
    }
}

// start[t] = start of the end of t's link chain (chains run to earlier
// classes, so they end).
__global__ void chase_kernel(uint32_t S, const uint32_t *__restrict__ dep,
                             uint32_t *__restrict__ start, int *__restrict__ err) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < S; t += gridDim.x * blockDim.x) {
        if (!dep[t]) continue;
        uint32_t x = dep[t] - 1, steps = 0;
        while (dep[x] && steps < kChaseLimit) {
            x = dep[x] - 1;
            steps++;
        }
        if (dep[x]) {
            atomicCAS(err, DEV_OK, DEV_LOOKBACK_TIMEOUT);
            continue;
        }
        start[t] = start[x];
    }
}

// Every member's place in its class: descend to its leaf recording the split
// nodes on the way, then compose the alternations upwards.
template <typename OT>
__global__ void place_kernel(Classes K, const uint32_t *__restrict__ start,
                             const uint32_t *__restrict__ melem, OT *__restrict__ out) {
    for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < K.M; u += gridDim.x * blockDim.x) {
        const uint32_t c = (uint32_t)(K.mkey[u] >> 32);
        const uint32_t mb = K.moff[c], k = K.size(c);
        const uint64_t x = K.midx[u];
        uint32_t pt[kMaxDepth], cl[kMaxDepth], cr[kMaxDepth];
        uint64_t side = 0;  // bit d: the member is in the right half of split d
        int depth = 0;
        uint32_t a = mb, b = mb + k;
        uint64_t lo = 0, hi = K.N;
        for (int d = 0; d < kMaxDepth && b - a >= 2; d++) {
            const uint64_t mid = lo + (hi - lo) / 2;
            const uint32_t cm = lower_bound_u32(K.midx, a, b, mid);
            if (a < cm && cm < b) {
                pt[depth] = cm - 1 - c;
                cl[depth] = cm - a;
                cr[depth] = b - cm;
                if (x >= mid) side |= 1ull << depth;
                depth++;
            }
            if (x < mid) {
                b = cm;
                hi = mid;
            } else {
                a = cm;
                lo = mid;
            }
        }
        uint32_t r = 0;
        for (int d = depth - 1; d >= 0; d--) {
            const uint32_t sd = (uint32_t)(side >> d) & 1u;
            const uint32_t p = cl[d] < cr[d] ? cl[d] : cr[d];
            r = r < p ? 2 * r + (sd == start[pt[d]] ? 0u : 1u) : p + r;
        }
        out[K.cstart[c] + r] = (OT)melem[u];
    }
}

// err[0] = 1 unless the positions strictly ascend.
template <typename PT>
__global__ void ascending_kernel(const PT *__restrict__ pos, uint32_t m, uint32_t *__restrict__ err) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i + 1 < m;
         i += gridDim.x * blockDim.x)
        if (pos[i] >= pos[i + 1]) *err = 1;
}

// One bit per chosen position.  Positions ascend, so a warp's lanes mostly
// share words: the lanes of one word combine their bits and one of them
// writes the word.
template <typename PT>
__global__ void pos_bits_kernel(const PT *__restrict__ pos, uint32_t m, uint32_t *__restrict__ bits) {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); i0 < m; i0 += stride) {
        const uint32_t i = i0 + (threadIdx.x & 31);
        const uint64_t p = i < m ? (uint64_t)pos[i] : ~0ull;
        const uint32_t w = (uint32_t)(p >> 5);  // past the end: a word no position has
        const unsigned peers = __match_any_sync(0xffffffffu, w);
        const uint32_t v = __reduce_or_sync(peers, i < m ? 1u << (p & 31) : 0u);
        if (i < m && (threadIdx.x & 31) == (uint32_t)(__ffs((int)peers) - 1)) atomicOr(&bits[w], v);
    }
}

__global__ void popc_words_kernel(const uint32_t *__restrict__ bits, uint64_t nw,
                                  uint32_t *__restrict__ wc) {
    for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < nw;
         w += (uint64_t)gridDim.x * blockDim.x)
        wc[w] = __popc(bits[w]);
}

// (prefix count, bits) of every bitmap word side by side: a rank lookup is
// one 8-byte load.
__global__ void rank_words_kernel(const uint32_t *__restrict__ bits,
                                  const uint32_t *__restrict__ wc, uint64_t nw,
                                  uint2 *__restrict__ rw) {
    for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < nw;
         w += (uint64_t)gridDim.x * blockDim.x)
        rw[w] = make_uint2(wc[w], bits[w]);
}

// Input index of each slot for ascending positions: the rank of its position
// among them (its word's prefix count + the bits below it in the word).
__global__ void pos_rank_kernel(const uint32_t *__restrict__ pos32, uint32_t m,
                                const uint2 *__restrict__ rw, uint32_t *__restrict__ idxf) {
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < m; r += gridDim.x * blockDim.x) {
        const uint32_t p = pos32[r];
        const uint2 e = __ldg(rw + (p >> 5));
        idxf[r] = e.x + __popc(e.y & ((1u << (p & 31)) - 1u));
    }
}

template <typename PT>
__global__ void pos_key_kernel(const PT *__restrict__ pos, uint32_t m, uint64_t *__restrict__ key) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x)
        key[i] = (uint64_t)pos[i];
}

__global__ void widen_u32_kernel(const uint32_t *__restrict__ v, uint32_t m,
                                 uint64_t *__restrict__ key) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x)
        key[i] = v[i];
}

}  // namespace

capssa_status reference_tie_order(Ctx &c, const TieArgs &t) {
    const uint64_t m = t.m;
    if (m < 2) return CAPSSA_OK;
    if (m > 0xFFFFFFFFull) return set_err(c, CAPSSA_EUNSUPPORTED, "tie order beyond 2^32-1 slots");
    const uint32_t mm = (uint32_t)m;
    const size_t m4 = (size_t)m * 4 + 64, m8 = (size_t)m * 8 + 64;
    uint32_t *pos32 = (uint32_t *)ws_get(c, WS_MISC, 2 * m4);
    uint32_t *cs = (uint32_t *)ws_get(c, WS_MISC2, 2 * m4);
    uint32_t *maps = (uint32_t *)ws_get(c, WS_MISC3, 2 * m4);
    uint64_t *ka = (uint64_t *)ws_get(c, WS_KEYS_A, m8);
    uint64_t *kb = (uint64_t *)ws_get(c, WS_KEYS_B, std::max(m8, scatter_hist_words(m) * 4));
    uint32_t *va = (uint32_t *)ws_get(c, WS_VALS_A, m4);
    uint32_t *vb = (uint32_t *)ws_get(c, WS_VALS_B, m4);
    if (!pos32 || !cs || !maps || !ka || !kb || !va || !vb)
        return set_err(c, CAPSSA_ENOMEM, "tie order workspace");
    uint32_t *tie = pos32 + m4 / 4, *ms = cs + m4 / 4;
    uint32_t *idxf = maps, *slot_of = maps + m4 / 4;
    const unsigned g = grid_for(m, 256);
    KernelTimes kt(profile_on());
    kt.start(c.stream);
    // 1. classes: adjacent Equal pairs
    if (t.out_bytes == 8)
        tie_flag_kernel<uint64_t><<<g, 256, 0, c.stream>>>((const uint64_t *)t.out, mm, t.key,
                                                           (const uint8_t *)t.text, t.sym_bytes,
                                                           t.lim, t.max_ctx, pos32, tie);
    else
        tie_flag_kernel<uint32_t><<<g, 256, 0, c.stream>>>((const uint32_t *)t.out, mm, t.key,
                                                           (const uint8_t *)t.text, t.sym_bytes,
                                                           t.lim, t.max_ctx, pos32, tie);
    CAPSSA_LAUNCHED(c);
    kt.mark(c.stream, "flags");
    // members (slots tied to a neighbour) listed in slot order into `cs`,
    // then class starts numbered over that list in `ms`
    member_mark_kernel<<<g, 256, 0, c.stream>>>(tie, mm, ms);
    CAPSSA_LAUNCHED(c);
    capssa_status s = scan_u32(c, ms, ms, m, false, false);
    if (s != CAPSSA_OK) return s;
    uint32_t *h = (uint32_t *)c.h_scratch;
    uint32_t *h_err = (uint32_t *)(c.d_flags + 1);  // a scratch device word
    CAPSSA_CUDA(c, cudaMemcpyAsync(h, ms + (m - 1), 4, cudaMemcpyDeviceToHost, c.stream));
    CAPSSA_CUDA(c, cudaMemcpyAsync(h + 1, tie + (m - 1), 4, cudaMemcpyDeviceToHost, c.stream));
    CAPSSA_CUDA(c, cudaStreamSynchronize(c.stream));
    const uint32_t M = h[0] + h[1];  // the last slot is a member iff tied to its left
    c.stats.tie_classes = 0;
    if (M == 0) return CAPSSA_OK;
    uint32_t *mslot = cs;
    member_list_kernel<<<g, 256, 0, c.stream>>>(tie, mm, ms, mslot);
    CAPSSA_LAUNCHED(c);
    const unsigned gM = grid_for(M, 256);
    uint32_t *cord = ms;  // the member scan is dead once the list is written
    start_mark_kernel<<<gM, 256, 0, c.stream>>>(tie, mslot, M, cord);
    CAPSSA_LAUNCHED(c);
    s = scan_u32(c, cord, cord, M, false, false);
    if (s != CAPSSA_OK) return s;
    CAPSSA_CUDA(c, cudaMemcpyAsync(h, cord + (M - 1), 4, cudaMemcpyDeviceToHost, c.stream));
    CAPSSA_CUDA(c, cudaStreamSynchronize(c.stream));
    const uint32_t C = h[0];  // an exclusive count: the last member never starts a class
    c.stats.tie_classes = C;
    kt.mark(c.stream, "classes");
    // 2. input index of every slot and slot of every input index
    bool ascending = false;
    if (t.positions) {  // strictly ascending positions (a filter's) rank through a bitmap
        CAPSSA_CUDA(c, cudaMemsetAsync(h_err, 0, 4, c.stream));
        if (t.pos_bytes == 8)
            ascending_kernel<uint64_t><<<g, 256, 0, c.stream>>>((const uint64_t *)t.positions, mm,
                                                                h_err);
        else
            ascending_kernel<uint32_t><<<g, 256, 0, c.stream>>>((const uint32_t *)t.positions, mm,
                                                                h_err);
        CAPSSA_LAUNCHED(c);
        CAPSSA_CUDA(c, cudaMemcpyAsync(h, h_err, 4, cudaMemcpyDeviceToHost, c.stream));
        CAPSSA_CUDA(c, cudaStreamSynchronize(c.stream));
        ascending = h[0] == 0;
    }
    // the slot of every input index (slot_of) is needed only if a walk runs
    // out of budget; for a whole text or ascending positions it is scattered
    // from idxf then, the other positions need it from the sorts below
    bool have_slots = false;
    if (!t.positions) {  // a whole text: the input index is the position
        idxf = pos32;
    } else if (ascending) {
        const uint64_t nw = (t.lim.n + 1) / 32 + 1;  // position n included
        uint32_t *bits = (uint32_t *)ws_get(c, WS_KEEP, nw * 4 + 64);
        uint2 *rw = (uint2 *)ws_get(c, WS_RANK, nw * 12 + 128);  // rw, then the counts
        if (!bits || !rw) return set_err(c, CAPSSA_ENOMEM, "tie order workspace");
        uint32_t *wc = (uint32_t *)(rw + nw);
        CAPSSA_CUDA(c, cudaMemsetAsync(bits, 0, nw * 4, c.stream));
        if (t.pos_bytes == 8)
            pos_bits_kernel<uint64_t><<<g, 256, 0, c.stream>>>((const uint64_t *)t.positions, mm,
                                                               bits);
        else
            pos_bits_kernel<uint32_t><<<g, 256, 0, c.stream>>>((const uint32_t *)t.positions, mm,
                                                               bits);
        CAPSSA_LAUNCHED(c);
        popc_words_kernel<<<grid_for(nw, 256), 256, 0, c.stream>>>(bits, nw, wc);
        CAPSSA_LAUNCHED(c);
        s = scan_u32(c, wc, wc, nw, false, false);
        if (s != CAPSSA_OK) return s;
        rank_words_kernel<<<grid_for(nw, 256), 256, 0, c.stream>>>(bits, wc, nw, rw);
        CAPSSA_LAUNCHED(c);
        pos_rank_kernel<<<g, 256, 0, c.stream>>>(pos32, mm, rw, idxf);
        CAPSSA_LAUNCHED(c);
    } else {
        // inputs and slots, each sorted by position (stably): the j-th of
        // both name the same suffix (repeated positions pair up in order)
        if (t.pos_bytes == 8)
            pos_key_kernel<uint64_t><<<g, 256, 0, c.stream>>>((const uint64_t *)t.positions, mm,
                                                              ka);
        else
            pos_key_kernel<uint32_t><<<g, 256, 0, c.stream>>>((const uint32_t *)t.positions, mm,
                                                              ka);
        CAPSSA_LAUNCHED(c);
        const int pbits = bits_upto(t.lim.n);
        bool in_b = false;
        s = radix::sort_pairs(c, ka, va, kb, vb, mm, 0, pbits, true, 0, &in_b);
        if (s != CAPSSA_OK) return s;
        uint32_t *inp = in_b ? vb : va;  // input indices by position
        uint32_t *spare = in_b ? va : vb;
        // slots by position: keys in kb (or ka), values in `spare` and idxf
        uint64_t *kx = in_b ? ka : kb, *ky = in_b ? kb : ka;
        widen_u32_kernel<<<g, 256, 0, c.stream>>>(pos32, mm, kx);
        CAPSSA_LAUNCHED(c);
        s = radix::sort_pairs(c, kx, spare, ky, slot_of, mm, 0, pbits, true, 0, &in_b);
        if (s != CAPSSA_OK) return s;
        uint32_t *slots = in_b ? slot_of : spare;
        // idxf[slot] = input; then slot_of[input] = slot (sorted keys are dead:
        // they hold the window pairs and counts)
        uint32_t *sl = slots;
        if (slots == slot_of) {  // keep slot_of free for its own scatter
            CAPSSA_CUDA(c, cudaMemcpyAsync(spare, slots, m * 4, cudaMemcpyDeviceToDevice,
                                           c.stream));
            sl = spare;
        }
        s = scatter_u32(c, sl, inp, m, idxf, m, ka, (uint32_t *)kb);
        if (s != CAPSSA_OK) return s;
        s = scatter_u32(c, inp, sl, m, slot_of, m, ka, (uint32_t *)kb);
        if (s != CAPSSA_OK) return s;
        have_slots = true;
        // pos32 still holds the slots' positions; `inp` and `sl` are dead
    }
    kt.mark(c.stream, "maps");
    // 3. members by class, then by input index
    const size_t c4 = (size_t)C * 4 + 64, s4 = (size_t)(M - C) * 4 + 64;
    char *w = (char *)ws_get(c, WS_PART, 3 * c4 + 6 * s4 + (size_t)M * 4 + 64);
    if (!w) return set_err(c, CAPSSA_ENOMEM, "tie order workspace");
    uint32_t *cstart = (uint32_t *)w, *moff = cstart + c4 / 4, *cstate = moff + c4 / 4;
    uint32_t *slo = cstate + c4 / 4, *shi = slo + s4 / 4, *scls = shi + s4 / 4;
    uint32_t *pred = scls + s4 / 4, *start = pred + s4 / 4, *dep = start + s4 / 4;
    uint32_t *midx = dep + s4 / 4;
    // members into ka / va (the maps above no longer need them)
    class_emit_kernel<<<gM, 256, 0, c.stream>>>(tie, mslot, M, cord, idxf, pos32, cstart, moff,
                                                ka, va);
    CAPSSA_LAUNCHED(c);
    bool in_b = false;
    s = radix::sort_pairs(c, ka, va, kb, vb, M, 0, 32 + bits_upto(C - 1), false, 0, &in_b);
    if (s != CAPSSA_OK) return s;
    const uint64_t *mkey = in_b ? kb : ka;
    const uint32_t *melem = in_b ? vb : va;
    member_idx_kernel<<<gM, 256, 0, c.stream>>>(mkey, M, midx);
    CAPSSA_LAUNCHED(c);
    Classes K{C, M, m, cstart, moff, mkey, midx};
    const uint32_t S = M - C;
    split_info_kernel<<<gM, 256, 0, c.stream>>>(K, slo, shi, scls, pred);
    CAPSSA_LAUNCHED(c);
    kt.mark(c.stream, "members");
    // 4. predecessors: walk, then scan what the walk left
    uint32_t *n_budget = (uint32_t *)(c.d_flags + 2);  // a scratch device word
    CAPSSA_CUDA(c, cudaMemsetAsync(n_budget, 0, 4, c.stream));
    walk_kernel<<<std::min<uint32_t>(C, (uint32_t)c.sm_count * 16), 256, 0, c.stream>>>(
        K, idxf, pred, cstate, n_budget);
    CAPSSA_LAUNCHED(c);
    kt.mark(c.stream, "walk");
    CAPSSA_CUDA(c, cudaMemcpyAsync(h, n_budget, 4, cudaMemcpyDeviceToHost, c.stream));
    CAPSSA_CUDA(c, cudaStreamSynchronize(c.stream));
    if (h[0]) {
        if (!have_slots) {  // pairs and counts in the sort buffers the members left free
            uint64_t *kfree = mkey == ka ? kb : ka;
            uint32_t *vfree = melem == va ? vb : va;
            s = scatter_u32(c, idxf, nullptr, m, slot_of, m, kfree, vfree);
            if (s != CAPSSA_OK) return s;
        }
        brute_kernel<<<grid_for((uint64_t)S * 32, 256, (unsigned)c.sm_count * 32), 256, 0,
                       c.stream>>>(K, S, slo, shi, scls, cstate, slot_of, pred);
        CAPSSA_LAUNCHED(c);
    }
    kt.mark(c.stream, "scan");
    // 5. first halves, links, places
    const unsigned gS = grid_for(S, 256);
    resolve_kernel<<<gS, 256, 0, c.stream>>>(K, S, slo, shi, pred, idxf, start, dep);
    CAPSSA_LAUNCHED(c);
    chase_kernel<<<gS, 256, 0, c.stream>>>(S, dep, start, c.d_flags);
    CAPSSA_LAUNCHED(c);
    if (t.out_bytes == 8)
        place_kernel<uint64_t><<<gM, 256, 0, c.stream>>>(K, start, melem, (uint64_t *)t.out);
    else
        place_kernel<uint32_t><<<gM, 256, 0, c.stream>>>(K, start, melem, (uint32_t *)t.out);
    CAPSSA_LAUNCHED(c);
    kt.mark(c.stream, "place");
    if (profile_on())
        std::fprintf(stderr, "capssa profile  tie order: %u classes, %u members, %u split nodes\n",
                     C, M, S);
    kt.print();
    return CAPSSA_OK;
}

}  // namespace capssa
