/*
 * capssa_oracle.c — CPU restatement of caps-sa's in-memory suffix-array path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU library and the timed
 * CPU baseline.  See capssa_oracle.h for the conventions and the reference
 * file:line each entry point follows.
 *
 * Parallelism: rayon::join in the reference's merge_sort
 * (src/sample_sort.rs:253-256) becomes OpenMP tasks; rayon's par_iter over
 * subarrays/partitions (src/ext_mem.rs:1213, 1382, 1913) becomes
 * `omp parallel for`.
 */
#include "capssa_oracle.h"

#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

#if !defined(__BYTE_ORDER__) || __BYTE_ORDER__ != __ORDER_LITTLE_ENDIAN__
#error "the word-at-a-time LCP below assumes a little-endian host"
#endif

static inline uint64_t sat_mul(uint64_t a, uint64_t b) {
    if (a == 0 || b == 0) return 0;
    if (a > UINT64_MAX / b) return UINT64_MAX;
    return a * b;
}

/* Byte-level first-mismatch search.  The reference dispatches to AVX-512BW /
 * AVX2 / NEON / scalar variants (src/lcp.rs:249-431); all return the index of
 * the first differing byte below lim = min(n-p, n-q, max_ctx).  This portable
 * restatement compares 8-byte words and finds the byte with a trailing-zero
 * count, which yields the same value on a little-endian host. */
static inline uint64_t lcp_bytes(const uint8_t *t, uint64_t nb, uint64_t p,
                                 uint64_t q, uint64_t max) {
    uint64_t lim_p = nb > p ? nb - p : 0;
    uint64_t lim_q = nb > q ? nb - q : 0;
    uint64_t lim = lim_p < lim_q ? lim_p : lim_q;
    if (max < lim) lim = max;
    const uint8_t *a = t + p, *b = t + q;
    uint64_t i = 0;
    while (i + 8 <= lim) {
        uint64_t x, y;
        memcpy(&x, a + i, 8);
        memcpy(&y, b + i, 8);
        uint64_t d = x ^ y;
        if (d) return i + ((uint64_t)__builtin_ctzll(d) >> 3);
        i += 8;
    }
    while (i < lim) {
        if (a[i] != b[i]) return i;
        i++;
    }
    return i;
}

/* ---------------- LimitProvider (src/limits.rs) ---------------- */

#define DIR_MIN_ENDS 256ULL          /* src/limits.rs:207 */
#define DIR_MAX_BLOCKS 2000000ULL    /* src/limits.rs:208 */

static uint64_t next_pow2(uint64_t v) {
    if (v <= 1) return 1;
    if (v > (1ULL << 63)) return 1ULL << 63;
    v--;
    v |= v >> 1; v |= v >> 2; v |= v >> 4; v |= v >> 8; v |= v >> 16; v |= v >> 32;
    return v + 1;
}

/* SegmentedText::from_ends validation (src/limits.rs:261-282) and
 * BoundaryDirectory::build (src/limits.rs:210-235). */
int or_limits_init(or_limits *lp, uint64_t n, int segmented, int longer_first,
                   const uint64_t *ends, uint64_t n_ends) {
    memset(lp, 0, sizeof(*lp));
    lp->n = n;
    lp->segmented = segmented;
    lp->longer_first = longer_first;
    if (!segmented) return OR_OK;
    for (uint64_t i = 1; i < n_ends; i++)
        if (!(ends[i - 1] < ends[i])) return OR_EINVAL;
    if (n_ends == 0) {
        if (n != 0) return OR_EINVAL;
    } else if (ends[n_ends - 1] != n) {
        return OR_EINVAL;
    }
    lp->ends = ends;
    lp->n_ends = n_ends;
    if (n_ends < DIR_MIN_ENDS || n_ends > 0xFFFFFFFFULL || n == 0) return OR_OK;
    uint64_t target = n_ends * 2;
    if (target < 1) target = 1;
    if (target > DIR_MAX_BLOCKS) target = DIR_MAX_BLOCKS;
    uint64_t min_block = (n + target - 1) / target;
    uint64_t bs = next_pow2(min_block);
    uint32_t shift = (uint32_t)__builtin_ctzll(bs);
    uint64_t nb = (n + bs - 1) / bs;
    lp->dir = (uint32_t *)malloc((nb + 1) * sizeof(uint32_t));
    if (!lp->dir) return OR_ENOMEM;
    uint64_t e = 0;
    for (uint64_t b = 0; b <= nb; b++) {
        uint64_t bstart = b * bs < n ? b * bs : n;
        while (e < n_ends && ends[e] <= bstart) e++;
        lp->dir[b] = (uint32_t)e;
    }
    lp->n_dir = nb + 1;
    lp->block_shift = shift;
    return OR_OK;
}

void or_limits_free(or_limits *lp) {
    free(lp->dir);
    lp->dir = NULL;
}

int or_limits_has_directory(const or_limits *lp) { return lp->dir != NULL; }

/* first index i in [lo, hi) with ends[i] > p (partition_point(b <= p)) */
static inline uint64_t first_end_after(const uint64_t *ends, uint64_t lo,
                                       uint64_t hi, uint64_t p) {
    while (lo < hi) {
        uint64_t mid = lo + (hi - lo) / 2;
        if (ends[mid] <= p)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

/* PlainText::lim_at (src/limits.rs:144-148); SegmentedText::lim_at
 * (src/limits.rs:305-328). */
uint64_t or_lim_at(const or_limits *lp, uint64_t p) {
    if (!lp->segmented) return lp->n - p;
    if (lp->dir && p < lp->n) {
        uint64_t block = p >> lp->block_shift;
        uint64_t lo = lp->dir[block];
        uint64_t hi = lp->dir[block + 1];
        if (hi < lo + 1) hi = lo + 1;
        if (hi > lp->n_ends) hi = lp->n_ends;
        uint64_t i = first_end_after(lp->ends, lo, hi, p);
        return lp->ends[i] - p;
    }
    uint64_t i = first_end_after(lp->ends, 0, lp->n_ends, p);
    if (i < lp->n_ends) return lp->ends[i] - p;
    return lp->n - p;
}

/* LimitProvider::boundary_order default (src/limits.rs:66-75) and the STAR
 * override (src/sample_sort.rs:1006-1014). */
int or_boundary_order(const or_limits *lp, uint64_t p_a, uint64_t lim_a,
                      uint64_t p_b, uint64_t lim_b) {
    if (!lp->longer_first) return (lim_a > lim_b) - (lim_a < lim_b);
    if (lim_b != lim_a) return (lim_b > lim_a) - (lim_b < lim_a);
    return (p_a > p_b) - (p_a < p_b);
}

/* ---------------- LCP / comparator (src/lcp.rs) ---------------- */

uint64_t or_lcp(const void *text, uint64_t n, int sym_bytes, uint64_t p,
                uint64_t q, uint64_t max_ctx) {
    uint64_t k = (uint64_t)sym_bytes;
    uint64_t b = lcp_bytes((const uint8_t *)text, n * k, sat_mul(p, k), sat_mul(q, k),
                           sat_mul(max_ctx, k));
    return b / k;
}

static inline uint64_t sym_at(const void *text, int sym_bytes, uint64_t i) {
    switch (sym_bytes) {
    case 1: return ((const uint8_t *)text)[i];
    case 2: return ((const uint16_t *)text)[i];
    default: return ((const uint32_t *)text)[i];
    }
}

/* lcp_scalar (src/lcp.rs:233-246) */
uint64_t or_lcp_scalar(const void *text, uint64_t n, int sym_bytes, uint64_t p,
                       uint64_t q, uint64_t max_ctx) {
    uint64_t lim_p = n > p ? n - p : 0, lim_q = n > q ? n - q : 0;
    if (max_ctx < lim_p) lim_p = max_ctx;
    if (max_ctx < lim_q) lim_q = max_ctx;
    uint64_t lim = lim_p < lim_q ? lim_p : lim_q;
    uint64_t i = 0;
    while (i < lim) {
        if (sym_at(text, sym_bytes, p + i) != sym_at(text, sym_bytes, q + i)) return i;
        i++;
    }
    return i;
}

/* LcpDispatch::suffix_cmp_with (src/lcp.rs:184-201) */
int or_suffix_cmp(const void *text, int sym_bytes, const or_limits *lp,
                  uint64_t p, uint64_t q, uint64_t max_ctx) {
    uint64_t lim_p = or_lim_at(lp, p), lim_q = or_lim_at(lp, q);
    uint64_t lim = lim_p < lim_q ? lim_p : lim_q;
    if (max_ctx < lim) lim = max_ctx;
    uint64_t common = or_lcp(text, lp->n, sym_bytes, p, q, lim);
    if (common < lim) {
        uint64_t a = sym_at(text, sym_bytes, p + common);
        uint64_t b = sym_at(text, sym_bytes, q + common);
        return (a > b) - (a < b);
    }
    return or_boundary_order(lp, p, lim_p, q, lim_q);
}

/* ---------------- sample-sort sizing (src/ext_mem.rs) ---------------- */

#define PHASE1_TARGET_CHUNK 65536ULL  /* src/ext_mem.rs:1132 */
#define PHASE1_MAX_PARTITIONS 8192ULL /* src/ext_mem.rs:1136 */

/* effective_subproblem_count (src/ext_mem.rs:1159-1178) */
static uint64_t or_effective_subproblem_count(uint64_t n, uint64_t requested,
                                              uint64_t nthreads) {
    if (n == 0) return 0;
    uint64_t raw;
    if (requested == 0) {
        uint64_t nt = nthreads ? nthreads : 1;
        uint64_t from_size = (n + PHASE1_TARGET_CHUNK - 1) / PHASE1_TARGET_CHUNK;
        raw = from_size < nt ? nt : from_size;
        if (raw > PHASE1_MAX_PARTITIONS) raw = PHASE1_MAX_PARTITIONS;
    } else {
        raw = requested;
    }
    if (raw < 1) raw = 1;
    if (raw > n) raw = n;
    return raw;
}

/* sample_target_total (src/ext_mem.rs:1282-1287) */
static uint64_t or_sample_target_total(uint64_t n, uint64_t p) {
    double ln_n = log((double)n);
    if (ln_n < 1.0) ln_n = 1.0;
    uint64_t per = (uint64_t)ceil(4.0 * ln_n);
    uint64_t t = sat_mul(p, per);
    if (t < p) t = p;
    if (t > n) t = n;
    return t;
}

/* ---------------- per-(S, I) instantiations ---------------- */

#define S_T uint8_t
#define I_T uint32_t
#define SFX u8_u32
#include "oracle_tmpl.h"
#undef S_T
#undef I_T
#undef SFX
#define S_T uint8_t
#define I_T uint64_t
#define SFX u8_u64
#include "oracle_tmpl.h"
#undef S_T
#undef I_T
#undef SFX
#define S_T uint16_t
#define I_T uint32_t
#define SFX u16_u32
#include "oracle_tmpl.h"
#undef S_T
#undef I_T
#undef SFX
#define S_T uint16_t
#define I_T uint64_t
#define SFX u16_u64
#include "oracle_tmpl.h"
#undef S_T
#undef I_T
#undef SFX
#define S_T uint32_t
#define I_T uint32_t
#define SFX u32_u32
#include "oracle_tmpl.h"
#undef S_T
#undef I_T
#undef SFX
#define S_T uint32_t
#define I_T uint64_t
#define SFX u32_u64
#include "oracle_tmpl.h"
#undef S_T
#undef I_T
#undef SFX


int or_build_in_memory(const void *text, uint64_t n, int sym_bytes,
                       int idx_bytes, const void *positions, uint64_t m,
                       const or_limits *lp, uint64_t max_ctx, int threads,
                       void *out_sa, void *out_lcp) {
    if (lp->n != n) return OR_EINVAL;
    /* positions must address the text: p <= n (p == n is the empty suffix) */
    for (uint64_t i = 0; i < m; i++) {
        uint64_t p = idx_bytes == 4 ? ((const uint32_t *)positions)[i]
                                    : ((const uint64_t *)positions)[i];
        if (p > n) return OR_EINVAL;
    }
#define B_ARGS(S, I)                                                           \
    (const S *)text, n, (const I *)positions, m, lp, max_ctx, threads, (I *)out_sa, (I *)out_lcp
    if (sym_bytes == 1 && idx_bytes == 4) return build_u8_u32(B_ARGS(uint8_t, uint32_t));
    if (sym_bytes == 1 && idx_bytes == 8) return build_u8_u64(B_ARGS(uint8_t, uint64_t));
    if (sym_bytes == 2 && idx_bytes == 4) return build_u16_u32(B_ARGS(uint16_t, uint32_t));
    if (sym_bytes == 2 && idx_bytes == 8) return build_u16_u64(B_ARGS(uint16_t, uint64_t));
    if (sym_bytes == 4 && idx_bytes == 4) return build_u32_u32(B_ARGS(uint32_t, uint32_t));
    if (sym_bytes == 4 && idx_bytes == 8) return build_u32_u64(B_ARGS(uint32_t, uint64_t));
#undef B_ARGS
    return OR_EINVAL;
}

int or_merge(const void *text, int sym_bytes, int idx_bytes,
             const or_limits *lp, const void *x, uint64_t len_x,
             const void *lcp_x, const void *y, uint64_t len_y,
             const void *lcp_y, uint64_t max_ctx, void *z, void *lcp_z) {
#define M_CALL(S, I, SUF)                                                      \
    do {                                                                       \
        ctx_##SUF c = {(const S *)text, lp->n, lp, max_ctx};                   \
        merge_##SUF(&c, (const I *)x, len_x, (const I *)lcp_x, (const I *)y,   \
                    len_y, (const I *)lcp_y, (I *)z, (I *)lcp_z);              \
        return OR_OK;                                                          \
    } while (0)
    if (sym_bytes == 1 && idx_bytes == 4) M_CALL(uint8_t, uint32_t, u8_u32);
    if (sym_bytes == 1 && idx_bytes == 8) M_CALL(uint8_t, uint64_t, u8_u64);
    if (sym_bytes == 2 && idx_bytes == 4) M_CALL(uint16_t, uint32_t, u16_u32);
    if (sym_bytes == 2 && idx_bytes == 8) M_CALL(uint16_t, uint64_t, u16_u64);
    if (sym_bytes == 4 && idx_bytes == 4) M_CALL(uint32_t, uint32_t, u32_u32);
    if (sym_bytes == 4 && idx_bytes == 8) M_CALL(uint32_t, uint64_t, u32_u64);
#undef M_CALL
    return OR_EINVAL;
}

/* try_build_in_memory_sample_sort[_for_positions]_with picks u32 records when
 * text.len() <= u32::MAX + 1 (src/ext_mem.rs:763-782, 850-870). */
int or_sample_sort(const void *text, uint64_t n, int sym_bytes,
                   const uint64_t *positions, uint64_t m, const or_limits *lp,
                   uint64_t max_ctx, uint64_t requested_p, int threads,
                   uint64_t *out, uint64_t *out_p, uint64_t *out_pivots,
                   uint64_t *out_part_sizes, or_emit_fn emit, void *user) {
    if (lp->n != n) return OR_EINVAL;
    if (!positions) m = n;
    if (positions)
        for (uint64_t i = 0; i < m; i++)
            if (positions[i] > n) return OR_EINVAL;
    int idx = n <= 0xFFFFFFFFULL + 1 ? 4 : 8;
#define SS_ARGS(S)                                                             \
    (const S *)text, n, positions, m, lp, max_ctx, requested_p, threads, out, out_p, \
        out_pivots, out_part_sizes, emit, user
    if (sym_bytes == 1 && idx == 4) return sample_sort_u8_u32(SS_ARGS(uint8_t));
    if (sym_bytes == 1 && idx == 8) return sample_sort_u8_u64(SS_ARGS(uint8_t));
    if (sym_bytes == 2 && idx == 4) return sample_sort_u16_u32(SS_ARGS(uint16_t));
    if (sym_bytes == 2 && idx == 8) return sample_sort_u16_u64(SS_ARGS(uint16_t));
    if (sym_bytes == 4 && idx == 4) return sample_sort_u32_u32(SS_ARGS(uint32_t));
    if (sym_bytes == 4 && idx == 8) return sample_sort_u32_u64(SS_ARGS(uint32_t));
#undef SS_ARGS
    return OR_EINVAL;
}

/* ---------------- packed-prefix seed (src/pack.rs) ---------------- */

/* Packer::new + seed_params (src/pack.rs:103-176, 217-234).  The code table
 * is filled whenever a packer is available (identity when dense). */
int or_pack_params(const uint8_t *text, uint64_t n, int policy,
                   uint64_t max_extra_bytes, uint32_t *bits, uint32_t *k,
                   uint32_t *alphabet, uint8_t *code_table) {
    if (policy == 0) return 0;
    int present[256] = {0};
    for (uint64_t i = 0; i < n; i++) present[text[i]] = 1;
    uint32_t next = 0;
    int identity = 1;
    uint8_t code[256] = {0};
    for (int b = 0; b < 256; b++) {
        if (present[b]) {
            code[b] = (uint8_t)next;
            if ((int)next != b) identity = 0;
            next++;
        }
    }
    uint32_t bb = next <= 1 ? 1 : next <= 3 ? 2 : next <= 15 ? 4 : 8;
    if (!identity) {
        if (policy != 2) return 0;
        if (n > max_extra_bytes) return 0;
    }
    /* has_sentinel (src/pack.rs:174-176) */
    if (!((uint64_t)next < (1ULL << bb))) return 0;
    *bits = bb;
    *k = 64 / bb;
    *alphabet = next;
    for (int b = 0; b < 256; b++) code_table[b] = identity ? (uint8_t)b : code[b];
    return 1;
}

/* Packer::key_at_bounded (src/pack.rs:187-203) */
static inline uint64_t key_at_bounded(const uint8_t *text, uint64_t n,
                                      const uint8_t *code, uint32_t bits,
                                      uint32_t k, uint32_t alphabet,
                                      int longer_first, uint64_t p,
                                      uint64_t lim) {
    uint64_t take = k;
    if (lim < take) take = lim;
    if (n - p < take) take = n - p;
    uint64_t bias = longer_first ? 0 : 1;
    uint64_t pad = longer_first ? alphabet : 0;
    uint64_t key = 0;
    for (uint64_t i = 0; i < take; i++) key = (key << bits) | ((uint64_t)code[text[p + i]] + bias);
    for (uint64_t i = take; i < k; i++) key = (key << bits) | pad;
    return key;
}

void or_pack_keys(const uint8_t *text, uint64_t n, const uint8_t *code_table,
                  uint32_t bits, uint32_t k, uint32_t alphabet,
                  int longer_first, const or_limits *lp,
                  const uint64_t *positions, uint64_t m, uint64_t *keys) {
    for (uint64_t i = 0; i < m; i++) {
        uint64_t p = positions[i];
        keys[i] = key_at_bounded(text, n, code_table, bits, k, alphabet, longer_first, p,
                                 or_lim_at(lp, p));
    }
}

typedef struct {
    uint64_t key;
    uint64_t pos;
    uint64_t ord;
} keyed_t;

static int keyed_cmp(const void *a, const void *b) {
    const keyed_t *x = (const keyed_t *)a, *y = (const keyed_t *)b;
    if (x->key != y->key) return x->key < y->key ? -1 : 1;
    return (x->ord > y->ord) - (x->ord < y->ord);
}

/* seed_subarray (src/pack.rs:241-321).  The reference orders equal keys with
 * sort_unstable_by_key; here equal keys keep input order, which only matters
 * for comparator ties (never under PlainText or the STAR order). */
int or_seed_subarray(const uint8_t *text, uint64_t n, int idx_bytes,
                     const or_limits *lp, const uint8_t *code_table,
                     uint32_t bits, uint32_t k, uint32_t alphabet,
                     void *sa_v, void *lcp_v, uint64_t len) {
    if (len < 2) {
        if (len == 1) {
            if (idx_bytes == 4) ((uint32_t *)lcp_v)[0] = 0;
            else ((uint64_t *)lcp_v)[0] = 0;
        }
        return OR_OK;
    }
    keyed_t *kd = (keyed_t *)malloc(len * sizeof(keyed_t));
    if (!kd) return OR_ENOMEM;
    for (uint64_t i = 0; i < len; i++) {
        uint64_t p = idx_bytes == 4 ? ((uint32_t *)sa_v)[i] : ((uint64_t *)sa_v)[i];
        kd[i].key = key_at_bounded(text, n, code_table, bits, k, alphabet, lp->longer_first,
                                   p, or_lim_at(lp, p));
        kd[i].pos = p;
        kd[i].ord = i;
    }
    qsort(kd, len, sizeof(keyed_t), keyed_cmp);
    int rc = OR_OK;
#define SEED_BODY(I, SUF)                                                      \
    do {                                                                       \
        I *sa = (I *)sa_v, *lcp = (I *)lcp_v;                                  \
        for (uint64_t i = 0; i < len; i++) sa[i] = (I)kd[i].pos;               \
        I *sa_w = (I *)malloc(len * sizeof(I));                                \
        I *lcp_w = (I *)malloc(len * sizeof(I));                               \
        ctx_##SUF c = {text, n, lp, UINT64_MAX};                               \
        uint64_t i = 0;                                                        \
        while (i < len) {                                                      \
            uint64_t j = i + 1;                                                \
            while (j < len && kd[j].key == kd[i].key) j++;                     \
            if (j - i > 1)                                                     \
                merge_sort_task_local_##SUF(&c, sa + i, sa_w + i, lcp + i,     \
                                            lcp_w + i, j - i);                 \
            else                                                               \
                lcp[i] = 0;                                                    \
            if (i > 0) {                                                       \
                uint64_t a = sa[i - 1], b = sa[i];                             \
                uint64_t x = kd[i - 1].key ^ kd[i].key;                        \
                uint64_t shared = (x ? (uint64_t)__builtin_clzll(x) : 64) / bits; \
                uint64_t la = or_lim_at(lp, a), lb = or_lim_at(lp, b);         \
                if (la < shared) shared = la;                                  \
                if (lb < shared) shared = lb;                                  \
                lcp[i] = (I)shared;                                            \
            }                                                                  \
            i = j;                                                             \
        }                                                                      \
        lcp[0] = 0;                                                            \
        free(sa_w);                                                            \
        free(lcp_w);                                                           \
    } while (0)
    if (idx_bytes == 4)
        SEED_BODY(uint32_t, u8_u32);
    else
        SEED_BODY(uint64_t, u8_u64);
#undef SEED_BODY
    free(kd);
    return rc;
}

/* ---------------- brute force (test oracles) ---------------- */

typedef struct {
    const void *text;
    int sym_bytes;
    const or_limits *lp;
    uint64_t max_ctx;
} bf_ctx;

static int bf_less_eq(const bf_ctx *c, uint64_t a, uint64_t b) {
    int o = or_suffix_cmp(c->text, c->sym_bytes, c->lp, a, b, c->max_ctx);
    if (o != 0) return o < 0;
    return a <= b;
}

static void bf_sort(const bf_ctx *c, uint64_t *v, uint64_t *w, uint64_t n) {
    if (n < 2) return;
    uint64_t mid = n / 2;
    bf_sort(c, v, w, mid);
    bf_sort(c, v + mid, w, n - mid);
    uint64_t i = 0, j = mid, k = 0;
    while (i < mid && j < n) w[k++] = bf_less_eq(c, v[i], v[j]) ? v[i++] : v[j++];
    while (i < mid) w[k++] = v[i++];
    while (j < n) w[k++] = v[j++];
    memcpy(v, w, n * sizeof(uint64_t));
}

/* brute_force_sa / star_brute_force_sa restated (src/sample_sort.rs:643-647,
 * 1021-1040): a full-comparator sort, ties by ascending position. */
int or_brute_sa(const void *text, uint64_t n, int sym_bytes,
                const or_limits *lp, uint64_t max_ctx, const uint64_t *positions,
                uint64_t m, uint64_t *out) {
    (void)n;
    bf_ctx c = {text, sym_bytes, lp, max_ctx};
    for (uint64_t i = 0; i < m; i++) out[i] = positions ? positions[i] : i;
    uint64_t *w = (uint64_t *)malloc((m + 1) * sizeof(uint64_t));
    if (!w) return OR_ENOMEM;
    bf_sort(&c, out, w, m);
    free(w);
    return OR_OK;
}

int or_max_threads(void) { return omp_get_max_threads(); }

/* suffix_cmp_with (src/lcp.rs:184-201) of every adjacent pair of `sa`, in
 * parallel: out[i] = sign of cmp(sa[i], sa[i + 1]) for i < m - 1.  The
 * checker's tie classes (runs of 0) and order property (no +1) for outputs
 * too large for a per-pair call from the test driver. */
void or_adjacent_cmp(const void *text, int sym_bytes, const or_limits *lp, int idx_bytes,
                     const void *sa, uint64_t m, uint64_t max_ctx, int8_t *out) {
    if (m < 2) return;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)(m - 1); i++) {
        const uint64_t p = idx_bytes == 4 ? ((const uint32_t *)sa)[i] : ((const uint64_t *)sa)[i];
        const uint64_t q =
            idx_bytes == 4 ? ((const uint32_t *)sa)[i + 1] : ((const uint64_t *)sa)[i + 1];
        const int c = or_suffix_cmp(text, sym_bytes, lp, p, q, max_ctx);
        out[i] = (int8_t)(c < 0 ? -1 : c > 0 ? 1 : 0);
    }
}
