/*
 * capssa.h — C ABI of the GB300 suffix-array library (libcapssa_gb300.so).
 *
 * Drop-in for the in-memory suffix-array path of caps-sa 0.7.0 (Rust):
 * every entry point below names the reference item it replaces
 * (file:line inside the caps-sa crate).  The reference is generic over
 * `S: Symbol` and `I: Index`; a Rust FFI shim binds one monomorphized symbol
 * per (S, I) pair, which is how the names are formed here:
 *     S in {u8, u16, u32}    I in {u32, u64}
 *
 * Buffers may live in host memory (pageable or pinned) or in device memory
 * of the context's GPU; the library inspects each pointer and copies as
 * needed.  All work of one context runs on its CUDA stream and every call
 * returns after its outputs are complete.  A context is not thread-safe;
 * use one per host thread.
 *
 * There is no CPU fallback: without a usable CUDA device every builder
 * returns CAPSSA_ECUDA.
 */
#ifndef CAPSSA_H
#define CAPSSA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CAPSSA_ABI_VERSION 5

typedef enum capssa_status {
    CAPSSA_OK = 0,
    /* a contract violation the reference panics on (bad segment ends,
     * position beyond the text, index type too narrow) */
    CAPSSA_EINVAL = 1,
    CAPSSA_ENOMEM = 2,
    CAPSSA_ECUDA = 3,
    /* a bounded device-side wait ran out; the context stays usable */
    CAPSSA_ETIMEOUT = 4,
    /* the emit callback returned nonzero (BuildError::Emit,
     * src/ext_mem.rs:258-264) */
    CAPSSA_EEMIT = 5,
    /* outside what this build supports (e.g. a text of 2^32-1 or more
     * symbols) */
    CAPSSA_EUNSUPPORTED = 6
} capssa_status;

/* LimitProvider (src/limits.rs:27-105) as a tagged descriptor.
 * kind PLAIN     = PlainText (src/limits.rs:125-156), ends ignored;
 * kind SEGMENTED = SegmentedText::from_ends (src/limits.rs:261-282):
 *                  strictly increasing cumulative ends, last == n.
 * boundary SHORTER_FIRST  = the default boundary_order, lim_a.cmp(lim_b)
 *                           (src/limits.rs:66-75), BoundaryRank::ShorterFirst;
 * boundary LONGER_FIRST   = STAR's spacer-as-largest order,
 *                           lim_b.cmp(lim_a).then(p_a.cmp(p_b))
 *                           (src/limits.rs:48-57), BoundaryRank::LongerFirst.
 * Arbitrary Rust boundary_order closures cannot cross the ABI. */
typedef enum { CAPSSA_LIMITS_PLAIN = 0, CAPSSA_LIMITS_SEGMENTED = 1 } capssa_limits_kind;
typedef enum { CAPSSA_SHORTER_FIRST = 0, CAPSSA_LONGER_FIRST = 1 } capssa_boundary;

typedef struct capssa_limits {
    int32_t kind;     /* capssa_limits_kind */
    int32_t boundary; /* capssa_boundary */
    const uint64_t *ends;
    uint64_t n_ends;
} capssa_limits;

/* How the sort's first level splits suffixes into buckets. */
typedef enum {
    CAPSSA_PARTITION_AUTO = 0,
    /* splitter suffixes drawn by the reference's sampling rule, bucket
     * found by binary search with the full comparator */
    CAPSSA_PARTITION_SPLITTERS = 1,
    /* as SPLITTERS, but a small MLP trained on the splitter sample
     * predicts the bucket; every prediction is checked against its two
     * neighbouring splitters and corrected */
    CAPSSA_PARTITION_LEARNED = 2,
    /* as SPLITTERS, but a plain binary search over all the splitters (the
     * reference's upper_bound_by_pivot, src/ext_mem.rs:1705-1734), without
     * the index of the splitters' leading key bits */
    CAPSSA_PARTITION_BISECT = 3
} capssa_partition;

/* Where the sample sort's splitter sample comes from. */
typedef enum {
    /* PARTITION_FIRST for the sample-sort builders and plans over a whole
     * text with an unbounded context; REFERENCE otherwise */
    CAPSSA_SAMPLING_AUTO = 0,
    /* the reference's rule (phase 1, src/ext_mem.rs:1191-1305): evenly
     * spaced midpoints of every sorted chunk of the input; the chunks'
     * order comes from the full sort, so the partition follows the sort */
    CAPSSA_SAMPLING_REFERENCE = 1,
    /* the same number of samples as evenly spaced midpoints of the input
     * order, sorted on their own; every suffix is bucketed by comparison
     * with the pivots before the sort, and the buckets drive it.  Texts
     * whose sample or pivot comparisons run deeper than 2^16 symbols fall
     * back to REFERENCE (same output) */
    CAPSSA_SAMPLING_PARTITION_FIRST = 2
} capssa_sampling;

/* Order inside a tie class: suffixes the comparator calls Equal, which only
 * SegmentedText under ShorterFirst has (equal symbols up to equal limits).
 * The reference leaves it unpinned (src/sample_sort.rs:908-913); its merge
 * sort emits each class in a fixed order all the same. */
typedef enum {
    /* ascending input order (position for a whole text, index in the
     * positions array for a subset) */
    CAPSSA_TIES_POSITION = 0,
    /* the order the reference's in-memory merge sort emits
     * (build_in_memory* and build_in_memory_for_positions*:
     * src/sample_sort.rs:221-266, 430-497); the in-memory builders only */
    CAPSSA_TIES_REFERENCE = 1
} capssa_tie_order;

/* Opts{max_context} (src/sample_sort.rs:70-85) and the in-memory subset of
 * ExtMemOpts (src/ext_mem.rs:60-118).  Zero-initialise, then set
 * max_context = CAPSSA_UNBOUNDED for the reference default. */
#define CAPSSA_UNBOUNDED UINT64_MAX
typedef struct capssa_opts {
    uint64_t max_context;      /* comparison cap; CAPSSA_UNBOUNDED default */
    uint64_t subproblem_count; /* p of the sample sort; 0 = auto rule of
                                  effective_subproblem_count, src/ext_mem.rs:1159-1178 */
    int32_t partition;         /* capssa_partition (sample-sort builders) */
    int32_t host_threads;      /* thread count the auto p rule assumes; 0 = all cores */
    uint64_t flags;            /* no flags are defined: 0 */
    int32_t sampling;          /* capssa_sampling (sample-sort builders and plans) */
    int32_t tie_order;         /* capssa_tie_order (in-memory builders) */
    uint64_t reserved[4];
} capssa_opts;

void capssa_opts_default(capssa_opts *o);

/* Per-call statistics of the last builder call on a context. */
typedef struct capssa_stats {
    uint64_t n_suffixes;        /* suffixes sorted */
    uint32_t key_symbols;       /* symbols per packed prefix key */
    uint32_t key_bits_per_symbol;
    uint32_t refine_rounds;     /* rank-doubling rounds after the key sort */
    uint32_t partitions;        /* buckets of the sample sort (0 if none) */
    uint64_t refined_suffixes;  /* sum over rounds of suffixes still tied */
    uint64_t max_partition;     /* largest bucket */
    uint64_t mispredicted;      /* learned partition: predictions corrected */
    uint64_t kernel_launches;   /* kernels launched by the call */
    double device_ms;           /* device time of the call (CUDA events) */
    double h2d_ms;
    double d2h_ms;
    uint64_t h2d_bytes;
    uint64_t d2h_bytes;
    /* device time per phase of the last suffix sort (CUDA events on the
     * context's stream) */
    double keys_ms;       /* alphabet scan + packed-key build */
    double sort_ms;       /* initial radix sort, all passes */
    double refine_ms;     /* rank-doubling rounds */
    double finish_ms;     /* bounded-context pass, output ordering and copy */
    uint32_t sort_passes; /* radix passes executed by the initial sort */
    uint32_t sort_item_bytes; /* bytes per record the radix passes move: 8 (position packed
                                 below the key) or 12 (key + separate u32 position) */
    double sort_pass_ms;  /* summed duration of those radix-pass kernels */
    /* sample-sort partition (capssa_build_in_memory_sample_sort_*) */
    double partition_ms;        /* bucket of every suffix (search or prediction + fixup) */
    double train_ms;            /* learned partition: model training */
    uint64_t partition_probes;  /* suffix-vs-splitter comparisons of the partition */
    uint32_t train_samples;     /* learned partition: samples the model trained on */
    float model_loss;           /* learned partition: final mean squared CDF error */
    uint32_t radix_items;       /* records per thread of the radix passes (the context's
                                   autotuner picks it on its first large sort of each kind) */
    uint32_t sparse_subset;     /* 1: a subset build sorted only its own positions */
    uint32_t tie_classes;       /* tie classes of the output (CAPSSA_TIES_REFERENCE) */
    uint32_t reserved_u32;
    double tie_order_ms;        /* device time of the reference tie order */
} capssa_stats;

typedef struct capssa_ctx capssa_ctx;

/* Create a context on CUDA device `device`. */
capssa_status capssa_ctx_create(capssa_ctx **out, int device);
void capssa_ctx_destroy(capssa_ctx *ctx);
/* Run the context's work on an existing cudaStream_t (NULL = own stream). */
capssa_status capssa_ctx_set_stream(capssa_ctx *ctx, void *cuda_stream);
/* Text of the last error on this context ("" if none). */
const char *capssa_ctx_last_error(const capssa_ctx *ctx);
capssa_status capssa_ctx_stats(const capssa_ctx *ctx, capssa_stats *out);
/* Device bytes currently held by the context's workspace. */
uint64_t capssa_ctx_workspace_bytes(const capssa_ctx *ctx);
/* Release the context's cached workspace. */
void capssa_ctx_trim(capssa_ctx *ctx);
int capssa_abi_version(void);

/* Emit callback of the sample-sort builders: called in suffix order with
 * consecutive batches of positions (u64).  The reference calls
 * FnMut(u64) -> Result<(), E> once per position (src/ext_mem.rs:1932-1937);
 * a per-position FFI call would cost more than the sort, so batches cross
 * instead.  Return 0 to continue, nonzero to abort (-> CAPSSA_EEMIT). */
typedef int (*capssa_emit_fn)(void *user, const uint64_t *positions, uint64_t len);

/* ---------------------------------------------------------------------
 * Builders
 * ------------------------------------------------------------------- */

/* build_in_memory / _with_opts / _with (src/sample_sort.rs:97-127):
 * the suffix array of `text` (n symbols) into out_sa[0..n).
 * lp == NULL means PlainText, opts == NULL means Opts::default(). */
#define CAPSSA_DECL_BUILD(S, ST, I, IT)                                                   \
    capssa_status capssa_build_in_memory_##S##_##I(capssa_ctx *ctx, const ST *text,       \
                                                   uint64_t n, const capssa_limits *lp,   \
                                                   const capssa_opts *opts, IT *out_sa);

/* build_in_memory_for_positions / _with_opts / _with
 * (src/sample_sort.rs:143-206): the given positions (each <= n) reordered
 * by suffix into out_sa[0..m). */
#define CAPSSA_DECL_BUILD_POS(S, ST, I, IT)                                               \
    capssa_status capssa_build_in_memory_for_positions_##S##_##I(                         \
        capssa_ctx *ctx, const ST *text, uint64_t n, const IT *positions, uint64_t m,     \
        const capssa_limits *lp, const capssa_opts *opts, IT *out_sa);

/* merge_sort's postcondition (src/sample_sort.rs:208-216) exposed: the
 * suffix array plus lcp[0] = 0, lcp[i] = lcp(sa[i-1], sa[i]) capped by both
 * limits and max_context.  positions == NULL sorts every position. */
#define CAPSSA_DECL_BUILD_LCP(S, ST, I, IT)                                               \
    capssa_status capssa_build_in_memory_lcp_##S##_##I(                                   \
        capssa_ctx *ctx, const ST *text, uint64_t n, const IT *positions, uint64_t m,     \
        const capssa_limits *lp, const capssa_opts *opts, IT *out_sa, IT *out_lcp);

/* sample_sort::merge (src/sample_sort.rs:397-522, drain :614-636): merge two
 * LCP-annotated sorted runs into z / lcp_z (len_x + len_y), with the
 * reference's tie rule (a comparator tie outputs the stream not last
 * output from). */
#define CAPSSA_DECL_MERGE(S, ST, I, IT)                                                   \
    capssa_status capssa_merge_##S##_##I(                                                 \
        capssa_ctx *ctx, const ST *text, uint64_t n, const capssa_limits *lp,             \
        const IT *x, const IT *lcp_x, uint64_t len_x, const IT *y, const IT *lcp_y,       \
        uint64_t len_y, uint64_t max_context, IT *z, IT *lcp_z);

/* build_in_memory_sample_sort[_with] / try_* (src/ext_mem.rs:711-783):
 * positions emitted in suffix order through `emit`. */
#define CAPSSA_DECL_SS(S, ST)                                                             \
    capssa_status capssa_build_in_memory_sample_sort_##S(                                 \
        capssa_ctx *ctx, const ST *text, uint64_t n, const capssa_limits *lp,             \
        const capssa_opts *opts, capssa_emit_fn emit, void *user);                        \
    /* build_in_memory_sample_sort_for_positions[_with] / try_*                           \
     * (src/ext_mem.rs:785-871) */                                                        \
    capssa_status capssa_build_in_memory_sample_sort_for_positions_##S(                   \
        capssa_ctx *ctx, const ST *text, uint64_t n, const uint64_t *positions,           \
        uint64_t m, const capssa_limits *lp, const capssa_opts *opts, capssa_emit_fn emit, \
        void *user);                                                                      \
    /* LcpDispatch::lcp (src/lcp.rs:125-153) for `count` pairs (p[i], q[i]) */            \
    capssa_status capssa_lcp_##S(capssa_ctx *ctx, const ST *text, uint64_t n,             \
                                 const uint64_t *p, const uint64_t *q, uint64_t count,    \
                                 uint64_t max_context, uint64_t *out);                    \
    /* LcpDispatch::suffix_cmp_with (src/lcp.rs:184-201): -1, 0, 1 per pair */            \
    capssa_status capssa_suffix_cmp_##S(capssa_ctx *ctx, const ST *text, uint64_t n,      \
                                        const capssa_limits *lp, const uint64_t *p,       \
                                        const uint64_t *q, uint64_t count,                \
                                        uint64_t max_context, int8_t *out);

/* Many independent texts in one launch sequence: texts[offsets[t] ..
 * offsets[t+1]) is text t (offsets has n_texts+1 entries, offsets[0] == 0).
 * out_sa[offsets[t] + i] receives the i-th suffix of text t as a position
 * local to that text, exactly build_in_memory(text_t). */
#define CAPSSA_DECL_BATCHED(S, ST, I, IT)                                                 \
    capssa_status capssa_build_batched_##S##_##I(                                         \
        capssa_ctx *ctx, const ST *texts, const uint64_t *offsets, uint64_t n_texts,      \
        const capssa_opts *opts, IT *out_sa);

/* build_ext_mem_for_filter's position source (FilteredSource, bitmap +
 * popcount select, src/ext_mem.rs:927-1092) for the in-memory builder: the
 * positions p with lo <= text[p] < hi, sorted by suffix (as
 * build_in_memory_for_positions_with would sort them), selected on the GPU
 * by stream compaction.  *m_out = their count; out_sa (capacity >= the
 * count) may be null to learn the count only. */
#define CAPSSA_DECL_FILTER(S, ST, I, IT)                                                  \
    capssa_status capssa_build_in_memory_for_filter_##S##_##I(                            \
        capssa_ctx *ctx, const ST *text, uint64_t n, uint64_t lo, uint64_t hi,            \
        const capssa_limits *lp, const capssa_opts *opts, IT *out_sa, uint64_t *m_out);

/* build_ext_mem[_with] / try_* (src/ext_mem.rs:279-338), and the
 * _for_positions (src/ext_mem.rs:370-453) and _for_filter (keep =
 * lo <= text[p] < hi, src/ext_mem.rs:472-553) variants: every suffix (or
 * the given / kept positions) streamed to `emit` in suffix order, host
 * memory bounded by the text and two 32 MiB emit batches.  The working set
 * stays in device memory, so nothing is spilled to temp files (the
 * reference's work_dir / physical_file_count have no counterpart).
 * _for_filter reports the kept count in *m_out when m_out is not null. */
#define CAPSSA_DECL_EXTMEM(S, ST)                                                         \
    capssa_status capssa_build_ext_mem_##S(capssa_ctx *ctx, const ST *text, uint64_t n,   \
                                           const capssa_limits *lp,                       \
                                           const capssa_opts *opts, capssa_emit_fn emit,  \
                                           void *user);                                   \
    capssa_status capssa_build_ext_mem_for_positions_##S(                                 \
        capssa_ctx *ctx, const ST *text, uint64_t n, const uint64_t *positions,           \
        uint64_t m, const capssa_limits *lp, const capssa_opts *opts, capssa_emit_fn emit, \
        void *user);                                                                      \
    capssa_status capssa_build_ext_mem_for_filter_##S(                                    \
        capssa_ctx *ctx, const ST *text, uint64_t n, uint64_t lo, uint64_t hi,            \
        const capssa_limits *lp, const capssa_opts *opts, capssa_emit_fn emit, void *user, \
        uint64_t *m_out);

#define CAPSSA_DECL_ALL_I(S, ST)                                                          \
    CAPSSA_DECL_BUILD(S, ST, u32, uint32_t)                                               \
    CAPSSA_DECL_BUILD(S, ST, u64, uint64_t)                                               \
    CAPSSA_DECL_BUILD_POS(S, ST, u32, uint32_t)                                           \
    CAPSSA_DECL_BUILD_POS(S, ST, u64, uint64_t)                                           \
    CAPSSA_DECL_BUILD_LCP(S, ST, u32, uint32_t)                                           \
    CAPSSA_DECL_BUILD_LCP(S, ST, u64, uint64_t)                                           \
    CAPSSA_DECL_MERGE(S, ST, u32, uint32_t)                                               \
    CAPSSA_DECL_MERGE(S, ST, u64, uint64_t)                                               \
    CAPSSA_DECL_BATCHED(S, ST, u32, uint32_t)                                             \
    CAPSSA_DECL_BATCHED(S, ST, u64, uint64_t)                                             \
    CAPSSA_DECL_FILTER(S, ST, u32, uint32_t)                                              \
    CAPSSA_DECL_FILTER(S, ST, u64, uint64_t)                                              \
    CAPSSA_DECL_SS(S, ST)                                                                 \
    CAPSSA_DECL_EXTMEM(S, ST)

CAPSSA_DECL_ALL_I(u8, uint8_t)
CAPSSA_DECL_ALL_I(u16, uint16_t)
CAPSSA_DECL_ALL_I(u32, uint32_t)

/* ---------------------------------------------------------------------
 * Packed-prefix keys (src/pack.rs), u8 text only like the reference
 * (seed_params requires S == u8, src/pack.rs:223-228).
 * ------------------------------------------------------------------- */

typedef enum {
    CAPSSA_SEED_DISABLED = 0,
    CAPSSA_SEED_DENSE_ALPHABET_ONLY = 1,
    CAPSSA_SEED_REMAP = 2
} capssa_seed_policy;

typedef struct capssa_packer {
    uint32_t bits;      /* bits per packed field */
    uint32_t k;         /* symbols per u64 key */
    uint32_t alphabet;  /* distinct symbols; `alphabet` is the sentinel */
    uint32_t identity;  /* 1 when codes equal the bytes */
    uint8_t code[256];  /* byte -> code (order preserving) */
} capssa_packer;

/* Packer::new + seed_params (src/pack.rs:103-176, 217-234).  Returns
 * CAPSSA_OK and *available = 1 when a packer exists. */
capssa_status capssa_pack_params_u8(capssa_ctx *ctx, const uint8_t *text, uint64_t n,
                                    int32_t policy, uint64_t max_extra_bytes,
                                    capssa_packer *out, int32_t *available);
/* Packer::key_at_bounded for each position (src/pack.rs:187-203). */
capssa_status capssa_pack_keys_u8(capssa_ctx *ctx, const uint8_t *text, uint64_t n,
                                  const capssa_packer *pk, const capssa_limits *lp,
                                  const uint64_t *positions, uint64_t m, uint64_t *keys);
/* seed_subarray (src/pack.rs:241-321): sort `sa` in place by suffix using
 * the packed keys first, and fill lcp. */
capssa_status capssa_seed_subarray_u8_u32(capssa_ctx *ctx, const uint8_t *text, uint64_t n,
                                          const capssa_packer *pk, const capssa_limits *lp,
                                          uint32_t *sa, uint32_t *lcp, uint64_t m);
capssa_status capssa_seed_subarray_u8_u64(capssa_ctx *ctx, const uint8_t *text, uint64_t n,
                                          const capssa_packer *pk, const capssa_limits *lp,
                                          uint64_t *sa, uint64_t *lcp, uint64_t m);

/* ---------------------------------------------------------------------
 * Allocation-free merge.  No counterpart in the reference: it exists for
 * callers that cannot call cudaMalloc where they need a merge (an
 * application whose own pool allocator owns all device memory, a stream
 * where the synchronisation an allocation may imply is not acceptable, or a
 * caller without a capssa_ctx).
 *
 * Same result as capssa_merge_u8_u32, bit for bit, but it allocates
 * nothing: every pointer is a device pointer owned by the caller, and the
 * merge-path scratch lives in a fixed static device array of about 1.2 MiB that every GPU loading the
 * library holds until the process exits.
 *   - len_x + len_y must be at most 2^24 records; larger merges return
 *     CAPSSA_EINVAL.
 *   - text must be followed by at least 64 readable bytes (the vector LCP
 *     reads past the last compared byte).
 *   - ends == NULL / n_ends == 0 means PlainText; otherwise SegmentedText
 *     ends on the device (checked like from_ends).  boundary is a
 *     capssa_boundary.
 *   - runs on `cuda_stream` (NULL = legacy default stream) of the current
 *     device and returns after the merge has finished.  Every call looks up
 *     the scratch array's device address in the current context; the first
 *     call on a device also loads the library's device code, so make that
 *     first call before any stream capture.  An error already pending on
 *     the calling thread is reported as CAPSSA_ECUDA and left pending.
 *   - every call shares the one scratch array (it keeps the last call's
 *     contents); calls that overlap on the GPU, on any streams or host
 *     threads, race on it and must be serialised by the caller.
 * Returns CAPSSA_EINVAL for contract violations (position > n, bad ends,
 * oversize merge), CAPSSA_ECUDA for CUDA errors; no error text is kept. */
capssa_status capssa_merge_noalloc_u8_u32(void *cuda_stream, const uint8_t *text, uint64_t n,
                                          const uint64_t *ends, uint64_t n_ends,
                                          int32_t boundary, const uint32_t *x,
                                          const uint32_t *lcp_x, uint64_t len_x,
                                          const uint32_t *y, const uint32_t *lcp_y,
                                          uint64_t len_y, uint64_t max_context, uint32_t *z,
                                          uint32_t *lcp_z);

/* ---------------------------------------------------------------------
 * Sample-sort partition plan.
 *
 * The partition that capssa_build_in_memory_sample_sort_* computes before it
 * emits: the subproblem count p (effective_subproblem_count,
 * src/ext_mem.rs:1159-1178), the p - 1 pivots (phase 2, src/ext_mem.rs:
 * 1309-1342: samples drawn as evenly spaced midpoints of every sorted chunk,
 * :1191-1305, sorted, pivots at samples[j*ns/p]) and the size of every
 * partition (phase 3, src/ext_mem.rs:1361-1428: a suffix s belongs to
 * partition b = the number of pivots that compare less than s under
 * suffix_cmp_with).  opts->partition selects how b is found: by binary
 * search over the pivots (SPLITTERS, also AUTO), or by the learned CDF model
 * trained on the sample and checked against its neighbouring pivots
 * (LEARNED); both give the same b.  Pass null pivots/sizes to learn p first
 * (*p_out); otherwise they hold p - 1 and p entries.  positions may be null
 * (every suffix) or host/device u64 (m entries).
 * ------------------------------------------------------------------- */
#define CAPSSA_DECL_PLAN(S, ST)                                                               \
    capssa_status capssa_sample_sort_plan_##S(capssa_ctx *ctx, const ST *text, uint64_t n,   \
                                              const uint64_t *positions, uint64_t m,         \
                                              const capssa_limits *lp,                       \
                                              const capssa_opts *opts, uint64_t *p_out,      \
                                              uint64_t *pivots, uint64_t *sizes);
CAPSSA_DECL_PLAN(u8, uint8_t)
CAPSSA_DECL_PLAN(u16, uint16_t)
CAPSSA_DECL_PLAN(u32, uint32_t)

/* ---------------------------------------------------------------------
 * Learned CDF model of the learned partition (no reference counterpart).
 * 2 inputs from a 64-bit packed prefix (hi32 * 2^-31 - 1, lo32 * 2^-31 - 1),
 * 64 ReLU units, 1 output; CAPSSA_CDF_PARAMS floats laid out w1[h*2+d],
 * b1[h], w2[h], b2.  Host or device buffers.
 *
 * capssa_cdf_grad: mean-squared-error loss and its gradient over n
 * (prefix, target) samples, from the GPU forward/backward kernels that the
 * learned partition trains with.
 * capssa_cdf_train: `steps` full-batch Adam steps from the built-in
 * initialisation (the training the learned partition runs); writes the
 * trained parameters and the final loss.
 * capssa_cdf_infer: the model's output for n prefixes exactly as the
 * learned partition evaluates it: the parameters rounded to BF16, layer 1 on
 * the tensor cores (mma.sync m16n8k16, fp32 accumulation, each input split
 * into a BF16 high part and the BF16 rounding of its remainder), layer 2 in
 * fp32.
 * ------------------------------------------------------------------- */
/* Failure-detection self-test (no reference counterpart): one kernel
 * waits on a device word that nothing sets, polling `polls` times (1..2^20)
 * with the bounded wait every look-back uses, and gives up; the call returns
 * CAPSSA_ETIMEOUT and the context stays usable.  No GPU fault is involved. */
capssa_status capssa_selftest_bounded_wait(capssa_ctx *ctx, uint32_t polls);

#define CAPSSA_CDF_PARAMS 257
capssa_status capssa_cdf_grad(capssa_ctx *ctx, const float *params, const uint64_t *prefixes,
                              const float *targets, uint64_t n, float *grad, float *loss);
capssa_status capssa_cdf_train(capssa_ctx *ctx, const uint64_t *prefixes, const float *targets,
                               uint64_t n, int32_t steps, float *params, float *loss);
capssa_status capssa_cdf_infer(capssa_ctx *ctx, const float *params, const uint64_t *prefixes,
                               uint64_t n, float *out);

/* ---------------------------------------------------------------------
 * On-disk formats and emit sinks.
 *
 * capssa_emit_file_u64 / capssa_emit_file_u32: capssa_emit_fn sinks that
 * append each batch to the FILE* passed as `user` as little-endian u64 or
 * u32 values, the SA files of examples/caps_sa.rs:131-139 (u32) and
 * :147-172 (u64 stream).  They return nonzero (abort) on a write error, and
 * _u32 also on a position >= 2^32.
 *
 * capssa_checksum128: the order-sensitive 128-bit checksum the ruSTAR
 * replay prints over an emitted stream (examples/rustar_segmented_bench.rs:
 * 236-245).  Start from capssa_checksum128_init, feed the positions in
 * order; capssa_emit_checksum128 is the same as an emit sink
 * (user = capssa_checksum128 *).
 *
 * capssa_sa_lcp_records_{I}: SA and LCP arrays interleaved into SaLcp<I>
 * bucket records (pos, lcp), little-endian, 8 or 16 bytes each
 * (src/ext_bucket.rs:65-108), on the GPU; host or device buffers.
 * ------------------------------------------------------------------- */
typedef struct capssa_checksum128 {
    uint64_t count;
    uint64_t lo, hi; /* the 128-bit state */
} capssa_checksum128;
void capssa_checksum128_init(capssa_checksum128 *c);
void capssa_checksum128_update(capssa_checksum128 *c, const uint64_t *positions, uint64_t len);
int capssa_emit_checksum128(void *user, const uint64_t *positions, uint64_t len);
int capssa_emit_file_u64(void *user, const uint64_t *positions, uint64_t len);
int capssa_emit_file_u32(void *user, const uint64_t *positions, uint64_t len);
capssa_status capssa_sa_lcp_records_u32(capssa_ctx *ctx, const uint32_t *sa, const uint32_t *lcp,
                                        uint64_t n, void *out_records);
capssa_status capssa_sa_lcp_records_u64(capssa_ctx *ctx, const uint64_t *sa, const uint64_t *lcp,
                                        uint64_t n, void *out_records);

#ifdef __cplusplus
}
#endif
#endif /* CAPSSA_H */
