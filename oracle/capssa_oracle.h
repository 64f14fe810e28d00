/*
 * capssa_oracle.h — CPU restatement of caps-sa's in-memory suffix-array path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU library
 * and the timed CPU baseline; the product never links, loads or calls it.
 *
 * Every function restates one piece of the reference crate (caps-sa 0.7.0,
 * Rust) and cites the file:line it follows.  The reference cannot be compiled
 * in this environment (no rustc/cargo), so parity of this restatement is
 * pinned against the known-answer values in the reference's own unit tests
 * (tests/golden/ holds them together with the script that wrote them) and
 * against the reference's brute-force test oracles, restated here as
 * or_brute_sa_*.
 *
 * Conventions:
 *   - symbol widths: 1, 2, 4 bytes (u8 / u16 / u32, unsigned order);
 *   - index widths: 4, 8 bytes (u32 / u64), chosen per call like the
 *     reference's generic `I: Index`;
 *   - max_ctx == UINT64_MAX means unbounded (the reference's usize::MAX);
 *   - return codes: 0 ok, nonzero = contract violation the reference would
 *     panic on (OR_EINVAL) or an emit abort (OR_EEMIT).
 */
#ifndef CAPSSA_ORACLE_H
#define CAPSSA_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OR_OK 0
#define OR_EINVAL 1
#define OR_EEMIT 2
#define OR_ENOMEM 3

/* LimitProvider restatement (src/limits.rs:27-336).  `segmented` selects
 * SegmentedText (cumulative ends + coarse directory) over PlainText;
 * `longer_first` selects the STAR boundary order used by the reference's
 * tests (src/sample_sort.rs:1000-1015): lim_b.cmp(lim_a).then(p_a.cmp(p_b)),
 * with BoundaryRank::LongerFirst (src/pack.rs:347-349). */
typedef struct or_limits {
    uint64_t n;
    int segmented;
    int longer_first;
    const uint64_t *ends;
    uint64_t n_ends;
    uint32_t block_shift;
    uint32_t *dir; /* BoundaryDirectory::first_after_block_start or NULL */
    uint64_t n_dir;
} or_limits;

int or_limits_init(or_limits *lp, uint64_t n, int segmented, int longer_first,
                   const uint64_t *ends, uint64_t n_ends);
void or_limits_free(or_limits *lp);
uint64_t or_lim_at(const or_limits *lp, uint64_t p);
int or_limits_has_directory(const or_limits *lp);
int or_boundary_order(const or_limits *lp, uint64_t p_a, uint64_t lim_a,
                      uint64_t p_b, uint64_t lim_b);

/* LcpDispatch::lcp / suffix_cmp_with (src/lcp.rs:125-201). */
uint64_t or_lcp(const void *text, uint64_t n, int sym_bytes, uint64_t p,
                uint64_t q, uint64_t max_ctx);
uint64_t or_lcp_scalar(const void *text, uint64_t n, int sym_bytes, uint64_t p,
                       uint64_t q, uint64_t max_ctx);
int or_suffix_cmp(const void *text, int sym_bytes, const or_limits *lp,
                  uint64_t p, uint64_t q, uint64_t max_ctx);

/* build_in_memory_for_positions_with (src/sample_sort.rs:168-206).
 * positions/out_sa/out_lcp use `idx_bytes`-wide unsigned integers.
 * out_lcp may be NULL; when given it receives merge_sort's LCP postcondition
 * (src/sample_sort.rs:214-216).  `threads` <= 0 uses every core. */
int or_build_in_memory(const void *text, uint64_t n, int sym_bytes,
                       int idx_bytes, const void *positions, uint64_t m,
                       const or_limits *lp, uint64_t max_ctx, int threads,
                       void *out_sa, void *out_lcp);

/* sample_sort::merge (src/sample_sort.rs:397-522, drain :614-636). */
int or_merge(const void *text, int sym_bytes, int idx_bytes,
             const or_limits *lp, const void *x, uint64_t len_x,
             const void *lcp_x, const void *y, uint64_t len_y,
             const void *lcp_y, uint64_t max_ctx, void *z, void *lcp_z);

/* build_in_memory_sample_sort[_for_positions]_with
 * (src/ext_mem.rs:651-871, phases :1159-1428, :1705-1734, :1745-2389).
 * positions == NULL means every text position.  Emitted positions are
 * written in order to `out` (u64).  `requested_p` is ExtMemOpts
 * subproblem_count (0 = auto).  Optional outputs: the chosen p, the p-1
 * pivots (u64) and the p partition sizes. */
typedef int (*or_emit_fn)(void *user, const uint64_t *batch, uint64_t len);
int or_sample_sort(const void *text, uint64_t n, int sym_bytes,
                   const uint64_t *positions, uint64_t m, const or_limits *lp,
                   uint64_t max_ctx, uint64_t requested_p, int threads,
                   uint64_t *out, uint64_t *out_p, uint64_t *out_pivots,
                   uint64_t *out_part_sizes, or_emit_fn emit, void *user);

/* Packer (src/pack.rs:84-209) and seed_params (:217-234).
 * policy: 0 Disabled, 1 DenseAlphabetOnly, 2 Remap{max_extra_bytes}.
 * Returns 1 when a packer is available and fills bits/k/alphabet. */
int or_pack_params(const uint8_t *text, uint64_t n, int policy,
                   uint64_t max_extra_bytes, uint32_t *bits, uint32_t *k,
                   uint32_t *alphabet, uint8_t *code_table);
/* key_at_bounded for each position (src/pack.rs:187-203). */
void or_pack_keys(const uint8_t *text, uint64_t n, const uint8_t *code_table,
                  uint32_t bits, uint32_t k, uint32_t alphabet,
                  int longer_first, const or_limits *lp,
                  const uint64_t *positions, uint64_t m, uint64_t *keys);
/* seed_subarray (src/pack.rs:241-321); u8 text, idx_bytes-wide positions. */
int or_seed_subarray(const uint8_t *text, uint64_t n, int idx_bytes,
                     const or_limits *lp, const uint8_t *code_table,
                     uint32_t bits, uint32_t k, uint32_t alphabet,
                     void *sa, void *lcp, uint64_t m);

/* Brute-force test oracles (src/sample_sort.rs:643-647, 895-934,
 * 1021-1040): sort with a full suffix comparison, ties by position. */
int or_brute_sa(const void *text, uint64_t n, int sym_bytes,
                const or_limits *lp, uint64_t max_ctx, const uint64_t *positions,
                uint64_t m, uint64_t *out);

int or_max_threads(void);

/* Sign of suffix_cmp_with for every adjacent pair of sa (m - 1 entries). */
void or_adjacent_cmp(const void *text, int sym_bytes, const or_limits *lp, int idx_bytes,
                     const void *sa, uint64_t m, uint64_t max_ctx, int8_t *out);

/* Learned CDF model (no reference counterpart; cdf_oracle.c): 2 inputs from
 * the 64-bit packed prefix, OR_CDF_HIDDEN ReLU units, 1 output. */
#define OR_CDF_HIDDEN 64
#define OR_CDF_PARAMS (4 * OR_CDF_HIDDEN + 1)
void or_cdf_features(uint64_t prefix, float f[2]);
double or_cdf_forward(const float *params, uint64_t prefix);
double or_cdf_loss_grad(const float *params, const uint64_t *prefix, const float *target,
                        uint64_t n, double *grad);

#ifdef __cplusplus
}
#endif
#endif
