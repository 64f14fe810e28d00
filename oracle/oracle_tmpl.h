/*
 * oracle_tmpl.h — per-(symbol, index) instantiation of the merge-sort core.
 *
 * TEST INFRASTRUCTURE ONLY (see capssa_oracle.h).  Included by
 * capssa_oracle.c once per (S_T, I_T) pair with SFX naming the pair.
 *
 * The functions below restate, in order:
 *   merge_body!(direct) + merge + drain   src/sample_sort.rs:397-522, 614-636
 *   merge_sort (copy-back, rayon join)    src/sample_sort.rs:221-266
 *   merge_sort_task_local / ping_pong     src/sample_sort.rs:274-348
 *   build_in_memory_for_positions_with    src/sample_sort.rs:168-206
 */

#define OR_CAT2(a, b) a##_##b
#define OR_CAT(a, b) OR_CAT2(a, b)
#define FN(name) OR_CAT(name, SFX)

/* LcpDispatch::lcp with this symbol width (src/lcp.rs:125-153). */
static inline uint64_t FN(sym_lcp)(const S_T *text, uint64_t n, uint64_t p,
                                   uint64_t q, uint64_t max_ctx) {
    const uint64_t k = sizeof(S_T);
    uint64_t byte_lcp = lcp_bytes((const uint8_t *)text, n * k, sat_mul(p, k),
                                  sat_mul(q, k), sat_mul(max_ctx, k));
    return byte_lcp / k;
}

/* Shared state of one merge-sort invocation. */
typedef struct {
    const S_T *text;
    uint64_t n_text;
    const or_limits *lp;
    uint64_t max_ctx;
} FN(ctx);

/* sample_sort::merge — LCP-enhanced two-way merge with the swap-on-B
 * labelling (src/sample_sort.rs:397-502) and drain (:614-636). */
static void FN(merge)(const FN(ctx) *c, const I_T *x, uint64_t len_x,
                      const I_T *lcp_x, const I_T *y, uint64_t len_y,
                      const I_T *lcp_y, I_T *z, I_T *lcp_z) {
    if (len_x == 0) {
        memcpy(z, y, len_y * sizeof(I_T));
        memcpy(lcp_z, lcp_y, len_y * sizeof(I_T));
        return;
    }
    if (len_y == 0) {
        memcpy(z, x, len_x * sizeof(I_T));
        memcpy(lcp_z, lcp_x, len_x * sizeof(I_T));
        return;
    }
    const I_T *arr_a = x, *arr_b = y, *lcp_a = lcp_x, *lcp_b = lcp_y;
    uint64_t len_a = len_x, len_b = len_y;
    uint64_t i_a = 0, i_b = 0, m = 0, k = 0;
    /* lim caches keyed by the stream index (src/sample_sort.rs:427-461) */
    int ca_ok = 0, cb_ok = 0;
    uint64_t ca_idx = 0, ca_lim = 0, cb_idx = 0, cb_lim = 0;

    while (i_a < len_a && i_b < len_b) {
        uint64_t l_a = (uint64_t)lcp_a[i_a];
        int output_a;
        uint64_t lcp_out, new_m;
        if (l_a > m) {
            output_a = 1;
            lcp_out = l_a;
            new_m = m;
        } else if (l_a < m) {
            output_a = 0;
            lcp_out = m;
            new_m = l_a;
        } else {
            uint64_t p_a = (uint64_t)arr_a[i_a];
            uint64_t p_b = (uint64_t)arr_b[i_b];
            uint64_t lim_a, lim_b;
            if (ca_ok && ca_idx == i_a) {
                lim_a = ca_lim;
            } else {
                lim_a = or_lim_at(c->lp, p_a);
                ca_ok = 1;
                ca_idx = i_a;
                ca_lim = lim_a;
            }
            if (cb_ok && cb_idx == i_b) {
                lim_b = cb_lim;
            } else {
                lim_b = or_lim_at(c->lp, p_b);
                cb_ok = 1;
                cb_idx = i_b;
                cb_lim = lim_b;
            }
            uint64_t cap = lim_a < lim_b ? lim_a : lim_b;
            if (c->max_ctx < cap) cap = c->max_ctx;
            uint64_t remaining = cap > m ? cap - m : 0;
            uint64_t ext = FN(sym_lcp)(c->text, c->n_text, p_a + m, p_b + m, remaining);
            uint64_t total = m + ext;
            int a_smaller;
            if (total < cap) {
                a_smaller = c->text[p_a + total] < c->text[p_b + total];
            } else {
                a_smaller = or_boundary_order(c->lp, p_a, lim_a, p_b, lim_b) < 0;
            }
            output_a = a_smaller;
            lcp_out = m;
            new_m = total;
        }
        if (output_a) {
            z[k] = arr_a[i_a];
            lcp_z[k] = (I_T)lcp_out;
            i_a++;
            ca_ok = 0;
        } else {
            z[k] = arr_b[i_b];
            lcp_z[k] = (I_T)lcp_out;
            i_b++;
            cb_ok = 0;
            /* swap roles: the stream just output from becomes A */
            const I_T *t;
            uint64_t u;
            int o;
            t = arr_a; arr_a = arr_b; arr_b = t;
            t = lcp_a; lcp_a = lcp_b; lcp_b = t;
            u = len_a; len_a = len_b; len_b = u;
            u = i_a; i_a = i_b; i_b = u;
            o = ca_ok; ca_ok = cb_ok; cb_ok = o;
            u = ca_idx; ca_idx = cb_idx; cb_idx = u;
            u = ca_lim; ca_lim = cb_lim; cb_lim = u;
        }
        m = new_m;
        k++;
    }
    /* drain (src/sample_sort.rs:614-636): first drained record carries m */
    for (int side = 0; side < 2; side++) {
        const I_T *arr = side == 0 ? arr_a : arr_b;
        const I_T *lcs = side == 0 ? lcp_a : lcp_b;
        uint64_t i = side == 0 ? i_a : i_b;
        uint64_t len = side == 0 ? len_a : len_b;
        int first = 1;
        while (i < len) {
            z[k] = arr[i];
            lcp_z[k] = first ? (I_T)m : lcs[i];
            first = 0;
            i++;
            k++;
        }
    }
}

/* Below this many records the recursion stays on one thread (the rayon join
 * of src/sample_sort.rs:253-256 has near-zero cost; OpenMP tasks do not). */
#define OR_PAR_CUTOFF 8192

/* merge_sort with copy-back (src/sample_sort.rs:221-266). */
static void FN(merge_sort)(const FN(ctx) *c, I_T *sa, I_T *sa_w, I_T *lcp,
                           I_T *lcp_w, uint64_t n, int par) {
    if (n <= 1) {
        if (n == 1) lcp[0] = 0;
        return;
    }
    uint64_t mid = n / 2;
    if (par && n >= OR_PAR_CUTOFF) {
#pragma omp task
        FN(merge_sort)(c, sa, sa_w, lcp, lcp_w, mid, par);
        FN(merge_sort)(c, sa + mid, sa_w + mid, lcp + mid, lcp_w + mid, n - mid, par);
#pragma omp taskwait
    } else {
        FN(merge_sort)(c, sa, sa_w, lcp, lcp_w, mid, 0);
        FN(merge_sort)(c, sa + mid, sa_w + mid, lcp + mid, lcp_w + mid, n - mid, 0);
    }
    FN(merge)(c, sa, mid, lcp, sa + mid, n - mid, lcp + mid, sa_w, lcp_w);
    memcpy(sa, sa_w, n * sizeof(I_T));
    memcpy(lcp, lcp_w, n * sizeof(I_T));
}

/* merge_sort_ping_pong (src/sample_sort.rs:303-348). */
static void FN(ping_pong)(const FN(ctx) *c, I_T *src_sa, I_T *src_lcp,
                          I_T *dst_sa, I_T *dst_lcp, uint64_t n) {
    if (n <= 1) {
        if (n == 1) {
            dst_sa[0] = src_sa[0];
            dst_lcp[0] = 0;
        }
        return;
    }
    uint64_t mid = n / 2;
    FN(ping_pong)(c, dst_sa, dst_lcp, src_sa, src_lcp, mid);
    FN(ping_pong)(c, dst_sa + mid, dst_lcp + mid, src_sa + mid, src_lcp + mid, n - mid);
    FN(merge)(c, src_sa, mid, src_lcp, src_sa + mid, n - mid, src_lcp + mid, dst_sa, dst_lcp);
}

/* merge_sort_task_local (src/sample_sort.rs:274-300). */
static void FN(merge_sort_task_local)(const FN(ctx) *c, I_T *sa, I_T *sa_w,
                                      I_T *lcp, I_T *lcp_w, uint64_t n) {
    if (n == 0) return;
    memcpy(sa_w, sa, n * sizeof(I_T));
    FN(ping_pong)(c, sa_w, lcp_w, sa, lcp, n);
}

/* build_in_memory_for_positions_with (src/sample_sort.rs:168-206). */
static int FN(build)(const S_T *text, uint64_t n_text, const I_T *positions,
                     uint64_t m, const or_limits *lp, uint64_t max_ctx,
                     int threads, I_T *out_sa, I_T *out_lcp) {
    if (m == 0) return OR_OK;
    I_T *sa_w = (I_T *)malloc(m * sizeof(I_T));
    I_T *lcp = out_lcp ? out_lcp : (I_T *)malloc(m * sizeof(I_T));
    I_T *lcp_w = (I_T *)malloc(m * sizeof(I_T));
    if (!sa_w || !lcp || !lcp_w) {
        free(sa_w);
        if (!out_lcp) free(lcp);
        free(lcp_w);
        return OR_ENOMEM;
    }
    memcpy(out_sa, positions, m * sizeof(I_T));
    memset(lcp, 0, m * sizeof(I_T));
    FN(ctx) c = {text, n_text, lp, max_ctx};
    int nt = threads > 0 ? threads : omp_get_max_threads();
    if (nt > 1 && m >= OR_PAR_CUTOFF) {
#pragma omp parallel num_threads(nt)
#pragma omp single
        FN(merge_sort)(&c, out_sa, sa_w, lcp, lcp_w, m, 1);
    } else {
        FN(merge_sort)(&c, out_sa, sa_w, lcp, lcp_w, m, 0);
    }
    free(sa_w);
    free(lcp_w);
    if (!out_lcp) free(lcp);
    return OR_OK;
}

/* upper_bound_by_pivot (src/ext_mem.rs:1705-1734). */
static uint64_t FN(upper_bound)(const FN(ctx) *c, const I_T *recs, uint64_t len,
                                uint64_t pivot) {
    uint64_t lo = 0, hi = len;
    while (lo < hi) {
        uint64_t mid = lo + (hi - lo) / 2;
        int o = or_suffix_cmp(c->text, (int)sizeof(S_T), c->lp, (uint64_t)recs[mid],
                              pivot, c->max_ctx);
        if (o > 0)
            hi = mid;
        else
            lo = mid + 1;
    }
    return lo;
}

/* build_in_memory_ss_inner (src/ext_mem.rs:651-702) over InMemBucket, with
 * phase 1 (:1191-1277), phase 2 (:1309-1342), phase 3 (:1361-1428) and the
 * phase-4 cascade merge (:2046-2108, :2194-2389).  Partition pieces are
 * appended in subarray order (the reference's order depends on mutex
 * acquisition, :1415-1417, and does not affect PlainText output). */
static int FN(sample_sort)(const S_T *text, uint64_t n_text,
                           const uint64_t *positions, uint64_t n,
                           const or_limits *lp, uint64_t max_ctx,
                           uint64_t requested_p, int threads, uint64_t *out,
                           uint64_t *out_p, uint64_t *out_pivots,
                           uint64_t *out_part_sizes, or_emit_fn emit,
                           void *user) {
    if (n == 0) {
        if (out_p) *out_p = 0;
        return OR_OK;
    }
    int nt = threads > 0 ? threads : omp_get_max_threads();
    uint64_t p = or_effective_subproblem_count(n, requested_p, (uint64_t)nt);
    if (out_p) *out_p = p;
    uint64_t chunk = (n + p - 1) / p;
    uint64_t total_samples = or_sample_target_total(n, p);
    int task_local = p >= (uint64_t)nt;
    FN(ctx) c = {text, n_text, lp, max_ctx};

    /* phase 1: every subarray sorted into (sa, lcp) in one SoA arena */
    I_T *sa = (I_T *)malloc(n * sizeof(I_T));
    I_T *lcp = (I_T *)malloc(n * sizeof(I_T));
    I_T *sa_w = (I_T *)malloc(n * sizeof(I_T));
    I_T *lcp_w = (I_T *)malloc(n * sizeof(I_T));
    uint64_t per = (total_samples + p - 1) / p;
    I_T *samples = (I_T *)malloc((per * p + 1) * sizeof(I_T));
    uint64_t *n_samp = (uint64_t *)calloc(p, sizeof(uint64_t));
    if (!sa || !lcp || !sa_w || !lcp_w || !samples || !n_samp) {
        free(sa); free(lcp); free(sa_w); free(lcp_w); free(samples); free(n_samp);
        return OR_ENOMEM;
    }
    for (uint64_t i = 0; i < n; i++) sa[i] = (I_T)(positions ? positions[i] : i);

#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
    for (uint64_t i = 0; i < p; i++) {
        uint64_t start = i * chunk < n ? i * chunk : n;
        uint64_t end = (i + 1) * chunk < n ? (i + 1) * chunk : n;
        uint64_t len = end - start;
        if (len == 0) continue;
        memset(lcp + start, 0, len * sizeof(I_T));
        if (task_local) {
            FN(merge_sort_task_local)(&c, sa + start, sa_w + start, lcp + start,
                                      lcp_w + start, len);
        } else {
            FN(merge_sort)(&c, sa + start, sa_w + start, lcp + start, lcp_w + start, len, 0);
        }
        /* evenly_spaced midpoints (src/ext_mem.rs:1291-1305) */
        uint64_t cnt = per < len ? per : len;
        for (uint64_t s = 0; s < cnt; s++) {
            uint64_t at = cnt >= len ? s : (2 * s + 1) * len / (2 * cnt);
            samples[i * per + s] = sa[start + at];
        }
        n_samp[i] = cnt;
    }
    /* concatenate samples in subarray order */
    uint64_t ns = 0;
    for (uint64_t i = 0; i < p; i++)
        for (uint64_t s = 0; s < n_samp[i]; s++) samples[ns++] = samples[i * per + s];

    /* phase 2: sort samples with merge_sort, pivots at j*ns/p */
    uint64_t n_piv = (p > 1 && ns > 0) ? p - 1 : 0;
    I_T *pivots = (I_T *)malloc((n_piv + 1) * sizeof(I_T));
    if (n_piv) {
        I_T *s_w = (I_T *)malloc(ns * sizeof(I_T));
        I_T *s_l = (I_T *)calloc(ns, sizeof(I_T));
        I_T *s_lw = (I_T *)malloc(ns * sizeof(I_T));
        FN(merge_sort)(&c, samples, s_w, s_l, s_lw, ns, 0);
        for (uint64_t j = 1; j < p; j++) pivots[j - 1] = samples[(j * ns) / p];
        free(s_w); free(s_l); free(s_lw);
    }
    if (out_pivots)
        for (uint64_t j = 0; j < n_piv; j++) out_pivots[j] = (uint64_t)pivots[j];

    /* phase 3: split each subarray at the pivots' upper bounds */
    uint64_t *splits = (uint64_t *)malloc(p * (p + 1) * sizeof(uint64_t));
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
    for (uint64_t i = 0; i < p; i++) {
        uint64_t start = i * chunk < n ? i * chunk : n;
        uint64_t end = (i + 1) * chunk < n ? (i + 1) * chunk : n;
        uint64_t *sp = splits + i * (p + 1);
        sp[0] = 0;
        for (uint64_t j = 0; j < n_piv; j++)
            sp[j + 1] = FN(upper_bound)(&c, sa + start, end - start, (uint64_t)pivots[j]);
        for (uint64_t j = n_piv + 1; j <= p; j++) sp[j] = end - start;
    }
    /* partition j = concatenation over subarrays i of records[sp[j]..sp[j+1]) */
    uint64_t *part_off = (uint64_t *)calloc(p + 1, sizeof(uint64_t));
    for (uint64_t j = 0; j < p; j++) {
        uint64_t tot = 0;
        for (uint64_t i = 0; i < p; i++) {
            uint64_t *sp = splits + i * (p + 1);
            tot += sp[j + 1] - sp[j];
        }
        part_off[j + 1] = part_off[j] + tot;
        if (out_part_sizes) out_part_sizes[j] = tot;
    }
    /* gather pieces into sa_w/lcp_w, resetting each piece's first LCP
     * (InMemBucket::add_slice_reset_first_lcp, src/ext_bucket.rs:220-228) */
    uint64_t *run_start = (uint64_t *)malloc((p * p + 1) * sizeof(uint64_t));
    uint64_t *n_runs = (uint64_t *)calloc(p, sizeof(uint64_t));
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
    for (uint64_t j = 0; j < p; j++) {
        uint64_t o = part_off[j];
        uint64_t r = 0;
        for (uint64_t i = 0; i < p; i++) {
            uint64_t start = i * chunk < n ? i * chunk : n;
            uint64_t *sp = splits + i * (p + 1);
            uint64_t lo = sp[j], hi = sp[j + 1];
            if (lo >= hi) continue;
            memcpy(sa_w + o, sa + start + lo, (hi - lo) * sizeof(I_T));
            memcpy(lcp_w + o, lcp + start + lo, (hi - lo) * sizeof(I_T));
            lcp_w[o] = 0;
            run_start[j * p + r] = hi - lo; /* run length */
            r++;
            o += hi - lo;
        }
        n_runs[j] = r;
    }

    /* phase 4: cascade merge per partition (src/ext_mem.rs:2194-2389) */
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
    for (uint64_t j = 0; j < p; j++) {
        uint64_t base = part_off[j];
        uint64_t len = part_off[j + 1] - base;
        if (len == 0) continue;
        uint64_t *lens = run_start + j * p;
        uint64_t nr = n_runs[j];
        I_T *a_sa = sa_w + base, *a_lcp = lcp_w + base;
        I_T *b_sa = sa + base, *b_lcp = lcp + base;
        int src_is_a = 1;
        while (nr > 1) {
            I_T *ssa = src_is_a ? a_sa : b_sa, *slcp = src_is_a ? a_lcp : b_lcp;
            I_T *dsa = src_is_a ? b_sa : a_sa, *dlcp = src_is_a ? b_lcp : a_lcp;
            uint64_t so = 0, nn = 0;
            for (uint64_t r = 0; r < nr;) {
                uint64_t l1 = lens[r];
                if (r + 1 < nr) {
                    uint64_t l2 = lens[r + 1];
                    FN(merge)(&c, ssa + so, l1, slcp + so, ssa + so + l1, l2, slcp + so + l1,
                              dsa + so, dlcp + so);
                    lens[nn++] = l1 + l2;
                    so += l1 + l2;
                    r += 2;
                } else {
                    memcpy(dsa + so, ssa + so, l1 * sizeof(I_T));
                    memcpy(dlcp + so, slcp + so, l1 * sizeof(I_T));
                    lens[nn++] = l1;
                    so += l1;
                    r += 1;
                }
            }
            nr = nn;
            src_is_a = !src_is_a;
        }
        I_T *res = src_is_a ? a_sa : b_sa;
        for (uint64_t t = 0; t < len; t++) out[base + t] = (uint64_t)res[t];
    }
    int rc = OR_OK;
    if (emit) {
        /* ordered emit, partition by partition (src/ext_mem.rs:1932-1937) */
        for (uint64_t j = 0; j < p && rc == OR_OK; j++) {
            uint64_t len = part_off[j + 1] - part_off[j];
            if (len && emit(user, out + part_off[j], len) != 0) rc = OR_EEMIT;
        }
    }
    free(sa); free(lcp); free(sa_w); free(lcp_w); free(samples); free(n_samp);
    free(pivots); free(splits); free(part_off); free(run_start); free(n_runs);
    return rc;
}

#undef FN
#undef OR_CAT
#undef OR_CAT2
