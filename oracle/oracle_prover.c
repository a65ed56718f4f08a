/*
 * ORACLE — test infrastructure only. The reference's generic prover flow
 * (prove_ex, the commitment scheme, FRI, lifted Merkle decommitment and the
 * CairoSerialize felt stream) restated in C over this oracle's CPU ops, so that
 * whole proofs of the CUDA path are checked against a second, independent
 * statement of the protocol. Nothing here is shared with the product's
 * provers; each step cites the reference function it follows.
 *
 * Supported proofs (the AIRs the native provers implement):
 *   orc_prove_fib_and_lookups — Wide-Fibonacci components
 *     (crates/examples/src/wide_fibonacci/mod.rs:76-98) and single-column
 *     LogUp components (relation entry of multiplicity -1 and values [v],
 *     finalize_logup, crates/constraint-framework/src/lib.rs:185-227), one
 *     lifted tree per phase, log_blowup_factor 1 (SubDomain evaluation with
 *     log_expansion 0, crates/stwo/src/prover/air/accumulation.rs:42-62).
 *   orc_prove_poseidon — the Poseidon2 AIR of crates/examples/src/poseidon/
 *     mod.rs:320-379 (ExtendToEvalDomain, coefficients stored).
 * FRI folds fold_step times per layer (leaves of 4 values when it is above one).
 */
#include <stdlib.h>
#include <string.h>

#include "blake2s.h"
#include "circle.h"
#include "fields.h"
#include "oracle.h"

/* ------------------------------------------------------------------ felt stream */

typedef struct {
    uint64_t *w;
    size_t n, cap;
} felts_t;

static void fpush(felts_t *f, uint64_t v) {
    if (f->n == f->cap) {
        f->cap = f->cap ? 2 * f->cap : 4096;
        f->w = (uint64_t *)realloc(f->w, sizeof(uint64_t) * f->cap);
    }
    f->w[f->n++] = v;
}
/* SecureField: its 4 M31 coordinates (crates/cairo-serialize/src/serialize.rs:45-49). */
static void fpush_qm31(felts_t *f, qm31 x) {
    fpush(f, x.a.a); fpush(f, x.a.b); fpush(f, x.b.a); fpush(f, x.b.b);
}
/* Blake2sHash: 8 little-endian u32 words (serialize.rs:203-210). */
static void fpush_hash(felts_t *f, const uint8_t h[32]) {
    for (int k = 0; k < 8; k++)
        fpush(f, (uint64_t)h[4 * k] | ((uint64_t)h[4 * k + 1] << 8) | ((uint64_t)h[4 * k + 2] << 16) |
                     ((uint64_t)h[4 * k + 3] << 24));
}

/* ------------------------------------------------------------------ small helpers */

static int cmp_u32(const void *a, const void *b) {
    uint32_t x = *(const uint32_t *)a, y = *(const uint32_t *)b;
    return x < y ? -1 : x > y;
}
/* sort + dedup in place (Queries::new, crates/stwo/src/core/queries.rs:41-46); returns the new length */
static uint32_t sort_dedup(uint32_t *v, uint32_t n) {
    qsort(v, n, sizeof(uint32_t), cmp_u32);
    uint32_t m = 0;
    for (uint32_t i = 0; i < n; i++)
        if (m == 0 || v[m - 1] != v[i]) v[m++] = v[i];
    return m;
}

static qpoint qpoint_double(qpoint p) {
    /* CirclePoint::double: (2x^2 - 1, 2xy) */
    qm31 xy = qm31_mul(p.x, p.y);
    qpoint r = {qcircle_double_x(p.x), qm31_add(xy, xy)};
    return r;
}
static qpoint qpoint_repeated_double(qpoint p, uint32_t n) {
    for (uint32_t i = 0; i < n; i++) p = qpoint_double(p);
    return p;
}
static qpoint qpoint_add_m31(qpoint p, cpoint q) { return qpoint_add(p, qpoint_from_cpoint(q)); }
static int qpoint_eq(qpoint a, qpoint b) { return qm31_eq(a.x, b.x) && qm31_eq(a.y, b.y); }
/* the derived Ord of (QM31, QM31): lexicographic over the 8 coordinates */
static int qpoint_cmp(qpoint a, qpoint b) {
    uint32_t wa[8], wb[8];
    qm31_to_words(a.x, wa); qm31_to_words(a.y, wa + 4);
    qm31_to_words(b.x, wb); qm31_to_words(b.y, wb + 4);
    for (int k = 0; k < 8; k++)
        if (wa[k] != wb[k]) return wa[k] < wb[k] ? -1 : 1;
    return 0;
}

/* QM31::from_partial_evals (crates/stwo/src/core/fields/qm31.rs:48-54). */
static qm31 from_partial_evals(const qm31 e[4]) {
    qm31 r = e[0];
    r = qm31_add(r, qm31_mul(e[1], qm31_make(0, 1, 0, 0)));
    r = qm31_add(r, qm31_mul(e[2], qm31_make(0, 0, 1, 0)));
    r = qm31_add(r, qm31_mul(e[3], qm31_make(0, 0, 0, 1)));
    return r;
}

/* coset_vanishing at a QM31 point (crates/stwo/src/core/constraints.rs:12-34). */
static qm31 coset_vanishing_at(coset_t c, qpoint p) {
    p = qpoint_add_m31(p, cpoint_conj(c.initial));
    p = qpoint_add_m31(p, cidx_to_point(c.step_size >> 1));
    qm31 x = p.x;
    for (uint32_t i = 1; i < c.log_size; i++) x = qcircle_double_x(x);
    return x;
}

/* ------------------------------------------------------------------ channel */

static qm31 draw_felt(orc_channel *ch) {
    uint32_t w[4];
    orc_channel_draw_secure_felt(ch, w);
    return qm31_from_words(w);
}
static void mix_qm31s(orc_channel *ch, const qm31 *v, uint32_t n) {
    uint32_t *w = (uint32_t *)malloc(sizeof(uint32_t) * 4 * (n ? n : 1));
    for (uint32_t i = 0; i < n; i++) qm31_to_words(v[i], w + 4 * i);
    orc_channel_mix_felts(ch, w, n);
    free(w);
}

/* ------------------------------------------------------------------ twiddles */

typedef struct {
    uint32_t *tw, *itw;
    uint32_t log; /* buffer of 2^log words */
} twiddles_t;

/* precompute_twiddles(CanonicCoset(domain_log).circle_domain().half_coset)
   (as crates/examples/src/wide_fibonacci/mod.rs:193-197 builds them). */
static twiddles_t twiddles_for(uint32_t domain_log) {
    twiddles_t t;
    t.log = domain_log - 1;
    t.tw = (uint32_t *)malloc(sizeof(uint32_t) << t.log);
    t.itw = (uint32_t *)malloc(sizeof(uint32_t) << t.log);
    orc_precompute_twiddles(cidx_subgroup_gen(domain_log + 1), t.log, t.tw, t.itw);
    return t;
}

/* TwiddleBuffer::extract_subdomain_twiddles (crates/stwo/src/prover/poly/twiddles.rs:40-76): in
   bit-reversed order a subdomain is a prefix, so each layer's first entries are kept. */
static uint32_t *extract_subdomain_twiddles(const uint32_t *buf, uint32_t buf_log, uint32_t domain_log,
                                            uint32_t sub_log) {
    uint32_t dh = domain_log - 1, sh = sub_log - 1;
    uint32_t skip = buf_log - dh;
    uint64_t bsz = 1ull << buf_log;
    uint32_t *out = (uint32_t *)malloc(sizeof(uint32_t) << sh);
    uint64_t o = 0;
    for (uint32_t layer = 0; layer < sh; layer++) {
        uint64_t start = bsz - (bsz >> (skip + layer));
        uint64_t sz = 1ull << (sh - 1 - layer);
        memcpy(out + o, buf + start, sizeof(uint32_t) * sz);
        o += sz;
    }
    out[o] = buf[bsz - 1];
    return out;
}

/* ------------------------------------------------------------------ commitment trees */

typedef struct {
    uint32_t n;            /* columns, in commit order */
    uint32_t *coeff_log;   /* log size of each polynomial */
    uint32_t **coeffs;     /* coefficients (kept: eval_at_point and ExtendToEvalDomain use them) */
    uint32_t *eval_log;    /* coeff_log + log_blowup_factor */
    uint32_t **evals;      /* evaluations on CanonicCoset(eval_log), bit-reversed */
    uint32_t height;       /* the tree's lifting log size */
    uint8_t *layers;       /* 2^(height+1) - 1 digests: leaves first, root last */
    uint8_t root[32];
} tree_t;

static uint64_t layer_offset(uint32_t height, uint32_t k) {
    /* digests before the layer of 2^k nodes: layers height, height-1, ..., k+1 */
    uint64_t off = 0;
    for (uint32_t j = height; j > k; j--) off += 1ull << j;
    return off;
}

/* CommitmentTreeProver::new (crates/stwo/src/prover/pcs/mod.rs:354-383) from coefficients:
   evaluate each polynomial on its blown-up canonic domain, then MerkleProverLifted::commit at
   the tree's lifting log size. The tree takes ownership of coeffs. */
static void tree_commit_coeffs(tree_t *t, uint32_t n, uint32_t **coeffs, const uint32_t *coeff_log,
                               uint32_t log_blowup, uint32_t lifting, const twiddles_t *tw) {
    memset(t, 0, sizeof(*t));
    t->n = n;
    t->coeffs = coeffs;
    t->coeff_log = (uint32_t *)malloc(sizeof(uint32_t) * (n ? n : 1));
    t->eval_log = (uint32_t *)malloc(sizeof(uint32_t) * (n ? n : 1));
    t->evals = (uint32_t **)malloc(sizeof(uint32_t *) * (n ? n : 1));
    for (uint32_t i = 0; i < n; i++) {
        t->coeff_log[i] = coeff_log[i];
        t->eval_log[i] = coeff_log[i] + log_blowup;
        t->evals[i] = (uint32_t *)malloc(sizeof(uint32_t) << t->eval_log[i]);
    }
    if (n) orc_evaluate_batch((const uint32_t **)t->coeffs, t->coeff_log, t->evals, t->eval_log, n, tw->tw, tw->log);
    t->height = n ? lifting : 0;
    t->layers = (uint8_t *)malloc(32 * ((2ull << t->height) - 1));
    orc_merkle_commit((const uint32_t **)t->evals, t->eval_log, n, t->height, t->root, t->layers);
}

/* TreeBuilder::extend_evals + commit (pcs/mod.rs:324-346): interpolate the trace-domain
   evaluations (copies), then commit. */
static void tree_commit_evals(tree_t *t, uint32_t n, const uint32_t *const *evals, const uint32_t *log,
                              uint32_t log_blowup, uint32_t lifting, const twiddles_t *tw) {
    uint32_t **coeffs = (uint32_t **)malloc(sizeof(uint32_t *) * (n ? n : 1));
    for (uint32_t i = 0; i < n; i++) {
        coeffs[i] = (uint32_t *)malloc(sizeof(uint32_t) << log[i]);
        memcpy(coeffs[i], evals[i], sizeof(uint32_t) << log[i]);
    }
    if (n) orc_interpolate_batch(coeffs, log, n, tw->itw, tw->log);
    tree_commit_coeffs(t, n, coeffs, log, log_blowup, lifting, tw);
}

static void tree_free(tree_t *t) {
    for (uint32_t i = 0; i < t->n; i++) { free(t->coeffs[i]); free(t->evals[i]); }
    free(t->coeffs); free(t->evals); free(t->coeff_log); free(t->eval_log); free(t->layers);
    memset(t, 0, sizeof(*t));
}

/* MerkleProverLifted::decommit's hash witness (crates/stwo/src/prover/vcs_lifted/prover.rs:97-157)
   for sorted, deduplicated positions into the leaf layer. Appends the witness digests to out
   (32 bytes each) and returns their number. */
static uint32_t merkle_witness(const uint8_t *layers, uint32_t height, const uint32_t *positions, uint32_t n_pos,
                               uint8_t **out, uint32_t *out_n) {
    uint32_t *prev = (uint32_t *)malloc(sizeof(uint32_t) * (n_pos ? n_pos : 1));
    uint32_t *cur = (uint32_t *)malloc(sizeof(uint32_t) * (n_pos ? n_pos : 1));
    memcpy(prev, positions, sizeof(uint32_t) * n_pos);
    uint32_t n_prev = n_pos, added = 0;
    for (int32_t layer = (int32_t)height - 1; layer >= 0; layer--) {
        const uint8_t *prev_hashes = layers + 32 * layer_offset(height, (uint32_t)layer + 1);
        uint32_t n_cur = 0;
        for (uint32_t i = 0; i < n_prev;) {
            uint32_t first = prev[i];
            uint32_t len = (i + 1 < n_prev && (first ^ 1u) == prev[i + 1]) ? 2 : 1;
            if (len == 1) {
                *out = (uint8_t *)realloc(*out, 32 * ((size_t)*out_n + 1));
                memcpy(*out + 32 * (size_t)*out_n, prev_hashes + 32 * (size_t)(first ^ 1u), 32);
                (*out_n)++;
                added++;
            }
            cur[n_cur++] = first >> 1;
            i += len;
        }
        uint32_t *tmp = prev; prev = cur; cur = tmp;
        n_prev = n_cur;
    }
    free(prev); free(cur);
    return added;
}

/* ------------------------------------------------------------------ line polynomial */

/* LineEvaluation::interpolate (crates/stwo/src/prover/line.rs:54-99): bit-reverse the values,
   line_ifft over the domain (ibutterflies by 1/x, doubling the domain each layer), scale by
   1/n. Returns the coefficients in the LinePoly's stored (bit-reversed) order. */
static void line_interpolate(qm31 *v, uint32_t log_n, uint32_t domain_initial_index) {
    uint64_t n = 1ull << log_n;
    for (uint64_t i = 0; i < n; i++) {
        uint64_t j = bit_reverse_index((uint32_t)i, log_n);
        if (j > i) { qm31 t = v[i]; v[i] = v[j]; v[j] = t; }
    }
    coset_t dom = coset_new(domain_initial_index, log_n);
    for (uint32_t lg = log_n; lg >= 1; lg--) {
        uint64_t size = 1ull << lg;
        for (uint64_t c = 0; c < n; c += size) {
            for (uint64_t i = 0; i < size / 2; i++) {
                m31 xinv = m31_inv(coset_at(dom, i).x);
                qm31 a = v[c + i], b = v[c + size / 2 + i];
                v[c + i] = qm31_add(a, b);
                v[c + size / 2 + i] = qm31_mul_m31(qm31_sub(a, b), xinv);
            }
        }
        dom = coset_double(dom);
    }
    m31 inv_n = m31_inv((m31)(n % M31_P));
    for (uint64_t i = 0; i < n; i++) v[i] = qm31_mul_m31(v[i], inv_n);
}

/* ------------------------------------------------------------------ the proof */

typedef struct {
    uint32_t pow_bits, log_blowup_factor, log_last_layer_degree_bound, n_queries, fold_step;
} fri_params_t;

/* per tree: per column, 0, 1 ([oods]) or 2 ([oods - step, oods]) mask samples */
typedef struct {
    uint32_t n_trees;
    tree_t *trees;        /* trees[0] is the preprocessed tree */
    uint8_t **n_samples;  /* [tree][column] */
} scheme_t;

static qm31 soa_get(uint32_t *const c[4], uint64_t i) { return qm31_make(c[0][i], c[1][i], c[2][i], c[3][i]); }
static void soa_put(uint32_t *const c[4], uint64_t i, qm31 v) {
    c[0][i] = v.a.a; c[1][i] = v.a.b; c[2][i] = v.b.a; c[3][i] = v.b.b;
}
static void soa_alloc(uint32_t *c[4], uint32_t log_n) {
    for (int k = 0; k < 4; k++) c[k] = (uint32_t *)calloc(1ull << log_n, sizeof(uint32_t));
}
static void soa_free(uint32_t *c[4]) { for (int k = 0; k < 4; k++) free(c[k]); }

typedef struct {
    qpoint point;
    qm31 value;
    qm31 rand;
    uint32_t tree, col;  /* the flattened column this sample belongs to */
    uint32_t eval_log;
} sample_t;

typedef struct {
    qpoint point;
    uint32_t log;        /* log size of partial (column eval log - log_blowup) */
    uint32_t *partial[4];
    qm31 first_linear;
} acc_num_t;

static int acc_cmp_idx(const acc_num_t *a, uint32_t ia, const acc_num_t *b, uint32_t ib) {
    int c = qpoint_cmp(a->point, b->point);
    if (c) return c;
    return ia < ib ? -1 : ia > ib;  /* stable */
}

/* compute_fri_quotients (crates/stwo/src/prover/pcs/quotient_ops.rs:86-160) with
   build_samples_with_randomness_and_periodicity (crates/stwo/src/core/pcs/quotients.rs:274-319)
   and ColumnSampleBatch::new_vec (:77-96); returns the quotient evaluation on CanonicCoset(L). */
static void fri_quotients(const scheme_t *s, qm31 **sampled, const qpoint *const *points, qm31 random_coeff,
                          uint32_t L, uint32_t b, const twiddles_t *tw, uint32_t *out[4]) {
    /* samples with randomness: per column (tree order), the periodicity sample first for columns
       with two samples, then the samples in order; powers 1, r, r^2, ... in that order */
    uint32_t total = 0;
    for (uint32_t t = 0; t < s->n_trees; t++)
        for (uint32_t c = 0; c < s->trees[t].n; c++) total += s->n_samples[t][c] == 2 ? 3 : s->n_samples[t][c];
    sample_t *smp = (sample_t *)malloc(sizeof(sample_t) * (total ? total : 1));
    uint32_t ns = 0;
    qm31 pw = qm31_from_m31(1);
    cpoint lift_step = cidx_to_point(cidx_subgroup_gen(L));  /* CanonicCoset(L).step() */
    for (uint32_t t = 0; t < s->n_trees; t++) {
        for (uint32_t c = 0; c < s->trees[t].n; c++) {
            uint32_t k = s->n_samples[t][c];
            uint32_t el = s->trees[t].eval_log[c];
            if (k == 2) {
                /* period generator: lifting step doubled log_size times */
                cpoint g = lift_step;
                for (uint32_t d = 0; d < el; d++) g = cpoint_double(g);
                sample_t x = {qpoint_add_m31(points[t][2 * c + 1], g), sampled[t][2 * c + 1], pw, t, c, el};
                smp[ns++] = x;
                pw = qm31_mul(pw, random_coeff);
            }
            for (uint32_t j = 0; j < k; j++) {
                sample_t x = {points[t][2 * c + j], sampled[t][2 * c + j], pw, t, c, el};
                smp[ns++] = x;
                pw = qm31_mul(pw, random_coeff);
            }
        }
    }
    /* columns (with at least one sample) grouped by eval log size, stably, ascending */
    uint32_t max_el = 0;
    for (uint32_t i = 0; i < ns; i++) if (smp[i].eval_log > max_el) max_el = smp[i].eval_log;
    acc_num_t *accs = (acc_num_t *)malloc(sizeof(acc_num_t) * (ns ? ns : 1));
    uint32_t n_acc = 0;
    uint32_t *in_group = (uint32_t *)malloc(sizeof(uint32_t) * (ns ? ns : 1));
    uint8_t *used = (uint8_t *)calloc(ns ? ns : 1, 1);
    for (uint32_t el = 0; el <= max_el; el++) {
        /* the samples of this size's columns in column order (samples of one column are adjacent) */
        uint32_t ng = 0;
        for (uint32_t i = 0; i < ns; i++) if (smp[i].eval_log == el) in_group[ng++] = i;
        if (!ng) continue;
        memset(used, 0, ns);
        /* batches by point, in order of first appearance */
        for (uint32_t a = 0; a < ng; a++) {
            if (used[a]) continue;
            qpoint pt = smp[in_group[a]].point;
            uint32_t n_terms = 0;
            for (uint32_t j = a; j < ng; j++) if (!used[j] && qpoint_eq(smp[in_group[j]].point, pt)) n_terms++;
            const uint32_t **cols = (const uint32_t **)malloc(sizeof(void *) * n_terms);
            uint32_t *coeffs = (uint32_t *)malloc(sizeof(uint32_t) * 12 * n_terms);
            uint32_t q = 0;
            for (uint32_t j = a; j < ng; j++) {
                const sample_t *x = &smp[in_group[j]];
                if (used[j] || !qpoint_eq(x->point, pt)) continue;
                used[j] = 1;
                cols[q] = s->trees[x->tree].evals[x->col];
                uint32_t py[4], val[4], rnd[4];
                qm31_to_words(pt.y, py); qm31_to_words(x->value, val); qm31_to_words(x->rand, rnd);
                /* complex_conjugate_line_coeffs (crates/stwo/src/core/constraints.rs:119-135) */
                orc_line_coeffs(py, val, rnd, coeffs + 12 * q);
                q++;
            }
            acc_num_t *A = &accs[n_acc++];
            A->point = pt;
            A->log = el - b;
            soa_alloc(A->partial, A->log);
            uint32_t fl[4];
            orc_accumulate_numerators(cols, n_terms, el, b, coeffs, A->partial, fl);
            A->first_linear = qm31_from_words(fl);
            free(cols); free(coeffs);
        }
    }
    free(in_group); free(used); free(smp);
    /* stable sort of the accumulations by sample point; one lifted accumulation per point */
    uint32_t *order = (uint32_t *)malloc(sizeof(uint32_t) * (n_acc ? n_acc : 1));
    for (uint32_t i = 0; i < n_acc; i++) order[i] = i;
    for (uint32_t i = 1; i < n_acc; i++) {  /* insertion sort (few entries) */
        uint32_t k = order[i];
        int64_t j = (int64_t)i - 1;
        while (j >= 0 && acc_cmp_idx(&accs[order[j]], order[j], &accs[k], k) > 0) { order[j + 1] = order[j]; j--; }
        order[j + 1] = k;
    }
    uint32_t n_pts = 0;
    const uint32_t **pt_accs = (const uint32_t **)malloc(sizeof(void *) * 4 * (n_acc ? n_acc : 1));
    uint32_t *pt_logs = (uint32_t *)malloc(sizeof(uint32_t) * (n_acc ? n_acc : 1));
    uint32_t *pt_words = (uint32_t *)malloc(sizeof(uint32_t) * 8 * (n_acc ? n_acc : 1));
    uint32_t *pt_fl = (uint32_t *)malloc(sizeof(uint32_t) * 4 * (n_acc ? n_acc : 1));
    for (uint32_t i = 0; i < n_acc;) {
        uint32_t j = i;
        while (j < n_acc && qpoint_eq(accs[order[j]].point, accs[order[i]].point)) j++;
        /* lift_and_accumulate over the group (ascending sizes) */
        uint32_t m = j - i;
        uint32_t **cols = (uint32_t **)malloc(sizeof(void *) * 4 * m);
        uint32_t *logs = (uint32_t *)malloc(sizeof(uint32_t) * m);
        qm31 fl = qm31_from_m31(0);
        for (uint32_t k = 0; k < m; k++) {
            acc_num_t *A = &accs[order[i + k]];
            for (int c = 0; c < 4; c++) cols[4 * k + c] = A->partial[c];
            logs[k] = A->log;
            fl = qm31_add(fl, A->first_linear);
        }
        orc_lift_and_accumulate(cols, logs, m);
        for (int c = 0; c < 4; c++) pt_accs[4 * n_pts + c] = cols[4 * (m - 1) + c];
        pt_logs[n_pts] = logs[m - 1];
        qm31_to_words(accs[order[i]].point.x, pt_words + 8 * n_pts);
        qm31_to_words(accs[order[i]].point.y, pt_words + 8 * n_pts + 4);
        qm31_to_words(fl, pt_fl + 4 * n_pts);
        n_pts++;
        free(cols); free(logs);
        i = j;
    }
    /* compute_quotients_and_combine: quotient on the subdomain of log L - b, interpolated there
       and evaluated on CanonicCoset(L) */
    uint32_t sub = L - b;
    uint32_t *q[4];
    soa_alloc(q, sub);
    orc_quotients_on_subdomain(pt_accs, pt_logs, n_pts, pt_words, pt_fl, L, b, q);
    uint32_t *sub_itw = extract_subdomain_twiddles(tw->itw, tw->log, L, sub);
    for (int c = 0; c < 4; c++) {
        /* the subdomain's half coset starts where CanonicCoset(L)'s does */
        orc_interpolate_on(q[c], sub, sub_itw, sub - 1, cidx_subgroup_gen(L + 1));
        orc_evaluate(q[c], sub, out[c], L, tw->tw, tw->log);
    }
    free(sub_itw);
    soa_free(q);
    for (uint32_t i = 0; i < n_acc; i++) soa_free(accs[i].partial);
    free(accs); free(order); free(pt_accs); free(pt_logs); free(pt_words); free(pt_fl);
}

/* One committed FRI layer (FriFirstLayerProver / FriInnerLayerProver, crates/stwo/src/prover/fri.rs:
   287-392): the 4 coordinate columns, the layer's fold step and its tree. With a fold step above
   one and at least 4 values, a leaf holds 4 consecutive values (pack_leaves_input: column
   coord + 4 offset holds coordinate coord of row 4 r + offset, the tree 2 levels lower). */
typedef struct {
    uint32_t log, step, packed, height;
    uint32_t *v[4];
    uint8_t *layers;
    uint8_t root[32];
} fri_layer_t;

static void fri_layer_commit(fri_layer_t *f, uint32_t *v[4], uint32_t log, uint32_t step) {
    f->log = log;
    f->step = step;
    f->packed = step > 1 && log >= 2;
    for (int c = 0; c < 4; c++) f->v[c] = v[c];
    if (!f->packed) {
        uint32_t logs[4] = {log, log, log, log};
        f->height = log;
        f->layers = (uint8_t *)malloc(32 * ((2ull << log) - 1));
        orc_merkle_commit((const uint32_t **)f->v, logs, 4, log, f->root, f->layers);
        return;
    }
    const uint32_t h = log - 2;
    const uint64_t rows = 1ull << h;
    uint32_t *pk[16];
    uint32_t logs[16];
    for (int c = 0; c < 16; c++) {
        pk[c] = (uint32_t *)malloc(sizeof(uint32_t) * rows);
        logs[c] = h;
    }
    for (uint64_t r = 0; r < rows; r++)
        for (int off = 0; off < 4; off++)
            for (int coord = 0; coord < 4; coord++) pk[coord + 4 * off][r] = v[coord][4 * r + off];
    f->height = h;
    f->layers = (uint8_t *)malloc(32 * ((2ull << h) - 1));
    orc_merkle_commit((const uint32_t **)pk, logs, 16, h, f->root, f->layers);
    for (int c = 0; c < 16; c++) free(pk[c]);
}

/* compute_decommitment_positions_and_witness_evals (fri.rs:398-430): every coset of 2^step
   positions around the queries, the values that are not queries as the witness, then the layer's
   Merkle witness of those positions (of the leaves holding them when packed, fri.rs:318-326);
   serialized as FriLayerProof (serialize.rs:69-79). */
static void fri_layer_decommit(const fri_layer_t *f, const uint32_t *queries, uint32_t nq, felts_t *out) {
    const uint32_t k = f->step, m = 1u << k;
    uint32_t *pos = (uint32_t *)calloc((size_t)m * (nq ? nq : 1), sizeof(uint32_t));
    qm31 *wit = (qm31 *)malloc(sizeof(qm31) * (size_t)m * (nq ? nq : 1));
    uint32_t npos = 0, nw = 0;
    for (uint32_t i = 0; i < nq;) {
        uint32_t j = i;
        while (j < nq && (queries[j] >> k) == (queries[i] >> k)) j++;
        uint32_t start = (queries[i] >> k) << k;
        uint32_t qi = i;
        for (uint32_t p = start; p < start + m; p++) {
            pos[npos++] = p;
            if (qi < j && queries[qi] == p) qi++;
            else wit[nw++] = soa_get((uint32_t *const *)f->v, p);
        }
        i = j;
    }
    uint32_t nmp = npos;
    if (f->packed) {  /* the leaves holding the positions, each once (positions are sorted) */
        nmp = 0;
        for (uint32_t i = 0; i < npos; i++)
            if (nmp == 0 || pos[nmp - 1] != (pos[i] >> 2)) pos[nmp++] = pos[i] >> 2;
    }
    uint8_t *hw = NULL;
    uint32_t nhw = 0;
    merkle_witness(f->layers, f->height, pos, nmp, &hw, &nhw);
    fpush(out, nw);
    for (uint32_t q = 0; q < nw; q++) fpush_qm31(out, wit[q]);
    fpush(out, nhw);
    for (uint32_t q = 0; q < nhw; q++) fpush_hash(out, hw + 32 * q);
    fpush_hash(out, f->root);
    free(hw); free(pos); free(wit);
}

/* Queries::fold (crates/stwo/src/core/queries.rs:50-56) in place; returns the new count. */
static uint32_t fold_queries_inplace(uint32_t *q, uint32_t n, uint32_t k) {
    uint32_t m = 0;
    for (uint32_t i = 0; i < n; i++) {
        uint32_t v = q[i] >> k;
        if (m == 0 || q[m - 1] != v) q[m++] = v;
    }
    return m;
}

/* The part of prove_ex after the composition tree is committed (crates/stwo/src/prover/mod.rs:75-135)
   with CommitmentSchemeProver::prove_values (pcs/mod.rs:224-315) and FriProver::commit /
   decommit (fri.rs:113-284). Appends the CairoSerialize felt stream of the StarkProof
   (serialize.rs:121-153) to out. oods / sampled / points are returned for the caller's check. */
static int prove_tail(scheme_t *s, orc_channel *ch, const fri_params_t *fp, uint32_t L, const twiddles_t *tw,
                      felts_t *out, qpoint *oods_out, qm31 ***sampled_out, uint64_t *oods_pow_out) {
    const uint32_t b = fp->log_blowup_factor;
    /* proof of work before the OODS point (mod.rs:75-80), OODS_POW_BITS = 16 */
    uint64_t oods_pow = orc_grind(ch->digest, 16);
    orc_channel_mix_u64(ch, oods_pow);
    /* CirclePoint::get_random_point (crates/stwo/src/core/circle.rs:150-160) */
    uint32_t t[4], px[4], py[4];
    orc_channel_draw_secure_felt(ch, t);
    orc_random_point_from_t(t, px, py);
    qpoint oods = {qm31_from_words(px), qm31_from_words(py)};
    const uint32_t mldb = L - b;
    /* mask points (crates/constraint-framework/src/component.rs:202-213): offset -1 is one step of
       CanonicCoset(max_log_degree_bound) back */
    cpoint step = cidx_to_point(cidx_subgroup_gen(mldb));
    qpoint prev_pt = qpoint_add_m31(oods, cpoint_conj(step));
    qpoint **points = (qpoint **)malloc(sizeof(void *) * s->n_trees);
    qm31 **sampled = (qm31 **)malloc(sizeof(void *) * s->n_trees);
    for (uint32_t tr = 0; tr < s->n_trees; tr++) {
        tree_t *T = &s->trees[tr];
        points[tr] = (qpoint *)malloc(sizeof(qpoint) * 2 * (T->n ? T->n : 1));
        sampled[tr] = (qm31 *)malloc(sizeof(qm31) * 2 * (T->n ? T->n : 1));
        for (uint32_t c = 0; c < T->n; c++) {
            if (s->n_samples[tr][c] == 2) { points[tr][2 * c] = prev_pt; points[tr][2 * c + 1] = oods; }
            else points[tr][2 * c] = oods;
        }
        /* compute_samples (pcs/mod.rs:174-222): each column at the point doubled down to its size */
#pragma omp parallel for schedule(dynamic, 1)
        for (int64_t c = 0; c < (int64_t)T->n; c++) {
            for (uint32_t j = 0; j < s->n_samples[tr][c]; j++) {
                qpoint p = qpoint_repeated_double(points[tr][2 * c + j], L - T->eval_log[c]);
                uint32_t x[4], y[4], v[4];
                qm31_to_words(p.x, x); qm31_to_words(p.y, y);
                orc_eval_at_point(T->coeffs[c], T->coeff_log[c], x, y, v);
                sampled[tr][2 * c + j] = qm31_from_words(v);
            }
        }
    }
    /* mix every sampled value, tree by tree, column by column (pcs/mod.rs:236-239) */
    {
        uint32_t n = 0;
        for (uint32_t tr = 0; tr < s->n_trees; tr++)
            for (uint32_t c = 0; c < s->trees[tr].n; c++) n += s->n_samples[tr][c];
        qm31 *all = (qm31 *)malloc(sizeof(qm31) * (n ? n : 1));
        n = 0;
        for (uint32_t tr = 0; tr < s->n_trees; tr++)
            for (uint32_t c = 0; c < s->trees[tr].n; c++)
                for (uint32_t j = 0; j < s->n_samples[tr][c]; j++) all[n++] = sampled[tr][2 * c + j];
        mix_qm31s(ch, all, n);
        free(all);
    }
    qm31 random_coeff = draw_felt(ch);
    uint32_t *quot[4];
    soa_alloc(quot, L);
    fri_quotients(s, sampled, (const qpoint *const *)points, random_coeff, L, b, tw, quot);

    /* FRI commitment (fri.rs:113-242): the first layer folds circle -> line then fold_step - 1 line
       folds with alpha^2, alpha^4, ...; each inner layer folds fold_step times (alpha, alpha^2,
       ...), the last one the 1..fold_step folds left */
    const uint32_t k = fp->fold_step;
    const uint32_t last_log = fp->log_last_layer_degree_bound + b;
    fri_layer_t first;
    fri_layer_commit(&first, quot, L, k);
    orc_channel_mix_root(ch, first.root);
    uint32_t n_inner_cap = L + 1, n_inner = 0;
    fri_layer_t *inner = (fri_layer_t *)malloc(sizeof(fri_layer_t) * n_inner_cap);
    qm31 alpha = draw_felt(ch);
    uint32_t *cur[4];
    soa_alloc(cur, L - 1);
    {
        uint32_t a[4];
        qm31_to_words(alpha, a);
        orc_fold_circle_into_line((const uint32_t *const *)first.v, L, a, cur);
    }
    uint32_t line_log = L - 1;
    uint32_t dom_index = cidx_subgroup_gen(line_log + 2);  /* LineDomain(Coset::half_odds(L - 1)) */
    /* fold `steps` times with a, a^2, a^4, ...; the folded columns replace cur */
    #define FOLD_STEPS(a_start, steps)                                                         \
        do {                                                                                   \
            qm31 fa = (a_start);                                                               \
            for (uint32_t st = 0; st < (steps); st++) {                                        \
                uint32_t aw[4], *nxt[4];                                                       \
                qm31_to_words(fa, aw);                                                         \
                soa_alloc(nxt, line_log - 1);                                                  \
                orc_fold_line((const uint32_t *const *)cur, dom_index, line_log, aw, nxt);     \
                if (st > 0 || !keep_cur) soa_free(cur);                                        \
                for (int cc = 0; cc < 4; cc++) cur[cc] = nxt[cc];                              \
                dom_index = (uint32_t)(((uint64_t)dom_index * 2) & CIRCLE_INDEX_MASK);         \
                line_log--;                                                                    \
                fa = qm31_mul(fa, fa);                                                         \
            }                                                                                  \
        } while (0)
    int keep_cur = 0;
    if (k > 1) FOLD_STEPS(qm31_mul(alpha, alpha), k - 1);
    if (line_log > last_log) {
        while (line_log > last_log + k) {
            fri_layer_t *lay = &inner[n_inner++];
            fri_layer_commit(lay, cur, line_log, k);
            orc_channel_mix_root(ch, lay->root);
            alpha = draw_felt(ch);
            keep_cur = 1;  /* the layer keeps its columns for the decommitment */
            FOLD_STEPS(alpha, k);
        }
        const uint32_t last_step = line_log - last_log;
        fri_layer_t *lay = &inner[n_inner++];
        fri_layer_commit(lay, cur, line_log, last_step);
        orc_channel_mix_root(ch, lay->root);
        alpha = draw_felt(ch);
        keep_cur = 1;
        FOLD_STEPS(alpha, last_step);
    }
    #undef FOLD_STEPS
    /* last layer (fri.rs:212-241): interpolate, the top coefficients must vanish */
    uint64_t n_last = 1ull << line_log;
    qm31 *lv = (qm31 *)malloc(sizeof(qm31) * n_last);
    for (uint64_t i = 0; i < n_last; i++) lv[i] = soa_get(cur, i);
    soa_free(cur);
    line_interpolate(lv, line_log, dom_index);
    uint64_t keep = 1ull << fp->log_last_layer_degree_bound;
    /* ordered coefficient k is stored at bit_reverse(k); the ordered tail must be zero */
    for (uint64_t k = keep; k < n_last; k++)
        if (!qm31_is_zero(lv[bit_reverse_index((uint32_t)k, line_log)])) {
            free(lv);
            return 2;  /* invalid degree */
        }
    uint32_t keep_log = fp->log_last_layer_degree_bound;
    qm31 *last_poly = (qm31 *)malloc(sizeof(qm31) * keep);
    for (uint64_t k = 0; k < keep; k++) {
        /* LinePoly::from_ordered_coefficients: stored in bit-reversed order of the kept length */
        uint64_t ordered = bit_reverse_index((uint32_t)k, keep_log);
        last_poly[k] = lv[bit_reverse_index((uint32_t)ordered, line_log)];
    }
    free(lv);
    mix_qm31s(ch, last_poly, (uint32_t)keep);

    /* FRI decommitment (fri.rs:244-284) */
    uint64_t fri_pow = orc_grind(ch->digest, fp->pow_bits);
    orc_channel_mix_u64(ch, fri_pow);
    uint32_t *queries = (uint32_t *)malloc(sizeof(uint32_t) * fp->n_queries);
    orc_channel_draw_queries(ch, L, fp->n_queries, queries);
    uint32_t nq = sort_dedup(queries, fp->n_queries);

    /* ---- the felt stream (serialize.rs:121-153) */
    fpush(out, fp->pow_bits); fpush(out, b); fpush(out, fp->log_last_layer_degree_bound);
    fpush(out, fp->n_queries); fpush(out, fp->fold_step);
    fpush(out, s->n_trees);
    for (uint32_t tr = 0; tr < s->n_trees; tr++) fpush_hash(out, s->trees[tr].root);
    fpush(out, oods_pow);
    fpush(out, s->n_trees);
    for (uint32_t tr = 0; tr < s->n_trees; tr++) {
        fpush(out, s->trees[tr].n);
        for (uint32_t c = 0; c < s->trees[tr].n; c++) {
            fpush(out, s->n_samples[tr][c]);
            for (uint32_t j = 0; j < s->n_samples[tr][c]; j++) fpush_qm31(out, sampled[tr][2 * c + j]);
        }
    }
    /* decommitments: the preprocessed tree answers no queries (prepare_preprocessed_query_positions
       of an empty tree, crates/stwo/src/core/pcs/utils.rs:185-192) */
    fpush(out, s->n_trees);
    for (uint32_t tr = 0; tr < s->n_trees; tr++) {
        tree_t *T = &s->trees[tr];
        uint8_t *hw = NULL;
        uint32_t nhw = 0;
        if (tr > 0) merkle_witness(T->layers, T->height, queries, nq, &hw, &nhw);
        fpush(out, nhw);
        for (uint32_t k = 0; k < nhw; k++) fpush_hash(out, hw + 32 * k);
        free(hw);
    }
    fpush(out, s->n_trees);
    for (uint32_t tr = 0; tr < s->n_trees; tr++) {
        tree_t *T = &s->trees[tr];
        fpush(out, T->n);
        for (uint32_t c = 0; c < T->n; c++) {
            uint32_t qn = tr > 0 ? nq : 0;
            fpush(out, qn);
            uint32_t shift = T->height - T->eval_log[c];
            for (uint32_t k = 0; k < qn; k++) {
                uint32_t p = queries[k];
                fpush(out, T->evals[c][((p >> (shift + 1)) << 1) + (p & 1)]);
            }
        }
    }
    /* FriProof: first layer, inner layers on folded queries, last-layer poly, proof of work */
    fri_layer_decommit(&first, queries, nq, out);
    fpush(out, n_inner);
    uint32_t *lq = (uint32_t *)malloc(sizeof(uint32_t) * (nq ? nq : 1));
    for (uint32_t q = 0; q < nq; q++) lq[q] = queries[q];
    uint32_t nlq = fold_queries_inplace(lq, nq, k);
    for (uint32_t i = 0; i < n_inner; i++) {
        fri_layer_decommit(&inner[i], lq, nlq, out);
        nlq = fold_queries_inplace(lq, nlq, inner[i].step);
    }
    fpush(out, keep);
    for (uint64_t k = 0; k < keep; k++) fpush_qm31(out, last_poly[k]);
    fpush(out, keep_log);
    fpush(out, fri_pow);

    for (uint32_t i = 0; i < n_inner; i++) { soa_free(inner[i].v); free(inner[i].layers); }
    soa_free(first.v); free(first.layers);
    free(inner); free(lq); free(queries); free(last_poly);
    *oods_out = oods;
    *sampled_out = sampled;
    *oods_pow_out = oods_pow;
    for (uint32_t tr = 0; tr < s->n_trees; tr++) free(points[tr]);
    free(points);
    return 0;
}

/* DomainEvaluationAccumulator (crates/stwo/src/prover/air/accumulation.rs:68-180): the
   random coefficient's powers 1, a, ..., a^(N-1); each component takes the last n of the
   remaining powers, reversed (constraint k of the component gets a^(n-1-k) times the shift of
   the components after it). */
typedef struct {
    qm31 *powers;
    uint32_t remaining;
    uint32_t *sub[32][4];  /* sub-accumulations by eval log size */
} accumulator_t;

static void accumulator_init(accumulator_t *A, qm31 random_coeff, uint32_t total) {
    memset(A, 0, sizeof(*A));
    A->powers = (qm31 *)malloc(sizeof(qm31) * (total ? total : 1));
    qm31 p = qm31_from_m31(1);
    for (uint32_t i = 0; i < total; i++) { A->powers[i] = p; p = qm31_mul(p, random_coeff); }
    A->remaining = total;
}
/* the rc table (4 words per constraint) of the next component's n constraints */
static uint32_t *accumulator_take(accumulator_t *A, uint32_t n) {
    uint32_t *rc = (uint32_t *)malloc(sizeof(uint32_t) * 4 * (n ? n : 1));
    for (uint32_t k = 0; k < n; k++) qm31_to_words(A->powers[A->remaining - 1 - k], rc + 4 * k);
    A->remaining -= n;
    return rc;
}
static uint32_t *const *accumulator_col(accumulator_t *A, uint32_t log) {
    if (!A->sub[log][0]) soa_alloc(A->sub[log], log);
    return A->sub[log];
}
/* finalize (accumulation.rs:126-178): lift and accumulate the sub-accumulations (ascending
   sizes), interpolate on CanonicCoset(log) of the largest (SubDomain with log_expansion 0 and
   ExtendToEvalDomain both use the canonic domain). Returns the 4 coordinate coefficient arrays
   and the composition log size. */
static uint32_t accumulator_finalize(accumulator_t *A, const twiddles_t *tw, uint32_t *coeffs[4]) {
    uint32_t **cols = (uint32_t **)malloc(sizeof(void *) * 4 * 32);
    uint32_t logs[32], m = 0;
    for (uint32_t l = 0; l < 32; l++) {
        if (!A->sub[l][0]) continue;
        for (int c = 0; c < 4; c++) cols[4 * m + c] = A->sub[l][c];
        logs[m++] = l;
    }
    orc_lift_and_accumulate(cols, logs, m);
    uint32_t log = logs[m - 1];
    for (int c = 0; c < 4; c++) {
        coeffs[c] = A->sub[log][c];
        A->sub[log][c] = NULL;
        orc_interpolate(coeffs[c], log, tw->itw, tw->log);
    }
    for (uint32_t l = 0; l < 32; l++) if (A->sub[l][0]) soa_free(A->sub[l]);
    free(cols); free(A->powers);
    return log;
}

/* prove_ex's composition commit (mod.rs:50-71): split_at_mid of each coordinate polynomial, the
   four left halves then the four right halves, committed as one tree. */
static void commit_composition(tree_t *t, uint32_t *coeffs[4], uint32_t log, uint32_t b, uint32_t L,
                               const twiddles_t *tw) {
    uint32_t **halves = (uint32_t **)malloc(sizeof(void *) * 8);
    uint32_t logs[8];
    uint64_t h = 1ull << (log - 1);
    for (int side = 0; side < 2; side++)
        for (int c = 0; c < 4; c++) {
            uint32_t *p = (uint32_t *)malloc(sizeof(uint32_t) * h);
            memcpy(p, coeffs[c] + side * h, sizeof(uint32_t) * h);
            halves[4 * side + c] = p;
            logs[4 * side + c] = log - 1;
        }
    soa_free(coeffs);
    tree_commit_coeffs(t, 8, halves, logs, b, L, tw);
}

static void scheme_free(scheme_t *s) {
    for (uint32_t t = 0; t < s->n_trees; t++) { tree_free(&s->trees[t]); free(s->n_samples[t]); }
    free(s->trees); free(s->n_samples);
}

static int finish_words(felts_t *f, uint64_t *words, size_t capacity, size_t *n_words) {
    *n_words = f->n;
    int rc = 0;
    if (words) {
        if (capacity < f->n) rc = -2;
        else memcpy(words, f->w, sizeof(uint64_t) * f->n);
    }
    free(f->w);
    return rc;
}

/* ------------------------------------------------------------ Wide-Fibonacci + LogUp */

int orc_prove_fib_and_lookups(const uint32_t fri[5], uint32_t n_fib, const uint32_t *fib_n_cols,
                              const uint32_t *fib_log_sizes, const uint32_t *const *fib_trace,
                              uint32_t n_lookups, const uint32_t *lookup_log_sizes,
                              const uint32_t *const *lookup_values, int check, uint32_t *claimed_out,
                              uint64_t *words, size_t capacity, size_t *n_words) {
    fri_params_t fp = {fri[0], fri[1], fri[2], fri[3], fri[4]};
    if (fp.log_blowup_factor != 1 || fp.fold_step < 1 || n_fib + n_lookups == 0) return -1;
    const uint32_t b = fp.log_blowup_factor;
    uint32_t max_log = 0, n_fib_cols = 0;
    for (uint32_t k = 0; k < n_fib; k++) {
        if (fib_n_cols[k] < 3) return -1;
        if (fib_log_sizes[k] > max_log) max_log = fib_log_sizes[k];
        n_fib_cols += fib_n_cols[k];
    }
    for (uint32_t k = 0; k < n_lookups; k++) if (lookup_log_sizes[k] > max_log) max_log = lookup_log_sizes[k];
    /* every tree after the preprocessed one is lifted to trace_lifting_log_size = max + blowup
       (wide_fibonacci/mod.rs:186-191) */
    const uint32_t L = max_log + b;
    twiddles_t tw = twiddles_for(L + 1);
    orc_channel ch;
    memset(&ch, 0, sizeof(ch));
    scheme_t s;
    s.n_trees = n_lookups ? 4 : 3;
    s.trees = (tree_t *)calloc(s.n_trees, sizeof(tree_t));
    s.n_samples = (uint8_t **)calloc(s.n_trees, sizeof(void *));

    /* preprocessed tree: empty, never lifted (pcs/mod.rs:83-98 with lifting_log_size(0) = 0) */
    tree_commit_evals(&s.trees[0], 0, NULL, NULL, b, 0, &tw);
    s.n_samples[0] = (uint8_t *)calloc(1, 1);
    orc_channel_mix_root(&ch, s.trees[0].root);

    /* trace tree: every Wide-Fibonacci column (components in order), then each LogUp
       component's value column */
    uint32_t n_trace = n_fib_cols + n_lookups;
    const uint32_t **tcols = (const uint32_t **)malloc(sizeof(void *) * n_trace);
    uint32_t *tlogs = (uint32_t *)malloc(sizeof(uint32_t) * n_trace);
    uint32_t c = 0;
    for (uint32_t k = 0; k < n_fib; k++)
        for (uint32_t j = 0; j < fib_n_cols[k]; j++) { tcols[c] = fib_trace[c]; tlogs[c] = fib_log_sizes[k]; c++; }
    for (uint32_t k = 0; k < n_lookups; k++) { tcols[c] = lookup_values[k]; tlogs[c] = lookup_log_sizes[k]; c++; }
    tree_commit_evals(&s.trees[1], n_trace, tcols, tlogs, b, L, &tw);
    free(tcols);
    s.n_samples[1] = (uint8_t *)malloc(n_trace);
    memset(s.n_samples[1], 1, n_trace);
    orc_channel_mix_root(&ch, s.trees[1].root);

    /* lookup elements (LookupElements::draw: z then alpha, crates/constraint-framework/src/logup.rs:70-79)
       and the interaction tree of running sums; the claimed sums belong to the statement and are
       mixed before the interaction root */
    qm31 z = qm31_from_m31(0);
    qm31 *claimed = (qm31 *)malloc(sizeof(qm31) * (n_lookups ? n_lookups : 1));
    tree_t *inter = NULL;
    if (n_lookups) {
        z = draw_felt(&ch);
        (void)draw_felt(&ch);  /* alpha: a one-value relation does not use it */
        uint32_t **icols = (uint32_t **)malloc(sizeof(void *) * 4 * n_lookups);
        uint32_t *ilogs = (uint32_t *)malloc(sizeof(uint32_t) * 4 * n_lookups);
        uint32_t zw[4];
        qm31_to_words(z, zw);
#pragma omp parallel for schedule(dynamic, 1)
        for (int64_t k = 0; k < (int64_t)n_lookups; k++) {
            uint32_t *o[4];
            for (int j = 0; j < 4; j++) {
                o[j] = (uint32_t *)malloc(sizeof(uint32_t) << lookup_log_sizes[k]);
                icols[4 * k + j] = o[j];
                ilogs[4 * k + j] = lookup_log_sizes[k];
            }
            uint32_t cw[4];
            orc_logup_running_sum(lookup_values[k], lookup_log_sizes[k], zw, o, cw);
            claimed[k] = qm31_from_words(cw);
        }
        mix_qm31s(&ch, claimed, n_lookups);
        inter = &s.trees[2];
        tree_commit_evals(inter, 4 * n_lookups, (const uint32_t *const *)icols, ilogs, b, L, &tw);
        for (uint32_t k = 0; k < 4 * n_lookups; k++) free(icols[k]);
        free(icols); free(ilogs);
        s.n_samples[2] = (uint8_t *)malloc(4 * n_lookups);
        memset(s.n_samples[2], 2, 4 * n_lookups);  /* the running sum is read at offsets -1 and 0 */
        orc_channel_mix_root(&ch, inter->root);
        if (claimed_out)
            for (uint32_t k = 0; k < n_lookups; k++) qm31_to_words(claimed[k], claimed_out + 4 * k);
    }

    /* composition polynomial (ComponentProvers::compute_composition_polynomial,
       crates/stwo/src/prover/air/component_prover.rs:113-138): components in order, each on its
       committed evaluation (SubDomain, log_expansion 0) */
    qm31 random_coeff = draw_felt(&ch);
    uint32_t total = n_fib_cols - 2 * n_fib + n_lookups;
    accumulator_t A;
    accumulator_init(&A, random_coeff, total);
    const tree_t *T = &s.trees[1];
    c = 0;
    for (uint32_t k = 0; k < n_fib; k++) {
        uint32_t n = fib_n_cols[k], l = fib_log_sizes[k];
        uint32_t *rc = accumulator_take(&A, n - 2);
        orc_wide_fib_composition((const uint32_t **)(T->evals + c), n, l + b, l, rc, accumulator_col(&A, l + b));
        free(rc);
        c += n;
    }
    for (uint32_t k = 0; k < n_lookups; k++) {
        uint32_t l = lookup_log_sizes[k];
        uint32_t *rc = accumulator_take(&A, 1);
        uint32_t zw[4], cw[4];
        qm31_to_words(z, zw);
        qm31_to_words(claimed[k], cw);
        orc_logup_composition(T->evals[n_fib_cols + k], (const uint32_t *const *)(inter->evals + 4 * k), l + b, l, zw,
                              cw, rc, accumulator_col(&A, l + b));
        free(rc);
    }
    uint32_t *comp[4];
    uint32_t comp_log = accumulator_finalize(&A, &tw, comp);
    tree_t *ct = &s.trees[s.n_trees - 1];
    commit_composition(ct, comp, comp_log, b, L, &tw);
    s.n_samples[s.n_trees - 1] = (uint8_t *)malloc(8);
    memset(s.n_samples[s.n_trees - 1], 1, 8);
    orc_channel_mix_root(&ch, ct->root);

    felts_t f = {0};
    qpoint oods;
    qm31 **sampled = NULL;
    uint64_t oods_pow;
    int rc = prove_tail(&s, &ch, &fp, L, &tw, &f, &oods, &sampled, &oods_pow);
    if (rc == 0 && check) {
        /* sanity check (mod.rs:121-132): the composition from its samples against the constraints
           at the OODS point (Components::eval_composition_polynomial_at_point, Horner over every
           constraint in order, each divided by V(max_log_degree_bound) at the point) */
        const uint32_t mldb = L - b;
        qm31 e4[4];
        for (int k = 0; k < 4; k++) e4[k] = sampled[s.n_trees - 1][2 * (4 + k)];
        qm31 e0[4];
        for (int k = 0; k < 4; k++) e0[k] = sampled[s.n_trees - 1][2 * k];
        qm31 left = from_partial_evals(e0);
        qm31 right = from_partial_evals(e4);
        qm31 x = qpoint_repeated_double(oods, mldb - 1).x;
        qm31 comp_oods = qm31_add(left, qm31_mul(x, right));
        qm31 den_inv = qm31_inv(coset_vanishing_at(coset_odds(mldb), oods));
        qm31 acc = qm31_from_m31(0);
        const qm31 *m = sampled[1];
        c = 0;
        for (uint32_t k = 0; k < n_fib; k++) {
            for (uint32_t j = 0; j + 2 < fib_n_cols[k]; j++) {
                qm31 a = m[2 * (c + j)], bb = m[2 * (c + j + 1)], cc = m[2 * (c + j + 2)];
                qm31 cons = qm31_sub(cc, qm31_add(qm31_sqr(a), qm31_sqr(bb)));
                acc = qm31_add(qm31_mul(acc, random_coeff), qm31_mul(den_inv, cons));
            }
            c += fib_n_cols[k];
        }
        for (uint32_t k = 0; k < n_lookups; k++) {
            qm31 prev4[4], cur4[4];
            for (int j = 0; j < 4; j++) {
                prev4[j] = sampled[2][2 * (4 * k + j)];
                cur4[j] = sampled[2][2 * (4 * k + j) + 1];
            }
            qm31 v = m[2 * (n_fib_cols + k)];
            qm31 shift = qm31_mul_m31(claimed[k], m31_inv((m31)((1ull << lookup_log_sizes[k]) % M31_P)));
            qm31 shifted = qm31_add(qm31_sub(from_partial_evals(cur4), from_partial_evals(prev4)), shift);
            qm31 cons = qm31_add(qm31_mul(shifted, qm31_sub(v, z)), qm31_from_m31(1));
            acc = qm31_add(qm31_mul(acc, random_coeff), qm31_mul(den_inv, cons));
        }
        if (!qm31_eq(acc, comp_oods)) rc = 1;  /* ProvingError::ConstraintsNotSatisfied */
    }
    if (sampled) {
        for (uint32_t tr = 0; tr < s.n_trees; tr++) free(sampled[tr]);
        free(sampled);
    }
    free(claimed); free(tlogs);
    scheme_free(&s);
    free(tw.tw); free(tw.itw);
    int wr = finish_words(&f, words, capacity, n_words);
    return rc ? rc : wr;
}

/* ------------------------------------------------------------------------ Poseidon2 */

#define PS_COLS_ALL 1264
#define PS_INTER_COLS 32
#define PS_N_CONSTRAINTS 1144
#define PS_LOG_EXPAND 2

int orc_prove_poseidon(const uint32_t fri[5], uint32_t log_n_rows, uint64_t *words, size_t capacity,
                       size_t *n_words) {
    fri_params_t fp = {fri[0], fri[1], fri[2], fri[3], fri[4]};
    if (fp.fold_step < 1 || log_n_rows < 1) return -1;
    const uint32_t b = fp.log_blowup_factor;
    const uint32_t n = log_n_rows;
    /* poseidon_pcs_config (crates/examples/src/poseidon/mod.rs:305-318): the split composition is
       LOG_EXPAND - 1 above the trace; twiddles for CanonicCoset(n + LOG_EXPAND + blowup) */
    const uint32_t L = n + PS_LOG_EXPAND - 1 + b;
    twiddles_t tw = twiddles_for(n + PS_LOG_EXPAND + b);
    orc_channel ch;
    memset(&ch, 0, sizeof(ch));
    scheme_t s;
    s.n_trees = 4;
    s.trees = (tree_t *)calloc(4, sizeof(tree_t));
    s.n_samples = (uint8_t **)calloc(4, sizeof(void *));
    tree_commit_evals(&s.trees[0], 0, NULL, NULL, b, 0, &tw);
    s.n_samples[0] = (uint8_t *)calloc(1, 1);
    orc_channel_mix_root(&ch, s.trees[0].root);

    /* trace (gen_trace, mod.rs:195-275) */
    uint32_t **trace = (uint32_t **)malloc(sizeof(void *) * PS_COLS_ALL);
    uint32_t *logs = (uint32_t *)malloc(sizeof(uint32_t) * PS_COLS_ALL);
    for (uint32_t i = 0; i < PS_COLS_ALL; i++) {
        trace[i] = (uint32_t *)malloc(sizeof(uint32_t) << n);
        logs[i] = n;
    }
    orc_poseidon_trace(n, trace);
    tree_commit_evals(&s.trees[1], PS_COLS_ALL, (const uint32_t *const *)trace, logs, b, L, &tw);
    s.n_samples[1] = (uint8_t *)malloc(PS_COLS_ALL);
    memset(s.n_samples[1], 1, PS_COLS_ALL);
    orc_channel_mix_root(&ch, s.trees[1].root);

    /* PoseidonElements::draw (z, alpha), gen_interaction_trace (mod.rs:277-303) */
    qm31 zq = draw_felt(&ch), aq = draw_felt(&ch);
    uint32_t lookup[8];
    qm31_to_words(zq, lookup);
    qm31_to_words(aq, lookup + 4);
    uint32_t **inter = (uint32_t **)malloc(sizeof(void *) * PS_INTER_COLS);
    for (uint32_t i = 0; i < PS_INTER_COLS; i++) inter[i] = (uint32_t *)malloc(sizeof(uint32_t) << n);
    uint32_t claimed[4];
    orc_poseidon_interaction((const uint32_t **)trace, n, lookup, lookup + 4, inter, claimed);
    for (uint32_t i = 0; i < PS_COLS_ALL; i++) free(trace[i]);
    free(trace);
    tree_commit_evals(&s.trees[2], PS_INTER_COLS, (const uint32_t *const *)inter, logs, b, L, &tw);
    for (uint32_t i = 0; i < PS_INTER_COLS; i++) free(inter[i]);
    free(inter);
    /* finalize_logup_in_pairs (crates/constraint-framework/src/lib.rs:185-227): the batches'
       cumulative columns are read at offset 0, the last one also at -1 */
    s.n_samples[2] = (uint8_t *)malloc(PS_INTER_COLS);
    memset(s.n_samples[2], 1, PS_INTER_COLS);
    memset(s.n_samples[2] + PS_INTER_COLS - 4, 2, 4);
    orc_channel_mix_root(&ch, s.trees[2].root);

    /* composition: ExtendToEvalDomain (accumulation.rs:42-62; constraint degree 2 above the trace
       exceeds the blowup), every trace and interaction polynomial evaluated on
       CanonicCoset(n + LOG_EXPAND) from its coefficients */
    qm31 random_coeff = draw_felt(&ch);
    accumulator_t A;
    accumulator_init(&A, random_coeff, PS_N_CONSTRAINTS);
    const uint32_t el = n + PS_LOG_EXPAND;
    uint32_t **ext = (uint32_t **)malloc(sizeof(void *) * (PS_COLS_ALL + PS_INTER_COLS));
    uint32_t *elogs = (uint32_t *)malloc(sizeof(uint32_t) * (PS_COLS_ALL + PS_INTER_COLS));
    const uint32_t **srcs = (const uint32_t **)malloc(sizeof(void *) * (PS_COLS_ALL + PS_INTER_COLS));
    uint32_t *slogs = (uint32_t *)malloc(sizeof(uint32_t) * (PS_COLS_ALL + PS_INTER_COLS));
    for (uint32_t i = 0; i < PS_COLS_ALL + PS_INTER_COLS; i++) {
        ext[i] = (uint32_t *)malloc(sizeof(uint32_t) << el);
        elogs[i] = el;
        srcs[i] = i < PS_COLS_ALL ? s.trees[1].coeffs[i] : s.trees[2].coeffs[i - PS_COLS_ALL];
        slogs[i] = n;
    }
    orc_evaluate_batch(srcs, slogs, ext, elogs, PS_COLS_ALL + PS_INTER_COLS, tw.tw, tw.log);
    uint32_t *rc = accumulator_take(&A, PS_N_CONSTRAINTS);
    orc_poseidon_composition((const uint32_t **)ext, (const uint32_t **)(ext + PS_COLS_ALL), el, n, lookup, claimed,
                             rc, accumulator_col(&A, el));
    free(rc);
    for (uint32_t i = 0; i < PS_COLS_ALL + PS_INTER_COLS; i++) free(ext[i]);
    free(ext); free(elogs); free(srcs); free(slogs); free(logs);
    uint32_t *comp[4];
    uint32_t comp_log = accumulator_finalize(&A, &tw, comp);
    commit_composition(&s.trees[3], comp, comp_log, b, L, &tw);
    s.n_samples[3] = (uint8_t *)malloc(8);
    memset(s.n_samples[3], 1, 8);
    orc_channel_mix_root(&ch, s.trees[3].root);

    felts_t f = {0};
    qpoint oods;
    qm31 **sampled = NULL;
    uint64_t oods_pow;
    /* the reference's own sanity check fails for this AIR in the lifted protocol (the composition
       is not lifted while the trace is); the words are those it computes before that check */
    int r = prove_tail(&s, &ch, &fp, L, &tw, &f, &oods, &sampled, &oods_pow);
    if (sampled) {
        for (uint32_t tr = 0; tr < s.n_trees; tr++) free(sampled[tr]);
        free(sampled);
    }
    scheme_free(&s);
    free(tw.tw); free(tw.itw);
    int wr = finish_words(&f, words, capacity, n_words);
    return r ? r : wr;
}
