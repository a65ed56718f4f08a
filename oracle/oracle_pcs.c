/*
 * ORACLE — test infrastructure only (see oracle_core.c). CPU restatement of
 * the reference's accumulation, DEEP-quotient and out-of-domain sampling ops.
 */
#include <stdlib.h>
#include <string.h>

#include "fields.h"
#include "circle.h"
#include "oracle.h"

static inline qm31 soa_at(const uint32_t *const c[4], uint64_t i) {
    return qm31_make(c[0][i], c[1][i], c[2][i], c[3][i]);
}
static inline void soa_set(uint32_t *const c[4], uint64_t i, qm31 v) {
    c[0][i] = v.a.a; c[1][i] = v.a.b; c[2][i] = v.b.a; c[3][i] = v.b.b;
}

/* AccumulationOps::accumulate (crates/stwo/src/prover/backend/cpu/accumulation.rs:9-14). */
void orc_accumulate(uint32_t *const col[4], const uint32_t *const other[4], uint64_t n) {
    for (uint64_t i = 0; i < n; i++) soa_set(col, i, qm31_add(soa_at((const uint32_t *const *)col, i), soa_at(other, i)));
}

/* generate_secure_powers (accumulation.rs:16-24). */
void orc_generate_secure_powers(const uint32_t felt[4], uint32_t n, uint32_t *out) {
    qm31 f = qm31_from_words(felt), acc = qm31_from_m31(1);
    for (uint32_t i = 0; i < n; i++) { qm31_to_words(acc, out + 4 * i); acc = qm31_mul(acc, f); }
}

/*
 * lift_and_accumulate (accumulation.rs:26-47): columns sorted by strictly
 * increasing length; cols is n_cols x 4 coordinate pointers (flattened), each
 * updated in place; the last one holds the result.
 */
void orc_lift_and_accumulate(uint32_t *const *cols, const uint32_t *log_sizes, uint32_t n_cols) {
    uint32_t cur_log = 1;
    qm31 zeros[2] = {qm31_from_m31(0), qm31_from_m31(0)};
    uint32_t *const *cur = NULL;
    for (uint32_t k = 0; k < n_cols; k++) {
        uint32_t *const *col = cols + 4 * k;
        uint32_t l = log_sizes[k];
        uint32_t log_ratio = l - cur_log;
        uint64_t n = 1ull << l;
        for (uint64_t i = 0; i < n; i++) {
            uint64_t j = ((i >> (log_ratio + 1)) << 1) + (i & 1);
            qm31 prev = cur ? soa_at((const uint32_t *const *)cur, j) : zeros[j];
            soa_set(col, i, qm31_add(soa_at((const uint32_t *const *)col, i), prev));
        }
        cur = col;
        cur_log = l;
    }
}

/* ------------------------------------------------------------ vanishing */

/* coset_vanishing (crates/stwo/src/core/constraints.rs:12-34) at a QM31 point. */
static qm31 coset_vanishing_q(coset_t c, qpoint p) {
    /* p - initial + half(step_size).to_point() */
    cpoint neg_init = cpoint_conj(c.initial);
    cpoint half_step = cidx_to_point(c.step_size >> 1);
    qpoint q = qpoint_add(qpoint_add(p, qpoint_from_cpoint(neg_init)), qpoint_from_cpoint(half_step));
    qm31 x = q.x;
    for (uint32_t i = 1; i < c.log_size; i++) x = qcircle_double_x(x);
    return x;
}

/* coset_vanishing at an M31 point (all arithmetic stays in M31). */
static m31 coset_vanishing_m(coset_t c, cpoint p) {
    cpoint q = cpoint_add(cpoint_add(p, cpoint_conj(c.initial)), cidx_to_point(c.step_size >> 1));
    m31 x = q.x;
    for (uint32_t i = 1; i < c.log_size; i++) x = circle_double_x(x);
    return x;
}

/* coset_vanishing_derivative (constraints.rs:37-53) at an M31 point. */
static m31 coset_vanishing_derivative_m(uint32_t log_size, cpoint p) {
    m31 exp = 1;
    for (uint32_t i = 1; i < log_size; i++) exp = m31_mul(exp, 4);
    m31 v = 1;
    for (uint32_t i = 1; i < log_size; i++) v = m31_mul(v, coset_vanishing_m(coset_odds(i), p));
    return m31_mul(exp, v);
}

/*
 * barycentric_weights_into (crates/stwo/src/prover/backend/cpu/circle.rs:100-132):
 * W_i = V_n(p) / (si_i * vi_p), si_i = -2 y_i * V'_n(x_i), vi_p = h.y / (1 + h.x),
 * h = p - x_i, x_i = domain.at(bitrev(i)).
 */
void orc_barycentric_weights(uint32_t log_n, const uint32_t px[4], const uint32_t py[4], uint32_t *const out[4]) {
    coset_t half = canonic_half_coset(log_n);
    qpoint p = {qm31_from_words(px), qm31_from_words(py)};
    qm31 vn_p = coset_vanishing_q(coset_odds(log_n), p);
    uint64_t n = 1ull << log_n;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; i++) {
        cpoint xi = domain_at(half, bit_reverse_index((uint32_t)i, log_n));
        m31 si = m31_mul(m31_mul(xi.y, m31_neg(2)), coset_vanishing_derivative_m(log_n, xi));
        /* point_vanishing(xi, p) = h.y / (1 + h.x), h = p - xi */
        qpoint h = qpoint_add(p, qpoint_from_cpoint(cpoint_conj(xi)));
        qm31 vi = qm31_mul(h.y, qm31_inv(qm31_add(qm31_from_m31(1), h.x)));
        qm31 w = qm31_mul(vn_p, qm31_inv(qm31_mul_m31(vi, si)));
        soa_set(out, i, w);
    }
}

/* barycentric_eval_at_point (cpu/circle.rs:134-140). */
void orc_barycentric_eval(const uint32_t *evals, uint32_t log_n, const uint32_t *const weights[4], uint32_t out[4]) {
    qm31 acc = qm31_from_m31(0);
    uint64_t n = 1ull << log_n;
    for (uint64_t i = 0; i < n; i++) acc = qm31_add(acc, qm31_mul_m31(soa_at(weights, i), evals[i]));
    qm31_to_words(acc, out);
}

/* ----------------------------------------------------------- quotients */

/*
 * complex_conjugate_line_coeffs (crates/stwo/src/core/constraints.rs:119-135):
 * a = conj(v) - v, c = conj(p.y) - p.y, b = v*c - a*p.y, all times alpha.
 * conj is with respect to CM31: (a + b u) -> (a - b u).
 */
void orc_line_coeffs(const uint32_t py[4], const uint32_t value[4], const uint32_t alpha[4], uint32_t out[12]) {
    qm31 y = qm31_from_words(py), v = qm31_from_words(value), al = qm31_from_words(alpha);
    qm31 vc = v; vc.b = cm31_neg(v.b);
    qm31 yc = y; yc.b = cm31_neg(y.b);
    qm31 a = qm31_sub(vc, v);
    qm31 c = qm31_sub(yc, y);
    qm31 b = qm31_sub(qm31_mul(v, c), qm31_mul(a, y));
    qm31_to_words(qm31_mul(al, a), out);
    qm31_to_words(qm31_mul(al, b), out + 4);
    qm31_to_words(qm31_mul(al, c), out + 8);
}

/*
 * accumulate_numerators for one sample batch (crates/stwo/src/prover/backend/cpu/quotients.rs:23-49
 * with accumulate_row_partial_numerators, crates/stwo/src/core/pcs/quotients.rs:191-203):
 * row r < 2^(l - log_blowup): sum_t (c_t * col_t[r] - b_t). coeffs holds (a, b, c)
 * per term (12 words). first_linear_out = sum_t a_t.
 */
void orc_accumulate_numerators(const uint32_t **cols, uint32_t n_terms, uint32_t log_size, uint32_t log_blowup,
                               const uint32_t *coeffs, uint32_t *const out[4], uint32_t first_linear_out[4]) {
    uint64_t rows = 1ull << (log_size - log_blowup);
    qm31 sum_a = qm31_from_m31(0);
    for (uint32_t t = 0; t < n_terms; t++) sum_a = qm31_add(sum_a, qm31_from_words(coeffs + 12 * t));
    qm31_to_words(sum_a, first_linear_out);
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < (int64_t)rows; r++) {
        qm31 acc = qm31_from_m31(0);
        for (uint32_t t = 0; t < n_terms; t++) {
            qm31 b = qm31_from_words(coeffs + 12 * t + 4), c = qm31_from_words(coeffs + 12 * t + 8);
            acc = qm31_add(acc, qm31_sub(qm31_mul_m31(c, cols[t][r]), b));
        }
        soa_set(out, r, acc);
    }
}

/*
 * compute_quotients_and_combine, first half (cpu/quotients.rs:51-81): the
 * quotient on the subdomain of log L - b, in bit-reversed order. accs is
 * n_points x 4 coordinate pointers (flattened) of log sizes acc_logs;
 * points holds x (4 words) then y (4 words) per sample point.
 * denominator_inverses: crates/stwo/src/core/pcs/quotients.rs:233-256.
 */
void orc_quotients_on_subdomain(const uint32_t *const *accs, const uint32_t *acc_logs, uint32_t n_points,
                                const uint32_t *points, const uint32_t *first_linear, uint32_t lifting_log_size,
                                uint32_t log_blowup, uint32_t *const out[4]) {
    uint32_t sub_log = lifting_log_size - log_blowup;
    /* eval_domain.split(log_blowup).0: half coset Coset(eval half initial, L - 1 - b) */
    coset_t eval_half = canonic_half_coset(lifting_log_size);
    coset_t sub_half = coset_new(eval_half.initial_index, sub_log - 1);
    uint64_t rows = 1ull << sub_log;
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < (int64_t)rows; r++) {
        cpoint dp = domain_at(sub_half, bit_reverse_index((uint32_t)r, sub_log));
        qm31 q = qm31_from_m31(0);
        for (uint32_t k = 0; k < n_points; k++) {
            qm31 px = qm31_from_words(points + 8 * k), py = qm31_from_words(points + 8 * k + 4);
            /* (prx - x) * piy - (pry - y) * pix, in CM31 */
            cm31 prx = px.a, pix = px.b, pry = py.a, piy = py.b;
            cm31 dx = cm31_sub(prx, cm31_make(dp.x, 0)), dy = cm31_sub(pry, cm31_make(dp.y, 0));
            cm31 den = cm31_sub(cm31_mul(dx, piy), cm31_mul(dy, pix));
            cm31 den_inv = cm31_inv(den);
            uint32_t l = acc_logs[k];
            uint32_t log_ratio = sub_log - l;
            uint64_t li = (((uint64_t)r >> (log_ratio + 1)) << 1) + ((uint64_t)r & 1);
            qm31 num = qm31_sub(soa_at((const uint32_t *const *)(accs + 4 * k), li),
                                qm31_mul_m31(qm31_from_words(first_linear + 4 * k), dp.y));
            q = qm31_add(q, qm31_mul_cm31(num, den_inv));
        }
        soa_set(out, r, q);
    }
}

/*
 * decompose (crates/stwo/src/prover/backend/cpu/fri.rs:39-61,134-145):
 * lambda = (sum first half - sum second half) / n; g = f - lambda (first
 * half), f + lambda (second half).
 */
void orc_decompose(const uint32_t *const in[4], uint32_t log_n, uint32_t *const out[4], uint32_t lambda_out[4]) {
    uint64_t n = 1ull << log_n, half = n / 2;
    qm31 a = qm31_from_m31(0), b = qm31_from_m31(0);
    for (uint64_t i = 0; i < half; i++) a = qm31_add(a, soa_at(in, i));
    for (uint64_t i = half; i < n; i++) b = qm31_add(b, soa_at(in, i));
    qm31 lambda = qm31_mul_m31(qm31_sub(a, b), m31_inv((m31)(n % M31_P)));
    qm31_to_words(lambda, lambda_out);
    for (uint64_t i = 0; i < half; i++) soa_set(out, i, qm31_sub(soa_at(in, i), lambda));
    for (uint64_t i = half; i < n; i++) soa_set(out, i, qm31_add(soa_at(in, i), lambda));
}

/* Circle point of a QM31 random draw: CirclePoint::get_random_point (crates/stwo/src/core/circle.rs:150-160). */
void orc_random_point_from_t(const uint32_t t_w[4], uint32_t px[4], uint32_t py[4]) {
    qm31 t = qm31_from_words(t_w);
    qm31 t2 = qm31_sqr(t);
    qm31 inv = qm31_inv(qm31_add(t2, qm31_from_m31(1)));
    qm31_to_words(qm31_mul(qm31_sub(qm31_from_m31(1), t2), inv), px);
    qm31_to_words(qm31_mul(qm31_add(t, t), inv), py);
}

/* ------------------------------------------------------ Wide-Fibonacci AIR */

/*
 * FrameworkComponent<WideFibonacciEval<N>>::evaluate_constraint_quotients_on_domain
 * for CpuBackend (crates/constraint-framework/src/prover/component_prover.rs:195-268)
 * in the SubDomain mode with log_expansion 0: the evaluation domain is
 * CanonicCoset(eval_log).circle_domain(); row r accumulates
 * sum_k rc[k] * (c_{k+2}[r] - (c_k[r]^2 + c_{k+1}[r]^2))
 * (crates/examples/src/wide_fibonacci/mod.rs:87-97) with rc the reversed
 * powers of the random coefficient, times
 * denom_inv[r >> trace_log] = bit-reversed 1/V_trace(eval_domain.at(i))
 * (component_prover.rs:101-108). out is added to (accumulator semantics).
 */
void orc_wide_fib_composition(const uint32_t **cols, uint32_t n_cols, uint32_t eval_log, uint32_t trace_log,
                              const uint32_t *rc, uint32_t *const out[4]) {
    uint32_t log_expand = eval_log - trace_log;
    uint32_t n_den = 1u << log_expand;
    m31 *den = (m31 *)malloc(sizeof(m31) * n_den);
    coset_t eval_half = canonic_half_coset(eval_log);
    coset_t trace_coset = coset_odds(trace_log);
    for (uint32_t i = 0; i < n_den; i++) den[i] = m31_inv(coset_vanishing_m(trace_coset, domain_at(eval_half, i)));
    orc_bit_reverse(den, log_expand);
    uint64_t n = 1ull << eval_log;
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < (int64_t)n; r++) {
        qm31 acc = qm31_from_m31(0);
        for (uint32_t k = 0; k + 2 < n_cols; k++) {
            m31 a = cols[k][r], b = cols[k + 1][r], c = cols[k + 2][r];
            m31 cons = m31_sub(c, m31_add(m31_sqr(a), m31_sqr(b)));
            acc = qm31_add(acc, qm31_mul_m31(qm31_from_words(rc + 4 * k), cons));
        }
        acc = qm31_mul_m31(acc, den[(uint64_t)r >> trace_log]);
        qm31 prev = soa_at((const uint32_t *const *)out, r);
        soa_set(out, r, qm31_add(prev, acc));
    }
    free(den);
}

/* Wide-Fibonacci trace (crates/examples/src/wide_fibonacci/mod.rs:27-48): column 0 = a,
   column 1 = b, then (a, b) <- (b, a^2 + b^2). */
void orc_wide_fib_trace(const uint32_t *a0, const uint32_t *b0, uint32_t log_n, uint32_t n_cols, uint32_t **cols) {
    uint64_t n = 1ull << log_n;
    for (uint64_t r = 0; r < n; r++) {
        m31 a = a0[r], b = b0[r];
        cols[0][r] = a;
        cols[1][r] = b;
        for (uint32_t k = 2; k < n_cols; k++) {
            m31 c = m31_add(m31_sqr(a), m31_sqr(b));
            a = b;
            b = c;
            cols[k][r] = b;
        }
    }
}

/* ------------------------------------------------------------------ LogUp */

/*
 * One LogUp interaction column finalized as the last column
 * (LogupTraceGenerator::col_from_iter + finalize_last,
 * crates/constraint-framework/src/prover/logup.rs:50-130): fractions
 * 1 / (z - v_i), claimed_sum = sum of them, each shifted by claimed_sum / n,
 * then inclusive_prefix_sum in coset order
 * (inclusive_prefix_sum_slow, crates/stwo/src/prover/backend/simd/prefix_sum.rs:132-149,
 * coset_order_to_circle_domain_order, crates/stwo/src/core/utils.rs:177-188).
 * values and out are in bit-reversed circle-domain order.
 */
void orc_logup_running_sum(const uint32_t *values, uint32_t log_n, const uint32_t z_w[4], uint32_t *const out[4],
                           uint32_t claimed_out[4]) {
    uint64_t n = 1ull << log_n;
    qm31 z = qm31_from_words(z_w);
    qm31 *f = (qm31 *)malloc(sizeof(qm31) * n);
    qm31 claimed = qm31_from_m31(0);
    for (uint64_t i = 0; i < n; i++) {
        f[i] = qm31_inv(qm31_sub(z, qm31_from_m31(values[i])));
        claimed = qm31_add(claimed, f[i]);
    }
    qm31_to_words(claimed, claimed_out);
    qm31 shift = qm31_mul_m31(claimed, m31_inv((m31)(n % M31_P)));
    qm31 acc = qm31_from_m31(0);
    for (uint64_t k = 0; k < n; k++) {
        uint64_t c = (k & 1) ? n / 2 + (n - 1 - k) / 2 : k / 2;  /* circle-domain index of coset index k */
        uint64_t p = bit_reverse_index((uint32_t)c, log_n);
        acc = qm31_add(acc, qm31_sub(f[p], shift));
        soa_set(out, p, acc);
    }
    free(f);
}

/*
 * LookupElements::combine (crates/constraint-framework/src/logup.rs:80-94) per row:
 * den[r] = sum_i alpha^i values_i[r] - z, alpha_powers holding alpha^i as 4 words each.
 */
void orc_logup_combine(const uint32_t *const *values, uint32_t n_values, uint32_t log_n,
                       const uint32_t *alpha_powers, const uint32_t z_w[4], uint32_t *const out[4]) {
    uint64_t n = 1ull << log_n;
    qm31 z = qm31_from_words(z_w);
    for (uint64_t r = 0; r < n; r++) {
        qm31 acc = qm31_from_m31(0);
        for (uint32_t i = 0; i < n_values; i++)
            acc = qm31_add(acc, qm31_mul_m31(qm31_from_words(alpha_powers + 4 * i), values[i][r]));
        soa_set(out, r, qm31_sub(acc, z));
    }
}

/*
 * LogupColGenerator::write_frac for every row, then finalize_col
 * (crates/constraint-framework/src/prover/logup.rs:133-196): out[r] = num[r] / den[r] + prev[r],
 * prev the generator's previous column (NULL: none). The numerator is QM31 (num, 4 coordinates)
 * or, when num is NULL, the M31 column num_m31.
 */
void orc_logup_gen_col(const uint32_t *const num[4], const uint32_t *num_m31, const uint32_t *const den[4],
                       const uint32_t *const prev[4], uint32_t log_n, uint32_t *const out[4]) {
    uint64_t n = 1ull << log_n;
    for (uint64_t r = 0; r < n; r++) {
        qm31 nu = num ? soa_at(num, r) : qm31_from_m31(num_m31[r]);
        qm31 v = qm31_mul(nu, qm31_inv(soa_at(den, r)));
        if (prev) v = qm31_add(v, soa_at(prev, r));
        soa_set(out, r, v);
    }
}

/*
 * LogupTraceGenerator::finalize_last (crates/constraint-framework/src/prover/logup.rs:96-130) in
 * place: claimed = the column's sum, every value minus claimed / n, then the inclusive prefix sum
 * in coset order over the bit-reversed circle-domain storage (inclusive_prefix_sum,
 * crates/stwo/src/prover/backend/simd/prefix_sum.rs:20-149).
 */
void orc_logup_finalize_last(uint32_t *const col[4], uint32_t log_n, uint32_t claimed_out[4]) {
    uint64_t n = 1ull << log_n;
    qm31 claimed = qm31_from_m31(0);
    for (uint64_t r = 0; r < n; r++) claimed = qm31_add(claimed, soa_at((const uint32_t *const *)col, r));
    qm31_to_words(claimed, claimed_out);
    qm31 shift = qm31_mul_m31(claimed, m31_inv((m31)(n % M31_P)));
    qm31 *f = (qm31 *)malloc(sizeof(qm31) * n);
    for (uint64_t r = 0; r < n; r++) f[r] = qm31_sub(soa_at((const uint32_t *const *)col, r), shift);
    qm31 acc = qm31_from_m31(0);
    for (uint64_t k = 0; k < n; k++) {
        uint64_t c = (k & 1) ? n / 2 + (n - 1 - k) / 2 : k / 2; /* circle-domain index of coset index k */
        uint64_t p = bit_reverse_index((uint32_t)c, log_n);
        acc = qm31_add(acc, f[p]);
        soa_set(col, p, acc);
    }
    free(f);
}

/*
 * Constraint quotients of a single-column LogUp component on an evaluation
 * domain: the relation entry (multiplicity -1, values [v]) finalized with
 * finalize_logup (crates/constraint-framework/src/lib.rs:185-227, batch size
 * 1): fraction -1 / (v - z); with cur and prev the interaction column at the
 * row and one trace step before (offset -1), the constraint is
 * (cur - prev + claimed / 2^trace_log) (v - z) + 1, weighted by rc and
 * divided by V_trace as for any component (component_prover.rs:195-268);
 * added to out. values / inter: the trace column and the 4 coordinates of
 * the interaction column on CanonicCoset(eval_log).
 */
void orc_logup_composition(const uint32_t *values, const uint32_t *const inter[4], uint32_t eval_log,
                           uint32_t trace_log, const uint32_t z_w[4], const uint32_t claimed_w[4],
                           const uint32_t rc_w[4], uint32_t *const out[4]) {
    uint32_t log_expand = eval_log - trace_log;
    uint32_t n_den = 1u << log_expand;
    m31 *den = (m31 *)malloc(sizeof(m31) * n_den);
    if (log_expand == 0) {
        den[0] = 1;
    } else {
        coset_t eval_half = canonic_half_coset(eval_log);
        coset_t trace_coset = coset_odds(trace_log);
        for (uint32_t i = 0; i < n_den; i++) den[i] = m31_inv(coset_vanishing_m(trace_coset, domain_at(eval_half, i)));
        orc_bit_reverse(den, log_expand);
    }
    qm31 z = qm31_from_words(z_w), rc = qm31_from_words(rc_w);
    qm31 shift = qm31_mul_m31(qm31_from_words(claimed_w), m31_inv((m31)((1ull << trace_log) % M31_P)));
    uint64_t n = 1ull << eval_log;
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < (int64_t)n; r++) {
        uint64_t pr = orc_prev_row((uint64_t)r, trace_log, eval_log);
        qm31 cur = soa_at(inter, r), prev = soa_at(inter, pr);
        qm31 shifted = qm31_add(qm31_sub(cur, prev), shift);
        qm31 cons = qm31_add(qm31_mul(shifted, qm31_sub(qm31_from_m31(values[r]), z)), qm31_from_m31(1));
        qm31 acc = qm31_mul_m31(qm31_mul(rc, cons), den[r >> trace_log]);
        soa_set(out, r, qm31_add(soa_at((const uint32_t *const *)out, r), acc));
    }
    free(den);
}
