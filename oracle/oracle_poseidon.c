/*
 * ORACLE — test infrastructure only (see oracle_core.c). CPU restatement of
 * the Poseidon2 AIR of crates/examples/src/poseidon/mod.rs: state width 16,
 * 4 + 4 full rounds and 14 partial rounds, x^5, all round constants 1234,
 * 8 instances per row (158 columns each, 1264 in all), and its LogUp
 * interaction: per instance the fraction 1/combine(initial) - 1/combine(final)
 * (finalize_logup_in_pairs), combine(v) = sum_i alpha^i v_i - z.
 */
#include <stdlib.h>
#include <string.h>

#include "fields.h"
#include "circle.h"
#include "oracle.h"

#define PS_STATE 16
#define PS_PARTIAL 14
#define PS_HALF_FULL 4
#define PS_INSTANCES 8
#define PS_COLS_PER_REP (PS_STATE * (1 + 2 * PS_HALF_FULL) + PS_PARTIAL) /* 158 */
#define PS_COLS (PS_INSTANCES * PS_COLS_PER_REP)                           /* 1264 */
#define PS_RC 1234u
#define PS_CONSTRAINTS (PS_INSTANCES * (2 * PS_HALF_FULL * PS_STATE + PS_PARTIAL) + PS_INSTANCES) /* 1144 */

/* apply_m4 (mod.rs:72-89): the 4x4 MDS matrix [[5,7,1,3],[4,6,1,1],[1,3,5,7],[1,1,4,6]]. */
static void ps_m4(m31 *x) {
    m31 t0 = m31_add(x[0], x[1]);
    m31 t02 = m31_add(t0, t0);
    m31 t1 = m31_add(x[2], x[3]);
    m31 t12 = m31_add(t1, t1);
    m31 t2 = m31_add(m31_add(x[1], x[1]), t1);
    m31 t3 = m31_add(m31_add(x[3], x[3]), t0);
    m31 t4 = m31_add(m31_add(t12, t12), t3);
    m31 t5 = m31_add(m31_add(t02, t02), t2);
    m31 t6 = m31_add(t3, t5);
    m31 t7 = m31_add(t2, t4);
    x[0] = t6; x[1] = t5; x[2] = t7; x[3] = t4;
}

/* apply_external_round_matrix (mod.rs:91-113): circ(2 M4, M4, M4, M4). */
static void ps_external(m31 *s) {
    for (int i = 0; i < 4; i++) ps_m4(s + 4 * i);
    for (int j = 0; j < 4; j++) {
        m31 t = m31_add(m31_add(s[j], s[j + 4]), m31_add(s[j + 8], s[j + 12]));
        for (int i = 0; i < 4; i++) s[4 * i + j] = m31_add(s[4 * i + j], t);
    }
}

/* apply_internal_round_matrix (mod.rs:115-129): s_i <- s_i * 2^(i+1) + sum(s). */
static void ps_internal(m31 *s) {
    m31 sum = 0;
    for (int i = 0; i < PS_STATE; i++) sum = m31_add(sum, s[i]);
    for (int i = 0; i < PS_STATE; i++) s[i] = m31_add(m31_mul(s[i], 1u << (i + 1)), sum);
}

static m31 ps_pow5(m31 x) {
    m31 x2 = m31_sqr(x);
    return m31_mul(m31_sqr(x2), x);
}

void orc_poseidon_m4(uint32_t x[4]) { ps_m4(x); }
void orc_poseidon_external(uint32_t s[16]) { ps_external(s); }
void orc_poseidon_internal(uint32_t s[16]) { ps_internal(s); }

/* gen_trace (mod.rs:195-275): row r, instance k starts from state_i = r + i + k. */
void orc_poseidon_trace(uint32_t log_n, uint32_t **cols) {
    uint64_t n = 1ull << log_n;
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < (int64_t)n; r++) {
        uint32_t c = 0;
        for (uint32_t k = 0; k < PS_INSTANCES; k++) {
            m31 s[PS_STATE];
            for (int i = 0; i < PS_STATE; i++) {
                s[i] = (m31)(r + i + k);
                cols[c++][r] = s[i];
            }
            for (int round = 0; round < 2 * PS_HALF_FULL + 1; round++) {
                if (round == PS_HALF_FULL) {
                    for (int p = 0; p < PS_PARTIAL; p++) {
                        s[0] = m31_add(s[0], PS_RC);
                        ps_internal(s);
                        s[0] = ps_pow5(s[0]);
                        cols[c++][r] = s[0];
                    }
                    continue;
                }
                for (int i = 0; i < PS_STATE; i++) s[i] = m31_add(s[i], PS_RC);
                ps_external(s);
                for (int i = 0; i < PS_STATE; i++) {
                    s[i] = ps_pow5(s[i]);
                    cols[c++][r] = s[i];
                }
            }
        }
    }
}

/* combine (crates/constraint-framework/src/logup.rs:80-93) of 16 M31 values. */
static qm31 ps_combine(const qm31 *alpha_pow, const m31 *v, qm31 z) {
    qm31 acc = qm31_from_m31(0);
    for (int i = 0; i < PS_STATE; i++) acc = qm31_add(acc, qm31_mul_m31(alpha_pow[i], v[i]));
    return qm31_sub(acc, z);
}

static void ps_alpha_powers(qm31 alpha, qm31 *out) {
    qm31 cur = qm31_from_m31(1);
    for (int i = 0; i < PS_STATE; i++) { out[i] = cur; cur = qm31_mul(cur, alpha); }
}

/*
 * gen_interaction_trace (mod.rs:277-303) with LogupTraceGenerator
 * (crates/constraint-framework/src/prover/logup.rs:55-130): QM31 column k < 7
 * holds, per row, the sum of the fractions of instances 0..k; column 7 holds
 * the row total minus claimed_sum / n, inclusive-prefix-summed in coset order
 * (inclusive_prefix_sum, crates/stwo/src/prover/backend/simd/prefix_sum.rs:20).
 * trace: the 1264 trace columns (bit-reversed order); out: 32 coordinate
 * columns (QM31 column k = out[4k .. 4k + 4]).
 */
void orc_poseidon_interaction(const uint32_t **trace, uint32_t log_n, const uint32_t z_w[4],
                              const uint32_t alpha_w[4], uint32_t **out, uint32_t claimed_out[4]) {
    uint64_t n = 1ull << log_n;
    qm31 z = qm31_from_words(z_w), ap[PS_STATE];
    ps_alpha_powers(qm31_from_words(alpha_w), ap);
    qm31 *total = (qm31 *)malloc(sizeof(qm31) * n);
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < (int64_t)n; r++) {
        qm31 acc = qm31_from_m31(0);
        for (uint32_t k = 0; k < PS_INSTANCES; k++) {
            m31 init[PS_STATE], fin[PS_STATE];
            for (int i = 0; i < PS_STATE; i++) {
                init[i] = trace[k * PS_COLS_PER_REP + i][r];
                fin[i] = trace[k * PS_COLS_PER_REP + PS_COLS_PER_REP - PS_STATE + i][r];
            }
            qm31 d0 = ps_combine(ap, init, z), d1 = ps_combine(ap, fin, z);
            acc = qm31_add(acc, qm31_mul(qm31_sub(d1, d0), qm31_inv(qm31_mul(d0, d1))));
            if (k + 1 < PS_INSTANCES) {
                out[4 * k][r] = acc.a.a; out[4 * k + 1][r] = acc.a.b;
                out[4 * k + 2][r] = acc.b.a; out[4 * k + 3][r] = acc.b.b;
            }
        }
        total[r] = acc;
    }
    qm31 claimed = qm31_from_m31(0);
    for (uint64_t r = 0; r < n; r++) claimed = qm31_add(claimed, total[r]);
    qm31_to_words(claimed, claimed_out);
    qm31 shift = qm31_mul_m31(claimed, m31_inv((m31)(n % M31_P)));
    qm31 run = qm31_from_m31(0);
    uint32_t **last = out + 4 * (PS_INSTANCES - 1);
    for (uint64_t k = 0; k < n; k++) {
        uint64_t c = (k & 1) ? n / 2 + (n - 1 - k) / 2 : k / 2; /* circle-domain index of coset index k */
        uint64_t p = bit_reverse_index((uint32_t)c, log_n);
        run = qm31_add(run, qm31_sub(total[p], shift));
        last[0][p] = run.a.a; last[1][p] = run.a.b; last[2][p] = run.b.a; last[3][p] = run.b.b;
    }
    free(total);
}

/* coset_vanishing at an M31 point (constraints.rs:12-35). */
static m31 ps_coset_vanishing(coset_t c, cpoint p) {
    cpoint q = cpoint_add(cpoint_add(p, cpoint_conj(c.initial)), cidx_to_point(c.step_size >> 1));
    m31 x = q.x;
    for (uint32_t i = 1; i < c.log_size; i++) x = circle_double_x(x);
    return x;
}

/* The row `offset` trace steps from row r of a bit-reversed evaluation domain:
   offset_bit_reversed_circle_domain_index (crates/stwo/src/core/utils.rs:144-160)
   when the domain is larger than the trace (the natural index moves by
   offset * 2^(eval_log - trace_log - 1) forward in the first half and backward in
   the second, modulo the half), the coset-order neighbour
   (crates/constraint-framework/src/prover/assert.rs:58-66) when it is the trace domain. */
uint64_t orc_offset_row(uint64_t r, int64_t offset, uint32_t trace_log, uint32_t eval_log) {
    int64_t i = (int64_t)bit_reverse_index((uint32_t)r, eval_log);
    int64_t n = 1ll << eval_log, half = n / 2;
    if (eval_log > trace_log) {
        int64_t step = offset * (1ll << (eval_log - trace_log - 1));
        if (i < half)
            i = (((i + step) % half) + half) % half;
        else
            i = (((i - step) % half) + half) % half + half;
    } else {
        int64_t k = i < half ? 2 * i : 2 * (n - 1 - i) + 1; /* coset index */
        k = (((k + offset) % n) + n) % n;
        i = (k & 1) ? n / 2 + (n - 1 - k) / 2 : k / 2;
    }
    return bit_reverse_index((uint32_t)i, eval_log);
}

uint64_t orc_prev_row(uint64_t r, uint32_t trace_log, uint32_t eval_log) {
    return orc_offset_row(r, -1, trace_log, eval_log);
}

/* orc_offset_row for every row of the domain. */
void orc_offset_rows(int64_t offset, uint32_t trace_log, uint32_t eval_log, uint64_t *out) {
    for (uint64_t r = 0; r < (1ull << eval_log); r++) out[r] = orc_offset_row(r, offset, trace_log, eval_log);
}

/* orc_prev_row for every row of the domain. */
void orc_prev_rows(uint32_t trace_log, uint32_t eval_log, uint64_t *out) {
    for (uint64_t r = 0; r < (1ull << eval_log); r++) out[r] = orc_prev_row(r, trace_log, eval_log);
}

/*
 * Constraint quotients of the Poseidon component on an evaluation domain
 * (FrameworkComponent::evaluate_constraint_quotients_on_domain,
 * crates/constraint-framework/src/prover/component_prover.rs:195-268, for
 * eval_poseidon_constraints, mod.rs:137-189): per row, sum_k rc[k] C_k with
 * the 1144 constraints in evaluation order (142 per instance, then the 8
 * LogUp batch constraints of finalize_logup_batched, lib.rs:185-222), times
 * the bit-reversed 1/V_trace(eval_domain.at(i)) (component_prover.rs:101-108),
 * added to out. trace / inter: the 1264 and 32 columns on the evaluation
 * domain CanonicCoset(eval_log). lookup = (z, alpha). When eval_log equals
 * trace_log the rows are the trace domain itself: no denominator is applied
 * (every row sum is then zero for a valid trace).
 */
void orc_poseidon_composition(const uint32_t **trace, const uint32_t **inter, uint32_t eval_log, uint32_t trace_log,
                              const uint32_t lookup_w[8], const uint32_t claimed_w[4], const uint32_t *rc,
                              uint32_t *const out[4]) {
    uint32_t log_expand = eval_log - trace_log;
    uint32_t n_den = 1u << log_expand;
    m31 *den = (m31 *)malloc(sizeof(m31) * n_den);
    if (log_expand == 0) {
        den[0] = 1;
    } else {
        coset_t eval_half = canonic_half_coset(eval_log);
        coset_t trace_coset = coset_odds(trace_log);
        for (uint32_t i = 0; i < n_den; i++) den[i] = m31_inv(ps_coset_vanishing(trace_coset, domain_at(eval_half, i)));
        orc_bit_reverse(den, log_expand);
    }
    qm31 z = qm31_from_words(lookup_w), ap[PS_STATE];
    ps_alpha_powers(qm31_from_words(lookup_w + 4), ap);
    qm31 shift = qm31_mul_m31(qm31_from_words(claimed_w), m31_inv((m31)((1ull << trace_log) % M31_P)));
    uint64_t n = 1ull << eval_log;
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < (int64_t)n; r++) {
        qm31 acc = qm31_from_m31(0);
        uint32_t idx = 0, c = 0;
        qm31 num[PS_INSTANCES], dn[PS_INSTANCES];
        for (uint32_t k = 0; k < PS_INSTANCES; k++) {
            m31 s[PS_STATE], init[PS_STATE];
            for (int i = 0; i < PS_STATE; i++) init[i] = s[i] = trace[c++][r];
            for (int round = 0; round < 2 * PS_HALF_FULL + 1; round++) {
                if (round == PS_HALF_FULL) {
                    for (int p = 0; p < PS_PARTIAL; p++) {
                        s[0] = m31_add(s[0], PS_RC);
                        ps_internal(s);
                        s[0] = ps_pow5(s[0]);
                        m31 m = trace[c++][r];
                        acc = qm31_add(acc, qm31_mul_m31(qm31_from_words(rc + 4 * idx++), m31_sub(s[0], m)));
                        s[0] = m;
                    }
                    continue;
                }
                for (int i = 0; i < PS_STATE; i++) s[i] = m31_add(s[i], PS_RC);
                ps_external(s);
                for (int i = 0; i < PS_STATE; i++) {
                    m31 m = trace[c++][r];
                    acc = qm31_add(acc, qm31_mul_m31(qm31_from_words(rc + 4 * idx++), m31_sub(ps_pow5(s[i]), m)));
                    s[i] = m;
                }
            }
            qm31 d0 = ps_combine(ap, init, z), d1 = ps_combine(ap, s, z);
            num[k] = qm31_sub(d1, d0);
            dn[k] = qm31_mul(d0, d1);
        }
        uint64_t pr = orc_prev_row((uint64_t)r, trace_log, eval_log);
        qm31 prev_col = qm31_from_m31(0);
        for (uint32_t k = 0; k < PS_INSTANCES; k++) {
            qm31 cur = qm31_make(inter[4 * k][r], inter[4 * k + 1][r], inter[4 * k + 2][r], inter[4 * k + 3][r]);
            qm31 diff = qm31_sub(cur, prev_col);
            if (k + 1 == PS_INSTANCES) {
                qm31 prev_row = qm31_make(inter[4 * k][pr], inter[4 * k + 1][pr], inter[4 * k + 2][pr],
                                          inter[4 * k + 3][pr]);
                diff = qm31_add(qm31_sub(qm31_sub(cur, prev_row), prev_col), shift);
            }
            prev_col = cur;
            qm31 cons = qm31_sub(qm31_mul(diff, dn[k]), num[k]);
            acc = qm31_add(acc, qm31_mul(qm31_from_words(rc + 4 * idx++), cons));
        }
        acc = qm31_mul_m31(acc, den[(uint64_t)r >> trace_log]);
        qm31 old = qm31_make(out[0][r], out[1][r], out[2][r], out[3][r]);
        qm31 v = qm31_add(old, acc);
        out[0][r] = v.a.a; out[1][r] = v.a.b; out[2][r] = v.b.a; out[3][r] = v.b.b;
    }
    free(den);
}
