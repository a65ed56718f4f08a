/*
 * ORACLE — test infrastructure only (see fields.h).
 *
 * The circle group x^2+y^2=1 over M31 and QM31, cosets and circle domains.
 *   points, add, double, mul     crates/stwo/src/core/circle.rs:18-116
 *   M31_CIRCLE_GEN               crates/stwo/src/core/circle.rs:181-182
 *   SECURE_FIELD_CIRCLE_GEN      crates/stwo/src/core/circle.rs:188-191
 *   CirclePointIndex             crates/stwo/src/core/circle.rs:198-259
 *   Coset                        crates/stwo/src/core/circle.rs:262-377
 *   CanonicCoset / CircleDomain  crates/stwo/src/core/poly/circle/canonic.rs:43-68,
 *                                crates/stwo/src/core/poly/circle/domain.rs:117-160
 */
#ifndef STWO_ORACLE_CIRCLE_H
#define STWO_ORACLE_CIRCLE_H

#include "fields.h"

#define M31_CIRCLE_LOG_ORDER 31u
#define CIRCLE_INDEX_MASK ((1u << M31_CIRCLE_LOG_ORDER) - 1u)

typedef struct { m31 x, y; } cpoint;         /* CirclePoint<M31> */
typedef struct { qm31 x, y; } qpoint;        /* CirclePoint<QM31> */

static inline cpoint cpoint_zero(void) { cpoint p = {1, 0}; return p; }
static inline cpoint cpoint_add(cpoint p, cpoint q) {
    cpoint r;
    r.x = m31_sub(m31_mul(p.x, q.x), m31_mul(p.y, q.y));
    r.y = m31_add(m31_mul(p.x, q.y), m31_mul(p.y, q.x));
    return r;
}
static inline cpoint cpoint_double(cpoint p) { return cpoint_add(p, p); }
static inline cpoint cpoint_conj(cpoint p) { cpoint r = {p.x, m31_neg(p.y)}; return r; }
static inline cpoint cpoint_mul(cpoint p, uint64_t scalar) {
    cpoint r = cpoint_zero(), cur = p;
    while (scalar) { if (scalar & 1) r = cpoint_add(r, cur); cur = cpoint_double(cur); scalar >>= 1; }
    return r;
}
static inline m31 circle_double_x(m31 x) { m31 s = m31_sqr(x); return m31_sub(m31_add(s, s), 1); }

static inline cpoint m31_circle_gen(void) { cpoint g = {2u, 1268011823u}; return g; }

/* CirclePointIndex arithmetic is modulo 2^31. */
static inline uint32_t cidx_subgroup_gen(uint32_t log_size) { return 1u << (M31_CIRCLE_LOG_ORDER - log_size); }
static inline uint32_t cidx_add(uint32_t a, uint32_t b) { return (a + b) & CIRCLE_INDEX_MASK; }
static inline uint32_t cidx_mul(uint32_t a, uint64_t k) { return (uint32_t)(((uint64_t)a * k) & CIRCLE_INDEX_MASK); }
static inline uint32_t cidx_neg(uint32_t a) { return ((1u << M31_CIRCLE_LOG_ORDER) - a) & CIRCLE_INDEX_MASK; }
static inline cpoint cidx_to_point(uint32_t idx) { return cpoint_mul(m31_circle_gen(), idx); }

static inline qpoint qpoint_from_cpoint(cpoint p) { qpoint r = {qm31_from_m31(p.x), qm31_from_m31(p.y)}; return r; }
static inline qpoint qpoint_add(qpoint p, qpoint q) {
    qpoint r;
    r.x = qm31_sub(qm31_mul(p.x, q.x), qm31_mul(p.y, q.y));
    r.y = qm31_add(qm31_mul(p.x, q.y), qm31_mul(p.y, q.x));
    return r;
}
static inline qm31 qcircle_double_x(qm31 x) { qm31 s = qm31_sqr(x); return qm31_sub(qm31_add(s, s), qm31_from_m31(1)); }

typedef struct {
    uint32_t initial_index;
    cpoint initial;
    uint32_t step_size;
    cpoint step;
    uint32_t log_size;
} coset_t;

static inline coset_t coset_new(uint32_t initial_index, uint32_t log_size) {
    coset_t c;
    c.initial_index = initial_index;
    c.initial = cidx_to_point(initial_index);
    c.step_size = cidx_subgroup_gen(log_size);
    c.step = cidx_to_point(c.step_size);
    c.log_size = log_size;
    return c;
}
static inline coset_t coset_subgroup(uint32_t log_size) { return coset_new(0, log_size); }
static inline coset_t coset_odds(uint32_t log_size) { return coset_new(cidx_subgroup_gen(log_size + 1), log_size); }
static inline coset_t coset_half_odds(uint32_t log_size) { return coset_new(cidx_subgroup_gen(log_size + 2), log_size); }
static inline coset_t coset_double(coset_t c) {
    coset_t r;
    r.initial_index = cidx_mul(c.initial_index, 2);
    r.initial = cpoint_double(c.initial);
    r.step = cpoint_double(c.step);
    r.step_size = cidx_mul(c.step_size, 2);
    r.log_size = c.log_size ? c.log_size - 1 : 0;
    return r;
}
static inline uint32_t coset_index_at(coset_t c, uint64_t i) { return cidx_add(c.initial_index, cidx_mul(c.step_size, i)); }
static inline cpoint coset_at(coset_t c, uint64_t i) { return cidx_to_point(coset_index_at(c, i)); }
static inline coset_t coset_conjugate(coset_t c) {
    coset_t r;
    r.initial_index = cidx_neg(c.initial_index);
    r.initial = cidx_to_point(r.initial_index);
    r.step_size = cidx_neg(c.step_size);
    r.step = cidx_to_point(r.step_size);
    r.log_size = c.log_size;
    return r;
}

/* CanonicCoset(n): coset = odds(n); half_coset = half_odds(n-1); circle_domain(half_coset). */
static inline coset_t canonic_half_coset(uint32_t log_size) { return coset_half_odds(log_size - 1); }

/* CircleDomain::index_at: first the half coset, then its conjugate. */
static inline uint32_t domain_index_at(coset_t half, uint64_t i) {
    uint64_t hs = 1ull << half.log_size;
    if (i < hs) return coset_index_at(half, i);
    return cidx_neg(coset_index_at(half, i - hs));
}
static inline cpoint domain_at(coset_t half, uint64_t i) { return cidx_to_point(domain_index_at(half, i)); }

#endif
