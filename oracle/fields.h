/*
 * ORACLE — test infrastructure only. A CPU restatement of the reference
 * prover's arithmetic, used by tests/, the smoke check and bench.py's CPU
 * baseline as the checker. Nothing in the product links or calls this code.
 *
 * Fields: M31 = Z/(2^31-1), CM31 = M31[i]/(i^2+1), QM31 = CM31[u]/(u^2-2-i).
 *   M31   crates/stwo/src/core/fields/m31.rs:14 (P), :46-60 (partial_reduce,
 *         reduce), :78-108 (add/neg/sub/mul)
 *   CM31  crates/stwo/src/core/fields/cm31.rs:44-50 (mul), :64-69 (inverse)
 *   QM31  crates/stwo/src/core/fields/qm31.rs:14 (R = 2+i), :75-81 (mul),
 *         :113-122 (inverse)
 * Every operation maps canonical inputs in [0,P) to canonical outputs.
 */
#ifndef STWO_ORACLE_FIELDS_H
#define STWO_ORACLE_FIELDS_H

#include <stdint.h>
#include <stddef.h>

#define M31_P 0x7fffffffu

typedef uint32_t m31;
typedef struct { m31 a, b; } cm31;          /* a + b*i */
typedef struct { cm31 a, b; } qm31;         /* a + b*u */

/* m31.rs:58-60: v % P for v < P^2. */
static inline m31 m31_reduce64(uint64_t v) {
    return (m31)(((((v >> 31) + v + 1) >> 31) + v) & (uint64_t)M31_P);
}
/* m31.rs:46-48: v % P for v < 2P. */
static inline m31 m31_partial_reduce(uint32_t v) { return v >= M31_P ? v - M31_P : v; }
static inline m31 m31_add(m31 x, m31 y) { return m31_partial_reduce(x + y); }
static inline m31 m31_sub(m31 x, m31 y) { return m31_partial_reduce(x + M31_P - y); }
static inline m31 m31_neg(m31 x) { return m31_partial_reduce(M31_P - x); }
static inline m31 m31_mul(m31 x, m31 y) { return m31_reduce64((uint64_t)x * (uint64_t)y); }
static inline m31 m31_sqr(m31 x) { return m31_mul(x, x); }
static inline m31 m31_pow(m31 x, uint64_t e) {
    m31 r = 1;
    while (e) { if (e & 1) r = m31_mul(r, x); x = m31_sqr(x); e >>= 1; }
    return r;
}
/* Fermat inverse x^(P-2); the reference's addition chain gives the same value. */
static inline m31 m31_inv(m31 x) { return m31_pow(x, M31_P - 2); }

static inline cm31 cm31_make(m31 a, m31 b) { cm31 r = {a, b}; return r; }
static inline cm31 cm31_add(cm31 x, cm31 y) { return cm31_make(m31_add(x.a, y.a), m31_add(x.b, y.b)); }
static inline cm31 cm31_sub(cm31 x, cm31 y) { return cm31_make(m31_sub(x.a, y.a), m31_sub(x.b, y.b)); }
static inline cm31 cm31_neg(cm31 x) { return cm31_make(m31_neg(x.a), m31_neg(x.b)); }
static inline cm31 cm31_mul(cm31 x, cm31 y) {
    /* (a+bi)(c+di) = (ac-bd) + (ad+bc)i */
    return cm31_make(m31_sub(m31_mul(x.a, y.a), m31_mul(x.b, y.b)),
                     m31_add(m31_mul(x.a, y.b), m31_mul(x.b, y.a)));
}
static inline cm31 cm31_mul_m31(cm31 x, m31 y) { return cm31_make(m31_mul(x.a, y), m31_mul(x.b, y)); }
static inline int cm31_is_zero(cm31 x) { return x.a == 0 && x.b == 0; }
static inline cm31 cm31_inv(cm31 x) {
    /* 1/(a+bi) = (a-bi)/(a^2+b^2) */
    m31 d = m31_inv(m31_add(m31_sqr(x.a), m31_sqr(x.b)));
    return cm31_make(m31_mul(x.a, d), m31_mul(m31_neg(x.b), d));
}

static inline qm31 qm31_make(m31 a, m31 b, m31 c, m31 d) {
    qm31 r; r.a = cm31_make(a, b); r.b = cm31_make(c, d); return r;
}
static inline qm31 qm31_from_m31(m31 a) { return qm31_make(a, 0, 0, 0); }
static inline qm31 qm31_add(qm31 x, qm31 y) { qm31 r = {cm31_add(x.a, y.a), cm31_add(x.b, y.b)}; return r; }
static inline qm31 qm31_sub(qm31 x, qm31 y) { qm31 r = {cm31_sub(x.a, y.a), cm31_sub(x.b, y.b)}; return r; }
static inline qm31 qm31_neg(qm31 x) { qm31 r = {cm31_neg(x.a), cm31_neg(x.b)}; return r; }
static inline qm31 qm31_mul(qm31 x, qm31 y) {
    /* (a+bu)(c+du) = (ac + R*bd) + (ad+bc)u with R = 2+i */
    const cm31 R = {2, 1};
    qm31 r;
    r.a = cm31_add(cm31_mul(x.a, y.a), cm31_mul(R, cm31_mul(x.b, y.b)));
    r.b = cm31_add(cm31_mul(x.a, y.b), cm31_mul(x.b, y.a));
    return r;
}
static inline qm31 qm31_mul_m31(qm31 x, m31 y) { qm31 r = {cm31_mul_m31(x.a, y), cm31_mul_m31(x.b, y)}; return r; }
static inline qm31 qm31_mul_cm31(qm31 x, cm31 y) { qm31 r = {cm31_mul(x.a, y), cm31_mul(x.b, y)}; return r; }
static inline qm31 qm31_sqr(qm31 x) { return qm31_mul(x, x); }
static inline int qm31_is_zero(qm31 x) { return cm31_is_zero(x.a) && cm31_is_zero(x.b); }
static inline int qm31_eq(qm31 x, qm31 y) {
    return x.a.a == y.a.a && x.a.b == y.a.b && x.b.a == y.b.a && x.b.b == y.b.b;
}
static inline qm31 qm31_inv(qm31 x) {
    /* (a+bu)^-1 = (a-bu)/(a^2 - (2+i)b^2) */
    cm31 b2 = cm31_mul(x.b, x.b);
    cm31 ib2 = cm31_make(m31_neg(b2.b), b2.a);
    cm31 denom = cm31_sub(cm31_mul(x.a, x.a), cm31_add(cm31_add(b2, b2), ib2));
    cm31 di = cm31_inv(denom);
    qm31 r = {cm31_mul(x.a, di), cm31_mul(cm31_neg(x.b), di)};
    return r;
}
static inline qm31 qm31_pow(qm31 x, uint64_t e) {
    qm31 r = qm31_from_m31(1);
    while (e) { if (e & 1) r = qm31_mul(r, x); x = qm31_sqr(x); e >>= 1; }
    return r;
}
static inline void qm31_to_words(qm31 x, uint32_t w[4]) { w[0] = x.a.a; w[1] = x.a.b; w[2] = x.b.a; w[3] = x.b.b; }
static inline qm31 qm31_from_words(const uint32_t w[4]) { return qm31_make(w[0], w[1], w[2], w[3]); }

static inline uint32_t bit_reverse_index(uint32_t i, uint32_t log_size) {
    /* crates/stwo/src/core/utils.rs:106-111 */
    if (log_size == 0) return i;
    uint32_t r = 0;
    for (uint32_t k = 0; k < log_size; k++) r |= ((i >> k) & 1u) << (log_size - 1 - k);
    return r;
}

#endif
