// Device arithmetic over M31 = 2^31 - 1 and its extensions CM31 = M31[i]/(i^2+1),
// QM31 = CM31[u]/(u^2 - 2 - i), matching crates/stwo/src/core/fields/{m31,cm31,qm31}.rs.
// All results are canonical (in [0, P)), which is what the Merkle leaves hash.
#pragma once
#include <cstdint>

namespace cs {

constexpr uint32_t P = 0x7fffffffu;

__host__ __device__ __forceinline__ uint32_t m31_reduce_once(uint32_t s) {
  // s < 2P -> s mod P. Unsigned min picks s - P when s >= P (else s - P wraps high).
  uint32_t t = s - P;
  return t < s ? t : s;
}
__host__ __device__ __forceinline__ uint32_t m31_add(uint32_t a, uint32_t b) { return m31_reduce_once(a + b); }
__host__ __device__ __forceinline__ uint32_t m31_sub(uint32_t a, uint32_t b) { return m31_reduce_once(a + P - b); }
__host__ __device__ __forceinline__ uint32_t m31_neg(uint32_t a) { return m31_reduce_once(P - a); }
__host__ __device__ __forceinline__ uint32_t m31_mul(uint32_t a, uint32_t b) {
  // 62-bit product split at bit 31: lo + hi < 2^32, one conditional subtraction.
  uint64_t p = (uint64_t)a * (uint64_t)b;
  uint32_t lo = (uint32_t)p & P;
  uint32_t hi = (uint32_t)(p >> 31);
  return m31_reduce_once(lo + hi);
}
__host__ __device__ __forceinline__ uint32_t m31_sqr(uint32_t a) { return m31_mul(a, a); }
__host__ __device__ __forceinline__ uint32_t m31_pow(uint32_t a, uint32_t e) {
  uint32_t r = 1;
  while (e) {
    if (e & 1) r = m31_mul(r, a);
    a = m31_sqr(a);
    e >>= 1;
  }
  return r;
}
__host__ __device__ __forceinline__ uint32_t m31_sqn(uint32_t a, int n) {
  for (int i = 0; i < n; i++) a = m31_sqr(a);
  return a;
}
// a^(P - 2) (Fermat) by an addition chain on x^(2^k - 1): P - 2 = 4 (2^29 - 1) + 1, 30 squarings and
// 8 multiplications.
__host__ __device__ __forceinline__ uint32_t m31_inv(uint32_t a) {
  const uint32_t t2 = m31_mul(m31_sqr(a), a);            // 2^2 - 1
  const uint32_t t4 = m31_mul(m31_sqn(t2, 2), t2);       // 2^4 - 1
  const uint32_t t8 = m31_mul(m31_sqn(t4, 4), t4);       // 2^8 - 1
  const uint32_t t16 = m31_mul(m31_sqn(t8, 8), t8);      // 2^16 - 1
  const uint32_t t24 = m31_mul(m31_sqn(t16, 8), t8);     // 2^24 - 1
  const uint32_t t28 = m31_mul(m31_sqn(t24, 4), t4);     // 2^28 - 1
  const uint32_t t29 = m31_mul(m31_sqr(t28), a);         // 2^29 - 1
  return m31_mul(m31_sqn(t29, 2), a);                    // 4 (2^29 - 1) + 1
}

struct cm31 {
  uint32_t a, b;
};
struct qm31 {
  cm31 a, b;
};

__host__ __device__ __forceinline__ cm31 cm31_add(cm31 x, cm31 y) { return {m31_add(x.a, y.a), m31_add(x.b, y.b)}; }
__host__ __device__ __forceinline__ cm31 cm31_sub(cm31 x, cm31 y) { return {m31_sub(x.a, y.a), m31_sub(x.b, y.b)}; }
__host__ __device__ __forceinline__ cm31 cm31_neg(cm31 x) { return {m31_neg(x.a), m31_neg(x.b)}; }
__host__ __device__ __forceinline__ cm31 cm31_mul(cm31 x, cm31 y) {
  return {m31_sub(m31_mul(x.a, y.a), m31_mul(x.b, y.b)), m31_add(m31_mul(x.a, y.b), m31_mul(x.b, y.a))};
}
__host__ __device__ __forceinline__ cm31 cm31_mul_m31(cm31 x, uint32_t y) { return {m31_mul(x.a, y), m31_mul(x.b, y)}; }
__host__ __device__ __forceinline__ cm31 cm31_inv(cm31 x) {
  uint32_t d = m31_inv(m31_add(m31_sqr(x.a), m31_sqr(x.b)));
  return {m31_mul(x.a, d), m31_mul(m31_neg(x.b), d)};
}

__host__ __device__ __forceinline__ qm31 qm31_make(uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
  return {{a, b}, {c, d}};
}
__host__ __device__ __forceinline__ qm31 qm31_add(qm31 x, qm31 y) { return {cm31_add(x.a, y.a), cm31_add(x.b, y.b)}; }
__host__ __device__ __forceinline__ qm31 qm31_sub(qm31 x, qm31 y) { return {cm31_sub(x.a, y.a), cm31_sub(x.b, y.b)}; }
__host__ __device__ __forceinline__ qm31 qm31_neg(qm31 x) { return {cm31_neg(x.a), cm31_neg(x.b)}; }
__host__ __device__ __forceinline__ qm31 qm31_mul(qm31 x, qm31 y) {
  // (a + b u)(c + d u) = (ac + (2+i) bd) + (ad + bc) u
  cm31 bd = cm31_mul(x.b, y.b);
  // (2+i)(p+qi) = (2p - q) + (p + 2q) i
  cm31 rbd = {m31_sub(m31_add(bd.a, bd.a), bd.b), m31_add(bd.a, m31_add(bd.b, bd.b))};
  return {cm31_add(cm31_mul(x.a, y.a), rbd), cm31_add(cm31_mul(x.a, y.b), cm31_mul(x.b, y.a))};
}
__host__ __device__ __forceinline__ qm31 qm31_mul_m31(qm31 x, uint32_t y) {
  return {cm31_mul_m31(x.a, y), cm31_mul_m31(x.b, y)};
}
__host__ __device__ __forceinline__ qm31 qm31_mul_cm31(qm31 x, cm31 y) { return {cm31_mul(x.a, y), cm31_mul(x.b, y)}; }
__host__ __device__ __forceinline__ qm31 qm31_add_m31(qm31 x, uint32_t y) { return {{m31_add(x.a.a, y), x.a.b}, x.b}; }
__host__ __device__ __forceinline__ qm31 qm31_inv(qm31 x) {
  cm31 b2 = cm31_mul(x.b, x.b);
  cm31 ib2 = {m31_neg(b2.b), b2.a};
  cm31 denom = cm31_sub(cm31_mul(x.a, x.a), cm31_add(cm31_add(b2, b2), ib2));
  cm31 di = cm31_inv(denom);
  return {cm31_mul(x.a, di), cm31_mul(cm31_neg(x.b), di)};
}

// x * c for a QM31 c fixed across many products (a folding challenge, a random coefficient):
// with x = (a0 + a1 i) + (a2 + a3 i) u, coordinate r of the product is sum_j a_j k[r][j] for a
// table k built once from c (the rows expand (A + B u)(C + D u) = AC + (2 + i) BD + (AD + BC) u).
// Four 64-bit multiply-accumulates of canonical words stay below 2^64 and are reduced once, so
// the canonical product equals qm31_mul's.
struct qm31_const {
  uint32_t k[4][4];
};
__host__ __device__ inline qm31_const qm31_const_of(qm31 c) {
  const uint32_t b0 = c.a.a, b1 = c.a.b, b2 = c.b.a, b3 = c.b.b;
  const uint32_t two_b2_b3 = m31_sub(m31_add(b2, b2), b3), b2_two_b3 = m31_add(b2, m31_add(b3, b3));
  qm31_const t;
  const uint32_t rows[4][4] = {{b0, m31_neg(b1), two_b2_b3, m31_neg(b2_two_b3)},
                               {b1, b0, b2_two_b3, two_b2_b3},
                               {b2, m31_neg(b3), b0, m31_neg(b1)},
                               {b3, b2, b1, b0}};
  for (int r = 0; r < 4; r++)
    for (int j = 0; j < 4; j++) t.k[r][j] = rows[r][j];
  return t;
}
// x mod P for any 64-bit x (2^31 = 1 mod P, folded twice).
__host__ __device__ __forceinline__ uint32_t m31_reduce64(uint64_t x) {
  const uint64_t y = (x & P) + (x >> 31);                       // < 2^33 + 2^31
  return m31_reduce_once((uint32_t)(y & P) + (uint32_t)(y >> 31));  // < 2^31 + 5
}
__host__ __device__ __forceinline__ qm31 qm31_mul_const(qm31 x, const qm31_const& c) {
  const uint32_t a[4] = {x.a.a, x.a.b, x.b.a, x.b.b};
  uint32_t r[4];
#pragma unroll
  for (int i = 0; i < 4; i++) {
    uint64_t acc = (uint64_t)a[0] * c.k[i][0];
#pragma unroll
    for (int j = 1; j < 4; j++) acc += (uint64_t)a[j] * c.k[i][j];
    r[i] = m31_reduce64(acc);
  }
  return qm31_make(r[0], r[1], r[2], r[3]);
}

// Circle group over M31: (x1,y1)+(x2,y2) = (x1x2 - y1y2, x1y2 + y1x2).
struct cpoint {
  uint32_t x, y;
};
__host__ __device__ __forceinline__ cpoint cpoint_add(cpoint p, cpoint q) {
  return {m31_sub(m31_mul(p.x, q.x), m31_mul(p.y, q.y)), m31_add(m31_mul(p.x, q.y), m31_mul(p.y, q.x))};
}

}  // namespace cs
