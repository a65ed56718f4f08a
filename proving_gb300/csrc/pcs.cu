// Accumulation, DEEP quotients and out-of-domain sampling on sm_103a.
//
//  - accumulate / lift_and_accumulate: crates/stwo/src/prover/backend/cpu/accumulation.rs:9-47
//  - barycentric weights / eval: crates/stwo/src/prover/backend/cpu/circle.rs:100-140
//  - eval_at_point on coefficients: cpu/circle.rs:81-98 with fold (crates/stwo/src/core/poly/utils.rs:27-38)
//  - accumulate_numerators: crates/stwo/src/prover/backend/cpu/quotients.rs:23-49
//  - quotients on the evaluation subdomain: cpu/quotients.rs:51-81 with
//    denominator_inverses (crates/stwo/src/core/pcs/quotients.rs:233-256)
//  - decompose: crates/stwo/src/prover/backend/cpu/fri.rs:39-61,134-145
//
// All field arithmetic is exact, so any evaluation order gives the
// reference's values. Two identities keep the kernels cheap:
//  * coset_vanishing(CanonicCoset(k).coset, q) = pi^(k-1)(q.x): the coset's
//    initial point and its half step cancel (constraints.rs:12-34), so the
//    barycentric derivative term is 4^(l-1) * prod_{k<l} pi^(k-1)(x_i).
//  * sums of M31 products are accumulated in 64 bits and reduced once.
#include <algorithm>
#include <vector>

#include "common.cuh"
#include "field.cuh"
#include "pcs.cuh"

namespace cs {

namespace {

__host__ __device__ __forceinline__ uint32_t reduce64(uint64_t v) {
  // v < 2^62: v mod P by folding at bit 31 twice
  uint64_t t = (v & P) + (v >> 31);
  uint32_t u = (uint32_t)((t & P) + (t >> 31));
  return m31_reduce_once(u);
}

struct SoA {
  uint32_t* c[4];
};
struct CSoA {
  const uint32_t* c[4];
};

__device__ __forceinline__ qm31 ld(const CSoA& a, uint32_t i) {
  return qm31_make(a.c[0][i], a.c[1][i], a.c[2][i], a.c[3][i]);
}
__device__ __forceinline__ qm31 ld(const SoA& a, uint32_t i) {
  return qm31_make(a.c[0][i], a.c[1][i], a.c[2][i], a.c[3][i]);
}
__device__ __forceinline__ void st(const SoA& a, uint32_t i, qm31 v) {
  a.c[0][i] = v.a.a;
  a.c[1][i] = v.a.b;
  a.c[2][i] = v.b.a;
  a.c[3][i] = v.b.b;
}

uint32_t grid_for(uint64_t n, uint32_t threads) {
  return (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>((n + threads - 1) / threads, 152 * 16));
}

// ---------------------------------------------------------------- accumulation

__global__ void accumulate_kernel(SoA col, CSoA other, uint32_t n) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    st(col, i, qm31_add(ld(col, i), ld(other, i)));
}

// col[i] += prev[(i >> (log_ratio + 1) << 1) + (i & 1)]; prev == nullptr means zeros.
__global__ void lift_add_kernel(SoA col, CSoA prev, bool has_prev, uint32_t log_n, uint32_t log_ratio) {
  const uint32_t n = 1u << log_n;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (!has_prev) continue;
    const uint32_t j = ((i >> (log_ratio + 1)) << 1) + (i & 1);
    st(col, i, qm31_add(ld(col, i), ld(prev, j)));
  }
}

// ---------------------------------------------------------------- barycentric

// Copies a domain's point tables into shared memory (all threads of the block).
__device__ __forceinline__ void stage_tables(const DomainTables& d, cpoint (*tab)[512]) {
  for (uint32_t i = threadIdx.x; i < 3 * 512; i += blockDim.x) tab[i >> 9][i & 511] = d.t[i >> 9][i & 511];
  __syncthreads();
}

// Point jj (< 2^27) of the first half of the tables' domain: two additions.
__device__ __forceinline__ cpoint table_point(const cpoint (*tab)[512], uint32_t jj) {
  return cpoint_add(cpoint_add(tab[0][jj & 511], tab[1][(jj >> 9) & 511]), tab[2][(jj >> 18) & 511]);
}

// Domain point j of the first half of CanonicCoset(log_n)'s circle domain is init + j step; with
// j = j0 + 2^9 j1 + 2^18 j2, it is T0[j0] + T1[j1] + T2[j2] (T0 holding init + j0 step), two point
// additions from tables staged in shared memory. The second half is the conjugate (x, -y) of the
// first: index -(init + (j - n/2) step).
struct BaryParams {
  DomainTables tables;
  uint32_t log_n;
  qm31 px, py, vn_p;  // sample point and V_n(p) = pi^(log_n - 1)(p.x)
  uint32_t si_plus;   // 2^log_n, the denominator factor of the points whose 2^(n-1) multiple is (0, -1)
  uint32_t half_init, half_step;  // index of the first point and index step of the first half
};

__global__ void bary_weights_kernel(const __grid_constant__ BaryParams p, SoA out) {
  __shared__ cpoint tab[3][512];
  stage_tables(p.tables, tab);
  const uint32_t n = 1u << p.log_n, hs = n >> 1;
  const uint32_t quarter = 3u << 29;  // index of (0, 1)
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t j = __brev(i) >> (32 - p.log_n);
    const bool second = j >= hs;
    const uint32_t jj = second ? j - hs : j;
    cpoint xi = table_point(tab, jj);
    uint32_t idx = (p.half_init + jj * p.half_step) & 0x7fffffffu;
    if (second) {
      xi.y = m31_neg(xi.y);
      idx = (0u - idx) & 0x7fffffffu;
    }
    // si = -2 y_i 4^(l-1) prod_{k=1}^{l-1} pi^(k-1)(x_i) = -2 y_i V'(x_i) = -2^l y(2^(l-1) x_i), and
    // 2^(l-1) x_i is (0, 1) or (0, -1) (V(x_i) = 0)
    const uint32_t si = ((idx << (p.log_n - 1)) & 0x7fffffffu) == quarter ? m31_neg(p.si_plus) : p.si_plus;
    // h = p - x_i = (px*x + py*y, py*x - px*y)
    const qm31 hx = qm31_add(qm31_mul_m31(p.px, xi.x), qm31_mul_m31(p.py, xi.y));
    const qm31 hy = qm31_sub(qm31_mul_m31(p.py, xi.x), qm31_mul_m31(p.px, xi.y));
    // W = V_n(p) * (1 + h.x) / (h.y * si)
    const qm31 num = qm31_mul(p.vn_p, qm31_add_m31(hx, 1));
    const qm31 den = qm31_mul_m31(hy, si);
    st(out, i, qm31_mul(num, qm31_inv(den)));
  }
}

// ---------------------------------------------------------------- reductions

__device__ __forceinline__ void block_reduce_u64x4(uint64_t acc[4], uint64_t* sh /* 4 * warps */) {
#pragma unroll
  for (int k = 0; k < 4; k++)
    for (int o = 16; o > 0; o >>= 1) acc[k] += __shfl_down_sync(0xffffffffu, acc[k], o);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0)
    for (int k = 0; k < 4; k++) sh[4 * warp + k] = acc[k];
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    for (int k = 0; k < 4; k++) acc[k] = lane < nw ? sh[4 * lane + k] : 0;
#pragma unroll
    for (int k = 0; k < 4; k++)
      for (int o = 16; o > 0; o >>= 1) acc[k] += __shfl_down_sync(0xffffffffu, acc[k], o);
  }
}

// Many columns at once: block (x, y) takes rows [2048 x, 2048 (x + 1)) of the 16 columns of group
// y. Each thread keeps the weights of its 8 rows in registers, loads the rows of the next two columns
// while it works on the current one, and adds the unreduced 64-bit products (folding below 2^34 after
// the first 4 of its 8 rows: 4 products below P^2 < 2^62 on top of a folded value stay below 2^64). A warp reduces the four coordinates of a column at once (a butterfly that halves the
// values per lane at each of the first two steps: 6 shuffles), writes them to shared memory, and the
// block sums its warps for all its columns after one barrier. The per-column partial sums (below
// 2^34) go to `partial`, one row of chunks per (column, coordinate), which bary_final_kernel sums
// with one warp per row (at most 2^19 chunks: below 2^53).
constexpr int kBaryThreads = 256;
constexpr int kBaryRows = 8;  // rows per thread
constexpr int kBaryChunk = kBaryThreads * kBaryRows;
constexpr int kBaryGroup = 16;  // columns per block

__device__ __forceinline__ uint64_t fold34(uint64_t v) { return (v & P) + (v >> 31); }

// acc + a * b with the 64-bit addend in the multiply (mad.wide.u32).
__device__ __forceinline__ uint64_t mad_wide(uint32_t a, uint32_t b, uint64_t acc) {
  uint64_t d;
  asm("mad.wide.u32 %0, %1, %2, %3;" : "=l"(d) : "r"(a), "r"(b), "l"(acc));
  return d;
}

// The warp's sum of r[0..3] (each below P) for coordinate lane >> 3, in lanes 0, 8, 16, 24.
__device__ __forceinline__ uint32_t warp_sum4(const uint32_t r[4], uint32_t lane) {
  const bool hi = (lane >> 4) & 1;  // keeps coordinates 2, 3
  uint32_t k0 = hi ? r[2] : r[0], k1 = hi ? r[3] : r[1];
  const uint32_t s0 = hi ? r[0] : r[2], s1 = hi ? r[1] : r[3];
  k0 = m31_add(k0, __shfl_xor_sync(0xffffffffu, s0, 16));
  k1 = m31_add(k1, __shfl_xor_sync(0xffffffffu, s1, 16));
  const bool odd = (lane >> 3) & 1;  // keeps the second of its pair
  uint32_t v = odd ? k1 : k0;
  v = m31_add(v, __shfl_xor_sync(0xffffffffu, odd ? k0 : k1, 8));
#pragma unroll
  for (int o = 4; o > 0; o >>= 1) v = m31_add(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

__global__ void __launch_bounds__(kBaryThreads, 3) bary_partial_kernel(const BaryColumns cols, uint32_t nb,
                                                                   uint32_t log_n, CSoA w,
                                                                   unsigned long long* partial) {
  __shared__ uint32_t sh[kBaryGroup][kBaryThreads / 32][4];
  const uint32_t n = 1u << log_n;
  const uint32_t base = blockIdx.x * kBaryChunk;
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint32_t wr[kBaryRows][4];
#pragma unroll
  for (int j = 0; j < kBaryRows; j++) {
    const uint32_t row = base + threadIdx.x + j * kBaryThreads;
#pragma unroll
    for (int k = 0; k < 4; k++) wr[j][k] = row < n ? __ldg(w.c[k] + row) : 0;
  }
  const uint32_t c0 = blockIdx.y * kBaryGroup;
  const uint32_t c1 = min(nb, c0 + kBaryGroup);
  // rows of the current column and of the next two, loaded ahead
  uint32_t x[kBaryRows], xn[kBaryRows], xnn[kBaryRows];
#pragma unroll
  for (int j = 0; j < kBaryRows; j++) {
    const uint32_t row = base + threadIdx.x + j * kBaryThreads;
    x[j] = row < n ? __ldg(cols.ptr[c0] + row) : 0;
    xn[j] = (row < n && c0 + 1 < c1) ? __ldg(cols.ptr[c0 + 1] + row) : 0;
  }
  for (uint32_t col = c0; col < c1; col++) {
    const uint32_t* vnn = cols.ptr[col + 2 < c1 ? col + 2 : col];
#pragma unroll
    for (int j = 0; j < kBaryRows; j++) {
      const uint32_t row = base + threadIdx.x + j * kBaryThreads;
      xnn[j] = (row < n && col + 2 < c1) ? __ldg(vnn + row) : 0;
    }
    uint64_t acc[4] = {0, 0, 0, 0};
#pragma unroll
    for (int j = 0; j < kBaryRows; j++) {
#pragma unroll
      for (int k = 0; k < 4; k++) {
        acc[k] = mad_wide(wr[j][k], x[j], acc[k]);
        if (j == 3) acc[k] = fold34(acc[k]);
      }
    }
    uint32_t r[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const uint64_t f = fold34(acc[k]);  // below 2^34
      r[k] = m31_reduce_once((uint32_t)fold34(f));
    }
    const uint32_t v = warp_sum4(r, lane);
    if ((lane & 7) == 0) sh[col - c0][warp][lane >> 3] = v;
#pragma unroll
    for (int j = 0; j < kBaryRows; j++) {
      x[j] = xn[j];
      xn[j] = xnn[j];
    }
  }
  __syncthreads();
  const uint32_t t = threadIdx.x;
  if (t < (c1 - c0) * 4) {
    const uint32_t ci = t >> 2, k = t & 3;
    uint64_t sum = 0;
#pragma unroll
    for (int q = 0; q < kBaryThreads / 32; q++) sum += sh[ci][q][k];
    partial[((size_t)(c0 + ci) * 4 + k) * gridDim.x + blockIdx.x] = sum;
  }
}

// One warp per (column, coordinate): its row of per-chunk partial sums, strided over the lanes.
__global__ void bary_final_kernel(const unsigned long long* partial, uint32_t n_chunks, uint32_t nb, uint32_t* out) {
  const uint32_t row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const uint32_t lane = threadIdx.x & 31;
  if (row >= nb * 4) return;  // whole warps leave together
  const unsigned long long* p = partial + (size_t)row * n_chunks;
  uint64_t t = 0;
  for (uint32_t ch = lane; ch < n_chunks; ch += 32) t += p[ch];
  for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
  if (lane == 0) out[row] = reduce64(t % P);
}

// ---------------------------------------------------------------- eval_at_point

struct FoldFactors {
  qm31 f[32];  // f[0] = y, f[1] = x, f[j] = pi^(j-1)(x)
  uint32_t log_n;
};

// One block per column. A warp folds a 256-coefficient chunk against the
// table T[m] = prod_{bits j of m} f[j] (m < 256), then scales by the chunk's
// high factor prod_{bits j of h} f[8 + j].
__global__ void eval_at_point_kernel(const BaryColumns cols, const FoldFactors ff, uint32_t* out) {
  __shared__ qm31 T[256];
  __shared__ qm31 warp_acc[32];
  const uint32_t log_n = ff.log_n;
  const uint32_t* c = cols.ptr[blockIdx.x];
  const uint32_t low = min(log_n, 8u);
  const uint32_t tsize = 1u << low;
  for (uint32_t m = threadIdx.x; m < tsize; m += blockDim.x) {
    qm31 b = qm31_make(1, 0, 0, 0);
    for (uint32_t j = 0; j < low; j++)
      if ((m >> j) & 1) b = qm31_mul(b, ff.f[j]);
    T[m] = b;
  }
  __syncthreads();
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const uint32_t n_chunks = 1u << (log_n - low);
  qm31 wacc = qm31_make(0, 0, 0, 0);
  for (uint32_t h = warp; h < n_chunks; h += nw) {
    uint64_t a[4] = {0, 0, 0, 0};
    for (uint32_t m = lane; m < tsize; m += 32) {
      const uint32_t x = __ldg(c + ((size_t)h << low) + m);
      const qm31 t = T[m];
      a[0] += m31_mul(t.a.a, x);
      a[1] += m31_mul(t.a.b, x);
      a[2] += m31_mul(t.b.a, x);
      a[3] += m31_mul(t.b.b, x);
    }
#pragma unroll
    for (int k = 0; k < 4; k++)
      for (int o = 16; o > 0; o >>= 1) a[k] += __shfl_down_sync(0xffffffffu, a[k], o);
    if (lane == 0) {
      qm31 s = qm31_make(reduce64(a[0] % P), reduce64(a[1] % P), reduce64(a[2] % P), reduce64(a[3] % P));
      for (uint32_t j = 0; (h >> j) != 0; j++)
        if ((h >> j) & 1) s = qm31_mul(s, ff.f[low + j]);
      wacc = qm31_add(wacc, s);
    }
  }
  if (lane == 0) warp_acc[warp] = wacc;
  __syncthreads();
  if (threadIdx.x == 0) {
    qm31 r = qm31_make(0, 0, 0, 0);
    for (uint32_t k = 0; k < nw; k++) r = qm31_add(r, warp_acc[k]);
    out[4 * blockIdx.x + 0] = r.a.a;
    out[4 * blockIdx.x + 1] = r.a.b;
    out[4 * blockIdx.x + 2] = r.b.a;
    out[4 * blockIdx.x + 3] = r.b.b;
  }
}

// ---------------------------------------------------------------- numerators

// row r: sum_t c_t * col_t[r] - sum_t b_t (the batch's partial numerator). Terms go in groups of 8:
// the 8 column values are loaded first, then their unreduced 64-bit products are added, folded below
// 2^34 after every 4 (4 products below P^2 < 2^62 on top of a folded value stay below 2^64).
__global__ void numerators_kernel(const NumeratorTerms terms, uint32_t rows, SoA out, bool accumulate) {
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += gridDim.x * blockDim.x) {
    uint64_t a[4] = {0, 0, 0, 0};
    uint32_t t = 0;
    for (; t + 8 <= terms.n; t += 8) {
      uint32_t v[8];
#pragma unroll
      for (int u = 0; u < 8; u++) v[u] = __ldg(terms.col[t + u] + r);
#pragma unroll
      for (int u = 0; u < 8; u++) {
        const qm31 c = terms.c[t + u];
        a[0] += (uint64_t)c.a.a * v[u];
        a[1] += (uint64_t)c.a.b * v[u];
        a[2] += (uint64_t)c.b.a * v[u];
        a[3] += (uint64_t)c.b.b * v[u];
        if (u == 3 || u == 7) {
#pragma unroll
          for (int k = 0; k < 4; k++) a[k] = fold34(a[k]);
        }
      }
    }
    for (; t < terms.n; t++) {
      const uint32_t v = __ldg(terms.col[t] + r);
      const qm31 c = terms.c[t];
      a[0] = fold34(a[0] + (uint64_t)c.a.a * v);
      a[1] = fold34(a[1] + (uint64_t)c.a.b * v);
      a[2] = fold34(a[2] + (uint64_t)c.b.a * v);
      a[3] = fold34(a[3] + (uint64_t)c.b.b * v);
    }
    qm31 s = qm31_make(reduce64(a[0] % P), reduce64(a[1] % P), reduce64(a[2] % P), reduce64(a[3] % P));
    s = qm31_sub(s, terms.b_sum);
    if (accumulate) s = qm31_add(s, ld(out, r));
    st(out, r, s);
  }
}

// ---------------------------------------------------------------- quotients

__global__ void quotients_kernel(const __grid_constant__ QuotientParams q, SoA out) {
  __shared__ cpoint tab[3][512];
  stage_tables(q.tables, tab);
  const uint32_t rows = 1u << q.sub_log, hs = rows >> 1;
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += gridDim.x * blockDim.x) {
    const uint32_t j = __brev(r) >> (32 - q.sub_log);
    cpoint dp = table_point(tab, j < hs ? j : j - hs);
    if (j >= hs) dp.y = m31_neg(dp.y);
    qm31 acc = qm31_make(0, 0, 0, 0);
    for (uint32_t k = 0; k < q.n_points; k++) {
      const qm31 px = q.px[k], py = q.py[k];
      // (prx - x) * piy - (pry - y) * pix in CM31
      const cm31 dx = cm31_sub(px.a, cm31{dp.x, 0}), dy = cm31_sub(py.a, cm31{dp.y, 0});
      const cm31 den = cm31_sub(cm31_mul(dx, py.b), cm31_mul(dy, px.b));
      const cm31 den_inv = cm31_inv(den);
      const uint32_t log_ratio = q.sub_log - q.acc_log[k];
      const uint32_t li = ((r >> (log_ratio + 1)) << 1) + (r & 1);
      const qm31 partial = qm31_make(q.acc[k].c[0][li], q.acc[k].c[1][li], q.acc[k].c[2][li], q.acc[k].c[3][li]);
      const qm31 num = qm31_sub(partial, qm31_mul_m31(q.first_linear[k], dp.y));
      acc = qm31_add(acc, qm31_mul_cm31(num, den_inv));
    }
    st(out, r, acc);
  }
}

// ---------------------------------------------------------------- decompose

__global__ void half_sums_kernel(CSoA in, uint32_t log_n, uint32_t* sums /* 8 words */) {
  __shared__ uint64_t sh[4 * 32];
  const uint32_t half = 1u << (log_n - 1);
  const uint32_t which = blockIdx.x;  // 0: first half, 1: second half
  uint64_t acc[4] = {0, 0, 0, 0};
  for (uint32_t i = threadIdx.x; i < half; i += blockDim.x) {
    const uint32_t idx = which * half + i;
#pragma unroll
    for (int k = 0; k < 4; k++) acc[k] += in.c[k][idx];
  }
  block_reduce_u64x4(acc, sh);
  if (threadIdx.x == 0)
    for (int k = 0; k < 4; k++) sums[4 * which + k] = reduce64(acc[k] % P);
}

__global__ void decompose_apply_kernel(CSoA in, SoA out, uint32_t log_n, qm31 lambda) {
  const uint32_t n = 1u << log_n, half = n >> 1;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    st(out, i, i < half ? qm31_sub(ld(in, i), lambda) : qm31_add(ld(in, i), lambda));
}

}  // namespace

GenPowersTable gen_powers() {
  GenPowersTable t;
  cpoint cur{2u, 1268011823u};
  for (int b = 0; b < 31; b++) {
    t.p[b] = cur;
    cur = cpoint_add(cur, cur);
  }
  return t;
}

void fill_domain_tables(DomainTables& d, uint32_t half_init, uint32_t half_step) {
  static const GenPowersTable g = gen_powers();
  const auto point_at_host = [&](uint32_t idx) {
    cpoint r{1, 0};
    for (int b = 0; b < 31; b++)
      if ((idx >> b) & 1) r = cpoint_add(r, g.p[b]);
    return r;
  };
  for (uint32_t t = 0; t < 3; t++) {
    // T0[a] = init + a step, T1[a] = 2^9 a step, T2[a] = 2^18 a step, one addition per entry
    const cpoint step = point_at_host(((1u << (9 * t)) * half_step) & 0x7fffffffu);
    d.t[t][0] = t == 0 ? point_at_host(half_init) : cpoint{1, 0};
    for (uint32_t a = 1; a < 512; a++) d.t[t][a] = cpoint_add(d.t[t][a - 1], step);
  }
}

cs_status quotients_on_subdomain(const QuotientParams& q, uint32_t* const out[4], cudaStream_t st) {
  SoA o;
  for (int k = 0; k < 4; k++) o.c[k] = out[k];
  const uint32_t rows = 1u << q.sub_log;
  quotients_kernel<<<grid_for(rows, 256), 256, 0, st>>>(q, o);
  CS_LAUNCHED("quotients_kernel");
  return CS_OK;
}

}  // namespace cs

using namespace cs;

static cs_status check4(const uint32_t* const p[4], const char* what) {
  CS_CHECK_ARG(p != nullptr, "%s: null coordinate table", what);
  for (int k = 0; k < 4; k++) CS_CHECK_ARG(p[k] != nullptr, "%s: coordinate %d is null", what, k);
  return CS_OK;
}

extern "C" cs_status cs_accumulate(uint32_t* const h_col[4], const uint32_t* const h_other[4], uint32_t log_size,
                                   cs_stream stream) {
  cs_status s = check4(h_col, "accumulate");
  if (s == CS_OK) s = check4(h_other, "accumulate");
  if (s != CS_OK) return s;
  CS_CHECK_ARG(log_size <= 30, "accumulate: log size %u too large", log_size);
  SoA c;
  CSoA o;
  for (int k = 0; k < 4; k++) {
    c.c[k] = h_col[k];
    o.c[k] = h_other[k];
  }
  const uint32_t n = 1u << log_size;
  accumulate_kernel<<<grid_for(n, 256), 256, 0, to_stream(stream)>>>(c, o, n);
  CS_LAUNCHED("accumulate_kernel");
  return CS_OK;
}

extern "C" cs_status cs_generate_secure_powers(const uint32_t felt[4], uint32_t n_powers, uint32_t* h_out) {
  CS_CHECK_ARG(felt != nullptr && (n_powers == 0 || h_out != nullptr), "generate_secure_powers: null pointer");
  const qm31 f = qm31_make(felt[0], felt[1], felt[2], felt[3]);
  qm31 acc = qm31_make(1, 0, 0, 0);
  for (uint32_t i = 0; i < n_powers; i++) {
    h_out[4 * i] = acc.a.a;
    h_out[4 * i + 1] = acc.a.b;
    h_out[4 * i + 2] = acc.b.a;
    h_out[4 * i + 3] = acc.b.b;
    acc = qm31_mul(acc, f);
  }
  return CS_OK;
}

extern "C" cs_status cs_lift_and_accumulate(uint32_t* const* h_cols, const uint32_t* h_log_sizes, uint32_t n_cols,
                                            cs_stream stream) {
  CS_CHECK_ARG(n_cols == 0 || (h_cols != nullptr && h_log_sizes != nullptr), "lift_and_accumulate: null table");
  uint32_t prev_log = 1;
  for (uint32_t k = 0; k < n_cols; k++) {
    const uint32_t l = h_log_sizes[k];
    CS_CHECK_ARG(l >= 1 && l <= 30, "lift_and_accumulate: column %u has log size %u", k, l);
    CS_CHECK_ARG(k == 0 ? l >= 1 : l > prev_log, "lift_and_accumulate: sizes must be strictly increasing (column %u)",
                 k);
    for (int c = 0; c < 4; c++) CS_CHECK_ARG(h_cols[4 * k + c] != nullptr, "lift_and_accumulate: null column");
    prev_log = l;
  }
  prev_log = 1;
  for (uint32_t k = 0; k < n_cols; k++) {
    const uint32_t l = h_log_sizes[k];
    if (k == 0) {
      prev_log = l;  // lifting zeros adds nothing
      continue;
    }
    SoA col;
    CSoA prev;
    for (int c = 0; c < 4; c++) {
      col.c[c] = h_cols[4 * k + c];
      prev.c[c] = h_cols[4 * (k - 1) + c];
    }
    lift_add_kernel<<<grid_for(1u << l, 256), 256, 0, to_stream(stream)>>>(col, prev, true, l, l - prev_log);
    CS_LAUNCHED("lift_add_kernel");
    prev_log = l;
  }
  return CS_OK;
}

extern "C" cs_status cs_barycentric_weights(uint32_t log_size, const uint32_t px[4], const uint32_t py[4],
                                            uint32_t* const h_out[4], cs_stream stream) {
  CS_CHECK_ARG(px != nullptr && py != nullptr, "barycentric_weights: null point");
  cs_status s = check4(h_out, "barycentric_weights");
  if (s != CS_OK) return s;
  CS_CHECK_ARG(log_size >= 1 && log_size <= 28, "barycentric_weights: log size %u out of range", log_size);
  static thread_local BaryParams p;
  p.half_init = subgroup_gen(log_size + 1);
  p.half_step = log_size >= 2 ? subgroup_gen(log_size - 1) : 0;
  p.log_n = log_size;
  fill_domain_tables(p.tables, p.half_init, p.half_step);
  p.si_plus = 1u << log_size;
  p.px = qm31_make(px[0], px[1], px[2], px[3]);
  p.py = qm31_make(py[0], py[1], py[2], py[3]);
  qm31 x = p.px;
  for (uint32_t i = 1; i < log_size; i++) {
    const qm31 sq = qm31_mul(x, x);
    x = qm31_sub(qm31_add(sq, sq), qm31_make(1, 0, 0, 0));
  }
  p.vn_p = x;
  SoA o;
  for (int k = 0; k < 4; k++) o.c[k] = h_out[k];
  bary_weights_kernel<<<grid_for(1u << log_size, 256), 256, 0, to_stream(stream)>>>(p, o);
  CS_LAUNCHED("bary_weights_kernel");
  return CS_OK;
}

extern "C" cs_status cs_barycentric_eval(const uint32_t* const* h_cols, uint32_t n_cols, uint32_t log_size,
                                         const uint32_t* const h_weights[4], uint32_t* d_out, cs_stream stream) {
  cs_status s = check4(h_weights, "barycentric_eval");
  if (s != CS_OK) return s;
  CS_CHECK_ARG(n_cols == 0 || (h_cols != nullptr && d_out != nullptr), "barycentric_eval: null pointer");
  CS_CHECK_ARG(log_size <= 30, "barycentric_eval: log size %u too large", log_size);
  CSoA w;
  for (int k = 0; k < 4; k++) w.c[k] = h_weights[k];
  for (uint32_t b0 = 0; b0 < n_cols; b0 += kMaxBatch) {
    const uint32_t nb = std::min<uint32_t>(kMaxBatch, n_cols - b0);
    BaryColumns cols;
    for (uint32_t i = 0; i < nb; i++) {
      CS_CHECK_ARG(h_cols[b0 + i] != nullptr, "barycentric_eval: column %u is null", b0 + i);
      cols.ptr[i] = h_cols[b0 + i];
    }
    const uint32_t n_chunks = ((1u << log_size) + kBaryChunk - 1) / kBaryChunk;
    cudaStream_t st = to_stream(stream);
    unsigned long long* partial = nullptr;
    CS_CUDA(stream_alloc(reinterpret_cast<void**>(&partial), sizeof(unsigned long long) * 4 * nb * n_chunks, st));
    bary_partial_kernel<<<dim3(n_chunks, (nb + kBaryGroup - 1) / kBaryGroup), kBaryThreads, 0, st>>>(
        cols, nb, log_size, w, partial);
    note_launch();
    bary_final_kernel<<<(4 * nb + 7) / 8, 256, 0, st>>>(partial, n_chunks, nb, d_out + 4 * b0);
    note_launch();
    cudaError_t e = cudaGetLastError();
    const cudaError_t ef = cudaFreeAsync(partial, st);
    if (e == cudaSuccess) e = ef;
    if (e != cudaSuccess) return from_cuda(e, "barycentric_eval");
  }
  return CS_OK;
}

extern "C" cs_status cs_eval_at_point(const uint32_t* const* h_coeffs, uint32_t n_cols, uint32_t log_size,
                                      const uint32_t px[4], const uint32_t py[4], uint32_t* d_out, cs_stream stream) {
  CS_CHECK_ARG(px != nullptr && py != nullptr, "eval_at_point: null point");
  CS_CHECK_ARG(n_cols == 0 || (h_coeffs != nullptr && d_out != nullptr), "eval_at_point: null pointer");
  CS_CHECK_ARG(log_size <= 30, "eval_at_point: log size %u too large", log_size);
  FoldFactors ff;
  ff.log_n = log_size;
  // mappings: y, x, pi(x), pi^2(x), ... (cpu/circle.rs:89-95)
  ff.f[0] = qm31_make(py[0], py[1], py[2], py[3]);
  qm31 x = qm31_make(px[0], px[1], px[2], px[3]);
  for (uint32_t j = 1; j < 32; j++) {
    ff.f[j] = x;
    const qm31 sq = qm31_mul(x, x);
    x = qm31_sub(qm31_add(sq, sq), qm31_make(1, 0, 0, 0));
  }
  for (uint32_t b0 = 0; b0 < n_cols; b0 += kMaxBatch) {
    const uint32_t nb = std::min<uint32_t>(kMaxBatch, n_cols - b0);
    BaryColumns cols;
    for (uint32_t i = 0; i < nb; i++) {
      CS_CHECK_ARG(h_coeffs[b0 + i] != nullptr, "eval_at_point: column %u is null", b0 + i);
      cols.ptr[i] = h_coeffs[b0 + i];
    }
    eval_at_point_kernel<<<nb, 256, 0, to_stream(stream)>>>(cols, ff, d_out + 4 * b0);
    CS_LAUNCHED("eval_at_point_kernel");
  }
  return CS_OK;
}

extern "C" cs_status cs_accumulate_numerators(const uint32_t* const* h_cols, uint32_t n_terms, uint32_t log_size,
                                              uint32_t log_blowup, const uint32_t* h_coeffs,
                                              uint32_t* const h_out[4], uint32_t first_linear_out[4],
                                              cs_stream stream) {
  cs_status s = check4(h_out, "accumulate_numerators");
  if (s != CS_OK) return s;
  CS_CHECK_ARG(n_terms > 0 && h_cols != nullptr && h_coeffs != nullptr && first_linear_out != nullptr,
               "accumulate_numerators: empty batch or null pointer");
  CS_CHECK_ARG(log_blowup <= log_size && log_size <= 30, "accumulate_numerators: bad sizes %u/%u", log_size,
               log_blowup);
  qm31 sum_a = qm31_make(0, 0, 0, 0);
  for (uint32_t t = 0; t < n_terms; t++) {
    CS_CHECK_ARG(h_cols[t] != nullptr, "accumulate_numerators: column %u is null", t);
    const uint32_t* a = h_coeffs + 12 * t;
    sum_a = qm31_add(sum_a, qm31_make(a[0], a[1], a[2], a[3]));
  }
  first_linear_out[0] = sum_a.a.a;
  first_linear_out[1] = sum_a.a.b;
  first_linear_out[2] = sum_a.b.a;
  first_linear_out[3] = sum_a.b.b;
  SoA o;
  for (int k = 0; k < 4; k++) o.c[k] = h_out[k];
  const uint32_t rows = 1u << (log_size - log_blowup);
  static thread_local NumeratorTerms terms;
  for (uint32_t t0 = 0; t0 < n_terms; t0 += kMaxTerms) {
    const uint32_t nt = std::min<uint32_t>(kMaxTerms, n_terms - t0);
    terms.n = nt;
    qm31 b_sum = qm31_make(0, 0, 0, 0);
    for (uint32_t t = 0; t < nt; t++) {
      const uint32_t* co = h_coeffs + 12 * (t0 + t);
      terms.col[t] = h_cols[t0 + t];
      b_sum = qm31_add(b_sum, qm31_make(co[4], co[5], co[6], co[7]));
      terms.c[t] = qm31_make(co[8], co[9], co[10], co[11]);
    }
    terms.b_sum = b_sum;
    numerators_kernel<<<grid_for(rows, 256), 256, 0, to_stream(stream)>>>(terms, rows, o, t0 > 0);
    CS_LAUNCHED("numerators_kernel");
  }
  return CS_OK;
}

extern "C" cs_status cs_quotients_on_subdomain(const uint32_t* const* h_accs, const uint32_t* h_acc_log_sizes,
                                               uint32_t n_points, const uint32_t* h_points,
                                               const uint32_t* h_first_linear, uint32_t lifting_log_size,
                                               uint32_t log_blowup, uint32_t* const h_out[4], cs_stream stream) {
  cs_status s = check4(h_out, "quotients");
  if (s != CS_OK) return s;
  CS_CHECK_ARG(n_points >= 1 && n_points <= kMaxPoints, "quotients: %u sample points (1..%u supported)", n_points,
               kMaxPoints);
  CS_CHECK_ARG(h_accs && h_acc_log_sizes && h_points && h_first_linear, "quotients: null pointer");
  CS_CHECK_ARG(log_blowup < lifting_log_size && lifting_log_size <= 30, "quotients: bad sizes");
  static thread_local QuotientParams q;
  q.sub_log = lifting_log_size - log_blowup;
  CS_CHECK_ARG(q.sub_log >= 1 && q.sub_log <= 28, "quotients: subdomain log size %u outside [1, 28]", q.sub_log);
  // eval_domain.split(log_blowup).0: half coset (eval half initial, log L - 1 - b)
  q.half_init = subgroup_gen(lifting_log_size + 1);
  q.half_step = q.sub_log >= 2 ? subgroup_gen(q.sub_log - 1) : 0;
  fill_domain_tables(q.tables, q.half_init, q.half_step);
  q.n_points = n_points;
  for (uint32_t k = 0; k < n_points; k++) {
    const uint32_t* pt = h_points + 8 * k;
    q.px[k] = qm31_make(pt[0], pt[1], pt[2], pt[3]);
    q.py[k] = qm31_make(pt[4], pt[5], pt[6], pt[7]);
    const uint32_t* fl = h_first_linear + 4 * k;
    q.first_linear[k] = qm31_make(fl[0], fl[1], fl[2], fl[3]);
    q.acc_log[k] = h_acc_log_sizes[k];
    CS_CHECK_ARG(q.acc_log[k] >= 1 && q.acc_log[k] <= q.sub_log, "quotients: accumulation %u has log size %u", k,
                 q.acc_log[k]);
    for (int c = 0; c < 4; c++) {
      CS_CHECK_ARG(h_accs[4 * k + c] != nullptr, "quotients: null accumulation column");
      q.acc[k].c[c] = h_accs[4 * k + c];
    }
  }
  return quotients_on_subdomain(q, h_out, to_stream(stream));
}

extern "C" cs_status cs_decompose(const uint32_t* const h_src[4], uint32_t log_size, uint32_t* const h_dst[4],
                                  uint32_t lambda_out[4], cs_stream stream) {
  cs_status s = check4(h_src, "decompose");
  if (s == CS_OK) s = check4(h_dst, "decompose");
  if (s != CS_OK) return s;
  CS_CHECK_ARG(lambda_out != nullptr && log_size >= 1 && log_size <= 30, "decompose: bad arguments");
  cudaStream_t st = to_stream(stream);
  CSoA in;
  SoA out;
  for (int k = 0; k < 4; k++) {
    in.c[k] = h_src[k];
    out.c[k] = h_dst[k];
  }
  uint32_t* d_sums = nullptr;
  CS_CUDA(stream_alloc(reinterpret_cast<void**>(&d_sums), 8 * sizeof(uint32_t), st));
  half_sums_kernel<<<2, 512, 0, st>>>(in, log_size, d_sums);
  note_launch();
  uint32_t sums[8];
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(sums, d_sums, sizeof(sums), cudaMemcpyDeviceToHost, st);
  cudaFreeAsync(d_sums, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return from_cuda(e, "decompose");
  const qm31 a = qm31_make(sums[0], sums[1], sums[2], sums[3]);
  const qm31 b = qm31_make(sums[4], sums[5], sums[6], sums[7]);
  // lambda = (a - b) / n, n = 2^log_size, 1/n = 2^(31 - log_size)
  const qm31 lambda = qm31_mul_m31(qm31_sub(a, b), 1u << (31 - log_size));
  lambda_out[0] = lambda.a.a;
  lambda_out[1] = lambda.a.b;
  lambda_out[2] = lambda.b.a;
  lambda_out[3] = lambda.b.b;
  decompose_apply_kernel<<<grid_for(1u << log_size, 256), 256, 0, st>>>(in, out, log_size, lambda);
  CS_LAUNCHED("decompose_apply_kernel");
  return CS_OK;
}
