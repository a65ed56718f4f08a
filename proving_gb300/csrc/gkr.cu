// GKR lookups on the device: the backend's GkrOps and MleOps
// (crates/stwo/src/prover/lookups/gkr_prover.rs:22-42, mle.rs:9-14), giving the
// values of the CPU backend (crates/stwo/src/prover/backend/cpu/lookups/gkr.rs,
// cpu/lookups/mle.rs). A secure column is 4 coordinate columns, a base column
// one. An MLE of n variables holds its 2^n values on the boolean hypercube in
// the reference's order: variable j is index bit n-1-j.
//
// Every kernel is a stream over HBM with a few QM31 products per element; the
// sums of sum_as_poly_in_first_variable are reduced per block and then by one
// block. Field arithmetic is exact, so the order of the sums does not matter.
#include <algorithm>

#include "common.cuh"
#include "field.cuh"

namespace cs {
namespace {

struct QIn {
  const uint32_t* c[4];
};
struct QOut {
  uint32_t* c[4];
};

__device__ __forceinline__ qm31 q_one() { return qm31_make(1, 0, 0, 0); }
__device__ __forceinline__ qm31 q_zero() { return qm31_make(0, 0, 0, 0); }
__device__ __forceinline__ qm31 q_double(qm31 x) { return qm31_add(x, x); }

__device__ __forceinline__ qm31 q_load(const QIn& s, uint32_t i) {
  return qm31_make(s.c[0][i], s.c[1][i], s.c[2][i], s.c[3][i]);
}
__device__ __forceinline__ void q_store(const QOut& d, uint32_t i, qm31 v) {
  d.c[0][i] = v.a.a;
  d.c[1][i] = v.a.b;
  d.c[2][i] = v.b.a;
  d.c[3][i] = v.b.b;
}
// values 2i and 2i + 1 of a secure column (8-byte loads: 2i is even)
__device__ __forceinline__ void q_load_pair(const QIn& s, uint32_t i, qm31& a, qm31& b) {
  uint2 w[4];
#pragma unroll
  for (int k = 0; k < 4; k++) w[k] = reinterpret_cast<const uint2*>(s.c[k])[i];
  a = qm31_make(w[0].x, w[1].x, w[2].x, w[3].x);
  b = qm31_make(w[0].y, w[1].y, w[2].y, w[3].y);
}

__device__ __forceinline__ uint32_t grid_stride() { return gridDim.x * blockDim.x; }
__device__ __forceinline__ uint32_t global_thread() { return blockIdx.x * blockDim.x + threadIdx.x; }

uint32_t stream_blocks(uint64_t n, uint32_t threads, uint32_t per_sm) {
  const uint64_t need = (n + threads - 1) / threads;
  return (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(need, 152ull * per_sm));
}

// ------------------------------------------------------------ gen_eq_evals

constexpr uint32_t kEqLowBits = 10;    // index bits of the per-block table
constexpr uint32_t kEqChunkBits = 14;  // values written per block
constexpr uint32_t kEqMaxVars = 28;

struct EqParams {
  qm31 v;
  qm31 y[kEqMaxVars];
  uint32_t n;
};

// evals[i] = v * prod_j eq(x_j, y_j), x_j = bit n-1-j of i (gen_eq_evals,
// cpu/lookups/gkr.rs:230-246: the loop over y in reverse doubles the table, so
// y[n-1] is index bit 0). Each block builds the factor of the low kEqLowBits
// bits as a table in shared memory by the same doubling, the factor of its own
// high bits directly, and writes their products.
__global__ void __launch_bounds__(256) eq_evals_kernel(const EqParams p, const QOut out) {
  __shared__ qm31 low[1u << kEqLowBits];
  __shared__ qm31 high[1u << (kEqChunkBits - kEqLowBits)];
  const uint32_t n = p.n;
  const uint32_t k = min(n, kEqLowBits);
  const uint32_t chunk = min(n, kEqChunkBits);
  if (threadIdx.x == 0) low[0] = q_one();
  __syncthreads();
  for (uint32_t t = 0; t < k; t++) {
    const qm31 yt = p.y[n - 1 - t];
    for (uint32_t j = threadIdx.x; j < (1u << t); j += blockDim.x) {
      const qm31 lj = low[j];
      const qm31 tmp = qm31_mul(lj, yt);
      low[j + (1u << t)] = tmp;
      low[j] = qm31_sub(lj, tmp);
    }
    __syncthreads();
  }
  const uint32_t first = blockIdx.x << chunk;
  if (threadIdx.x < (1u << (chunk - k))) {
    const uint32_t hi = (first >> k) + threadIdx.x;
    qm31 h = p.v;
    for (uint32_t t = k; t < n; t++) {
      const qm31 yt = p.y[n - 1 - t];
      h = qm31_mul(h, ((hi >> (t - k)) & 1u) ? yt : qm31_sub(q_one(), yt));
    }
    high[threadIdx.x] = h;
  }
  __syncthreads();
  const uint32_t low_mask = (1u << k) - 1;
  for (uint32_t e = threadIdx.x; e < (1u << chunk); e += blockDim.x)
    q_store(out, first + e, qm31_mul(high[e >> k], low[e & low_mask]));
}

// ------------------------------------------------------------ fix_first_variable

// dst[i] = a * (src[i + half] - src[i]) + src[i] for i < half (fold_mle_evals,
// crates/stwo/src/prover/lookups/utils.rs; MleOps, cpu/lookups/mle.rs:12-45).
// dst may be src itself: element i is written only by the thread that read it.
template <bool BASE>
__global__ void __launch_bounds__(256) fix_first_kernel(const QIn src, uint32_t half, qm31 a, const QOut dst) {
  for (uint32_t i = global_thread(); i < half; i += grid_stride()) {
    qm31 r;
    if constexpr (BASE) {
      const uint32_t l = src.c[0][i];
      r = qm31_add_m31(qm31_mul_m31(a, m31_sub(src.c[0][i + half], l)), l);
    } else {
      const qm31 l = q_load(src, i);
      r = qm31_add(qm31_mul(a, qm31_sub(q_load(src, i + half), l)), l);
    }
    q_store(dst, i, r);
  }
}

// ------------------------------------------------------------ next_layer

// Fraction addition n0/d0 + n1/d1 = (d1 n0 + d0 n1) / (d0 d1) (crates/stwo/src/core/fraction.rs:19-31).
__device__ __forceinline__ void frac_add(qm31 n0, qm31 d0, qm31 n1, qm31 d1, qm31& n, qm31& d) {
  n = qm31_add(qm31_mul(d1, n0), qm31_mul(d0, n1));
  d = qm31_mul(d0, d1);
}

// One output of the next layer from inputs 2i and 2i + 1
// (next_grand_product_layer / next_logup_layer, cpu/lookups/gkr.rs:248-281).
template <int KIND>
__global__ void __launch_bounds__(256) next_layer_kernel(const QIn num, const QIn den, uint32_t half,
                                                          const QOut out_num, const QOut out_den) {
  for (uint32_t i = global_thread(); i < half; i += grid_stride()) {
    qm31 d0, d1;
    q_load_pair(den, i, d0, d1);
    if constexpr (KIND == CS_GKR_GRAND_PRODUCT) {
      q_store(out_den, i, qm31_mul(d0, d1));
      continue;
    }
    qm31 n0, n1;
    if constexpr (KIND == CS_GKR_LOGUP_GENERIC) {
      q_load_pair(num, i, n0, n1);
    } else if constexpr (KIND == CS_GKR_LOGUP_MULTIPLICITIES) {
      const uint2 w = reinterpret_cast<const uint2*>(num.c[0])[i];
      n0 = qm31_make(w.x, 0, 0, 0);
      n1 = qm31_make(w.y, 0, 0, 0);
    } else {
      n0 = q_one();
      n1 = q_one();
    }
    qm31 n, d;
    frac_add(n0, d0, n1, d1, n, d);
    q_store(out_num, i, n);
    q_store(out_den, i, d);
  }
}

// ------------------------------------------------------------ sum_as_poly_in_first_variable

__device__ __forceinline__ qm31 q_shfl_add(qm31 v, int off) {
  return qm31_make(m31_add(v.a.a, __shfl_xor_sync(0xffffffffu, v.a.a, off)),
                   m31_add(v.a.b, __shfl_xor_sync(0xffffffffu, v.a.b, off)),
                   m31_add(v.b.a, __shfl_xor_sync(0xffffffffu, v.b.a, off)),
                   m31_add(v.b.b, __shfl_xor_sync(0xffffffffu, v.b.b, off)));
}

// Sum of two QM31 values over a 256-thread block; thread 0 gets the totals.
__device__ __forceinline__ void block_sum2(qm31& s0, qm31& s2) {
  __shared__ qm31 part[2][8];
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    s0 = q_shfl_add(s0, off);
    s2 = q_shfl_add(s2, off);
  }
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
    part[0][warp] = s0;
    part[1][warp] = s2;
  }
  __syncthreads();
  if (warp == 0) {
    s0 = lane < 8 ? part[0][lane] : q_zero();
    s2 = lane < 8 ? part[1][lane] : q_zero();
#pragma unroll
    for (int off = 4; off > 0; off >>= 1) {
      s0 = q_shfl_add(s0, off);
      s2 = q_shfl_add(s2, off);
    }
  }
}

// Per term i < n_terms the input layer at (r, t, bits(i), {0, 1}) for t = 0 (values 2i, 2i+1) and
// t = 1 (values 2(n_terms+i), +1); t = 2 is 2 v(t=1) - v(t=0). Adds eq[i] times the gate's output
// at t = 0 and t = 2 (eval_grand_product_sum / eval_logup_sum / eval_logup_singles_sum,
// cpu/lookups/gkr.rs:66-227); LogUp gates combine numerator + lambda * denominator.
template <int KIND>
__global__ void __launch_bounds__(256) sum_poly_kernel(const QIn eq, const QIn num, const QIn den, uint32_t n_terms,
                                                        const qm31_const lambda, uint32_t* partial) {
  qm31 s0 = q_zero(), s2 = q_zero();
  for (uint32_t i = global_thread(); i < n_terms; i += grid_stride()) {
    qm31 d00, d01, d10, d11;
    q_load_pair(den, i, d00, d01);
    q_load_pair(den, n_terms + i, d10, d11);
    const qm31 d20 = qm31_sub(q_double(d10), d00);
    const qm31 d21 = qm31_sub(q_double(d11), d01);
    qm31 g0, g2;
    if constexpr (KIND == CS_GKR_GRAND_PRODUCT) {
      g0 = qm31_mul(d00, d01);
      g2 = qm31_mul(d20, d21);
    } else {
      qm31 n00{}, n01{}, n10{}, n11{};
      if constexpr (KIND == CS_GKR_LOGUP_GENERIC) {
        q_load_pair(num, i, n00, n01);
        q_load_pair(num, n_terms + i, n10, n11);
      } else if constexpr (KIND == CS_GKR_LOGUP_MULTIPLICITIES) {
        const uint2 w0 = reinterpret_cast<const uint2*>(num.c[0])[i];
        const uint2 w1 = reinterpret_cast<const uint2*>(num.c[0])[n_terms + i];
        n00 = qm31_make(w0.x, 0, 0, 0);
        n01 = qm31_make(w0.y, 0, 0, 0);
        n10 = qm31_make(w1.x, 0, 0, 0);
        n11 = qm31_make(w1.y, 0, 0, 0);
      }
      qm31 num0, den0, num2, den2;
      if constexpr (KIND == CS_GKR_LOGUP_SINGLES) {
        // 1/a + 1/b = (a + b) / (a b) (Reciprocal, crates/stwo/src/prover/lookups/utils.rs)
        num0 = qm31_add(d00, d01);
        den0 = qm31_mul(d00, d01);
        num2 = qm31_add(d20, d21);
        den2 = qm31_mul(d20, d21);
      } else {
        const qm31 n20 = qm31_sub(q_double(n10), n00);
        const qm31 n21 = qm31_sub(q_double(n11), n01);
        frac_add(n00, d00, n01, d01, num0, den0);
        frac_add(n20, d20, n21, d21, num2, den2);
      }
      g0 = qm31_add(num0, qm31_mul_const(den0, lambda));
      g2 = qm31_add(num2, qm31_mul_const(den2, lambda));
    }
    const qm31 e = q_load(eq, i);
    s0 = qm31_add(s0, qm31_mul(e, g0));
    s2 = qm31_add(s2, qm31_mul(e, g2));
  }
  block_sum2(s0, s2);
  if (threadIdx.x == 0) {
    uint32_t* o = partial + 8 * blockIdx.x;
    o[0] = s0.a.a, o[1] = s0.a.b, o[2] = s0.b.a, o[3] = s0.b.b;
    o[4] = s2.a.a, o[5] = s2.a.b, o[6] = s2.b.a, o[7] = s2.b.b;
  }
}

__global__ void __launch_bounds__(256) sum_partials_kernel(const uint32_t* partial, uint32_t n_parts, uint32_t* out) {
  qm31 s0 = q_zero(), s2 = q_zero();
  for (uint32_t b = threadIdx.x; b < n_parts; b += blockDim.x) {
    const uint32_t* o = partial + 8 * b;
    s0 = qm31_add(s0, qm31_make(o[0], o[1], o[2], o[3]));
    s2 = qm31_add(s2, qm31_make(o[4], o[5], o[6], o[7]));
  }
  block_sum2(s0, s2);
  if (threadIdx.x == 0) {
    out[0] = s0.a.a, out[1] = s0.a.b, out[2] = s0.b.a, out[3] = s0.b.b;
    out[4] = s2.a.a, out[5] = s2.a.b, out[6] = s2.b.a, out[7] = s2.b.b;
  }
}

// ------------------------------------------------------------ host helpers

bool read_secure(const uint32_t* const h[4], QIn& q) {
  if (h == nullptr) return false;
  for (int k = 0; k < 4; k++) {
    if (h[k] == nullptr) return false;
    q.c[k] = h[k];
  }
  return true;
}
bool read_secure_out(uint32_t* const h[4], QOut& q) {
  if (h == nullptr) return false;
  for (int k = 0; k < 4; k++) {
    if (h[k] == nullptr) return false;
    q.c[k] = h[k];
  }
  return true;
}
qm31 host_qm31(const uint32_t v[4]) { return qm31_make(v[0] % P, v[1] % P, v[2] % P, v[3] % P); }
bool aligned8(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 7u) == 0; }

}  // namespace
}  // namespace cs

using namespace cs;

extern "C" cs_status cs_gkr_gen_eq_evals(const uint32_t* h_y, uint32_t n_y, const uint32_t h_v[4],
                                         uint32_t* const h_out[4], cs_stream stream) {
  CS_CHECK_ARG(n_y <= kEqMaxVars, "gkr_gen_eq_evals: %u variables (at most %u)", n_y, kEqMaxVars);
  CS_CHECK_ARG(h_v != nullptr && (n_y == 0 || h_y != nullptr), "gkr_gen_eq_evals: null pointer");
  QOut out;
  CS_CHECK_ARG(read_secure_out(h_out, out), "gkr_gen_eq_evals: null output column");
  EqParams p{};
  p.v = host_qm31(h_v);
  for (uint32_t j = 0; j < n_y; j++) p.y[j] = host_qm31(h_y + 4 * j);
  p.n = n_y;
  const uint32_t chunk = std::min(n_y, kEqChunkBits);
  eq_evals_kernel<<<1u << (n_y - chunk), 256, 0, to_stream(stream)>>>(p, out);
  CS_LAUNCHED("eq_evals_kernel");
  return CS_OK;
}

extern "C" cs_status cs_mle_fix_first_variable(const uint32_t* const h_src[4], uint32_t src_is_base,
                                               uint32_t log_n, const uint32_t h_assignment[4],
                                               uint32_t* const h_dst[4], cs_stream stream) {
  CS_CHECK_ARG(log_n >= 1 && log_n <= 31, "mle_fix_first_variable: log size %u (1..31)", log_n);
  CS_CHECK_ARG(h_assignment != nullptr, "mle_fix_first_variable: null assignment");
  QIn src{};
  if (src_is_base) {
    CS_CHECK_ARG(h_src != nullptr && h_src[0] != nullptr, "mle_fix_first_variable: null source column");
    src.c[0] = h_src[0];
  } else {
    CS_CHECK_ARG(read_secure(h_src, src), "mle_fix_first_variable: null source column");
  }
  QOut dst;
  CS_CHECK_ARG(read_secure_out(h_dst, dst), "mle_fix_first_variable: null output column");
  const uint32_t half = 1u << (log_n - 1);
  const qm31 a = host_qm31(h_assignment);
  const uint32_t blocks = stream_blocks(half, 256, 8);
  if (src_is_base)
    fix_first_kernel<true><<<blocks, 256, 0, to_stream(stream)>>>(src, half, a, dst);
  else
    fix_first_kernel<false><<<blocks, 256, 0, to_stream(stream)>>>(src, half, a, dst);
  CS_LAUNCHED("fix_first_kernel");
  return CS_OK;
}

extern "C" cs_status cs_gkr_next_layer(uint32_t kind, const uint32_t* const h_num[4], const uint32_t* const h_den[4],
                                       uint32_t log_n, uint32_t* const h_out_num[4], uint32_t* const h_out_den[4],
                                       cs_stream stream) {
  CS_CHECK_ARG(kind <= CS_GKR_LOGUP_SINGLES, "gkr_next_layer: unknown layer kind %u", kind);
  CS_CHECK_ARG(log_n >= 1 && log_n <= 31, "gkr_next_layer: log size %u (1..31)", log_n);
  QIn num{}, den{};
  QOut onum{}, oden{};
  CS_CHECK_ARG(read_secure(h_den, den), "gkr_next_layer: null denominator (or grand-product) column");
  CS_CHECK_ARG(read_secure_out(h_out_den, oden), "gkr_next_layer: null output column");
  if (kind == CS_GKR_LOGUP_GENERIC) CS_CHECK_ARG(read_secure(h_num, num), "gkr_next_layer: null numerator column");
  if (kind == CS_GKR_LOGUP_MULTIPLICITIES) {
    CS_CHECK_ARG(h_num != nullptr && h_num[0] != nullptr, "gkr_next_layer: null numerator column");
    num.c[0] = h_num[0];
  }
  if (kind != CS_GKR_GRAND_PRODUCT)
    CS_CHECK_ARG(read_secure_out(h_out_num, onum), "gkr_next_layer: null output numerator column");
  for (int k = 0; k < 4; k++)
    CS_CHECK_ARG(aligned8(den.c[k]) && (num.c[k] == nullptr || aligned8(num.c[k])),
                 "gkr_next_layer: input columns must be 8-byte aligned");
  const uint32_t half = 1u << (log_n - 1);
  const uint32_t blocks = stream_blocks(half, 256, 8);
  cudaStream_t st = to_stream(stream);
  switch (kind) {
    case CS_GKR_GRAND_PRODUCT:
      next_layer_kernel<CS_GKR_GRAND_PRODUCT><<<blocks, 256, 0, st>>>(num, den, half, onum, oden);
      break;
    case CS_GKR_LOGUP_GENERIC:
      next_layer_kernel<CS_GKR_LOGUP_GENERIC><<<blocks, 256, 0, st>>>(num, den, half, onum, oden);
      break;
    case CS_GKR_LOGUP_MULTIPLICITIES:
      next_layer_kernel<CS_GKR_LOGUP_MULTIPLICITIES><<<blocks, 256, 0, st>>>(num, den, half, onum, oden);
      break;
    default:
      next_layer_kernel<CS_GKR_LOGUP_SINGLES><<<blocks, 256, 0, st>>>(num, den, half, onum, oden);
  }
  CS_LAUNCHED("next_layer_kernel");
  return CS_OK;
}

extern "C" cs_status cs_gkr_sum_as_poly(uint32_t kind, const uint32_t* const h_eq[4], const uint32_t* const h_num[4],
                                        const uint32_t* const h_den[4], uint32_t log_n, const uint32_t h_lambda[4],
                                        uint32_t* d_out, cs_stream stream) {
  CS_CHECK_ARG(kind <= CS_GKR_LOGUP_SINGLES, "gkr_sum_as_poly: unknown layer kind %u", kind);
  CS_CHECK_ARG(log_n >= 2 && log_n <= 31, "gkr_sum_as_poly: input layer log size %u (2..31)", log_n);
  CS_CHECK_ARG(h_lambda != nullptr && d_out != nullptr, "gkr_sum_as_poly: null pointer");
  QIn eq{}, num{}, den{};
  CS_CHECK_ARG(read_secure(h_eq, eq), "gkr_sum_as_poly: null eq column");
  CS_CHECK_ARG(read_secure(h_den, den), "gkr_sum_as_poly: null denominator (or grand-product) column");
  if (kind == CS_GKR_LOGUP_GENERIC) CS_CHECK_ARG(read_secure(h_num, num), "gkr_sum_as_poly: null numerator column");
  if (kind == CS_GKR_LOGUP_MULTIPLICITIES) {
    CS_CHECK_ARG(h_num != nullptr && h_num[0] != nullptr, "gkr_sum_as_poly: null numerator column");
    num.c[0] = h_num[0];
  }
  for (int k = 0; k < 4; k++)
    CS_CHECK_ARG(aligned8(den.c[k]) && (num.c[k] == nullptr || aligned8(num.c[k])),
                 "gkr_sum_as_poly: input columns must be 8-byte aligned");
  const uint32_t n_terms = 1u << (log_n - 2);
  // up to 1024 terms one block sums them and writes the result itself (most sum-check rounds
  // are small: the columns halve every round); larger sums go through per-block partials
  const uint32_t blocks = n_terms <= 1024 ? 1 : stream_blocks(n_terms, 256, 4);
  const qm31_const lambda = qm31_const_of(host_qm31(h_lambda));
  cudaStream_t st = to_stream(stream);
  uint32_t* partial = d_out;
  if (blocks > 1) CS_CUDA(stream_alloc(reinterpret_cast<void**>(&partial), sizeof(uint32_t) * 8 * blocks, st));
  switch (kind) {
    case CS_GKR_GRAND_PRODUCT:
      sum_poly_kernel<CS_GKR_GRAND_PRODUCT><<<blocks, 256, 0, st>>>(eq, num, den, n_terms, lambda, partial);
      break;
    case CS_GKR_LOGUP_GENERIC:
      sum_poly_kernel<CS_GKR_LOGUP_GENERIC><<<blocks, 256, 0, st>>>(eq, num, den, n_terms, lambda, partial);
      break;
    case CS_GKR_LOGUP_MULTIPLICITIES:
      sum_poly_kernel<CS_GKR_LOGUP_MULTIPLICITIES><<<blocks, 256, 0, st>>>(eq, num, den, n_terms, lambda, partial);
      break;
    default:
      sum_poly_kernel<CS_GKR_LOGUP_SINGLES><<<blocks, 256, 0, st>>>(eq, num, den, n_terms, lambda, partial);
  }
  note_launch();
  cudaError_t e = cudaGetLastError();
  if (blocks == 1) {
    if (e != cudaSuccess) return from_cuda(e, "launch sum_poly_kernel");
    return CS_OK;
  }
  if (e == cudaSuccess) {
    sum_partials_kernel<<<1, 256, 0, st>>>(partial, blocks, d_out);
    note_launch();
    e = cudaGetLastError();
  }
  const cudaError_t ef = cudaFreeAsync(partial, st);
  if (e != cudaSuccess) return from_cuda(e, "launch sum_poly_kernel");
  if (ef != cudaSuccess) return from_cuda(ef, "cudaFreeAsync");
  return CS_OK;
}
