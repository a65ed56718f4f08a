// Device constraint evaluation and trace generation for the Wide-Fibonacci AIR
// (crates/examples/src/wide_fibonacci/mod.rs:27-48, 87-97), the analogue of
// FrameworkComponent::evaluate_constraint_quotients_on_domain for CpuBackend
// (crates/constraint-framework/src/prover/component_prover.rs:195-268).
//
// Row r of the evaluation domain accumulates
//   sum_k rc[k] * (c_{k+2}[r] - (c_k[r]^2 + c_{k+1}[r]^2)) * denom_inv[r >> trace_log]
// into the accumulator column. The 64-bit lazy sums stay exact: each term is
// reduced below 2^31 and at most 2^32 terms are added.
#include <algorithm>

#include "common.cuh"
#include "field.cuh"

namespace cs {

namespace {

constexpr uint32_t kMaxFibCols = 256;
constexpr uint32_t kMaxExpand = 5;

struct WideFibParams {
  const uint32_t* cols[kMaxFibCols];
  qm31 rc[kMaxFibCols];
  uint32_t den[1u << kMaxExpand];
  uint32_t n_cols, eval_log, trace_log;
};

__device__ __forceinline__ uint32_t fold64(uint64_t v) {
  const uint64_t t = (v & P) + (v >> 31);
  return m31_reduce_once((uint32_t)((t & P) + (t >> 31)));
}

__global__ void __launch_bounds__(256) wide_fib_composition_kernel(const __grid_constant__ WideFibParams p,
                                                                    uint32_t* a0, uint32_t* a1, uint32_t* a2,
                                                                    uint32_t* a3) {
  const uint32_t n = 1u << p.eval_log;
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    // Lazy sums: each weight x constraint product is below 2^62 and is added unreduced (one
    // 64-bit multiply-add per coordinate); folding every four constraints keeps the sums below
    // 2^64 (a fold leaves less than 2^34). Each column is squared once, for the constraint that
    // reads it as b and the next one that reads it as a.
    uint64_t acc[4] = {0, 0, 0, 0};
    uint32_t sa = m31_sqr(__ldg(p.cols[0] + r)), sb = m31_sqr(__ldg(p.cols[1] + r));
    for (uint32_t k = 0; k + 2 < p.n_cols; k++) {
      const uint32_t c = __ldg(p.cols[k + 2] + r);
      const uint32_t cons = m31_sub(c, m31_add(sa, sb));
      const qm31 w = p.rc[k];
      acc[0] += (uint64_t)w.a.a * cons;
      acc[1] += (uint64_t)w.a.b * cons;
      acc[2] += (uint64_t)w.b.a * cons;
      acc[3] += (uint64_t)w.b.b * cons;
      if ((k & 3) == 3) {
#pragma unroll
        for (int j = 0; j < 4; j++) acc[j] = (acc[j] & P) + (acc[j] >> 31);
      }
      sa = sb;
      sb = m31_sqr(c);
    }
    const uint32_t d = p.den[r >> p.trace_log];
    a0[r] = m31_add(a0[r], m31_mul(fold64(acc[0]), d));
    a1[r] = m31_add(a1[r], m31_mul(fold64(acc[1]), d));
    a2[r] = m31_add(a2[r], m31_mul(fold64(acc[2]), d));
    a3[r] = m31_add(a3[r], m31_mul(fold64(acc[3]), d));
  }
}

struct FibTraceCols {
  uint32_t* cols[kMaxFibCols];
};

__global__ void wide_fib_trace_kernel(const uint32_t* __restrict__ a0, const uint32_t* __restrict__ b0,
                                      uint32_t log_n, uint32_t n_cols, const __grid_constant__ FibTraceCols out) {
  const uint32_t n = 1u << log_n;
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    uint32_t a = a0[r], b = b0[r];
    out.cols[0][r] = a;
    out.cols[1][r] = b;
    for (uint32_t k = 2; k < n_cols; k++) {
      const uint32_t c = m31_add(m31_sqr(a), m31_sqr(b));
      a = b;
      b = c;
      out.cols[k][r] = c;
    }
  }
}

cpoint point_of(uint32_t idx) {
  cpoint r{1, 0}, cur{2u, 1268011823u};
  while (idx) {
    if (idx & 1) r = cpoint_add(r, cur);
    cur = cpoint_add(cur, cur);
    idx >>= 1;
  }
  return r;
}

}  // namespace
}  // namespace cs

using namespace cs;

extern "C" cs_status cs_wide_fib_composition(const uint32_t* const* h_cols, uint32_t n_cols, uint32_t eval_log,
                                             uint32_t trace_log, const uint32_t* h_rc, uint32_t* const h_accum[4],
                                             cs_stream stream) {
  CS_CHECK_ARG(h_cols != nullptr && h_rc != nullptr && h_accum != nullptr, "wide_fib_composition: null pointer");
  CS_CHECK_ARG(n_cols >= 3 && n_cols <= kMaxFibCols, "wide_fib_composition: %u columns (3..%u supported)", n_cols,
               kMaxFibCols);
  CS_CHECK_ARG(trace_log >= 1 && eval_log >= trace_log && eval_log - trace_log <= kMaxExpand && eval_log <= 30,
               "wide_fib_composition: bad sizes eval %u trace %u", eval_log, trace_log);
  static thread_local WideFibParams p;
  p.n_cols = n_cols;
  p.eval_log = eval_log;
  p.trace_log = trace_log;
  for (uint32_t k = 0; k < n_cols; k++) {
    CS_CHECK_ARG(h_cols[k] != nullptr, "wide_fib_composition: column %u is null", k);
    p.cols[k] = h_cols[k];
  }
  for (uint32_t k = 0; k + 2 < n_cols; k++)
    p.rc[k] = qm31_make(h_rc[4 * k] % P, h_rc[4 * k + 1] % P, h_rc[4 * k + 2] % P, h_rc[4 * k + 3] % P);
  // denom_inv[i] = 1 / V_trace(eval_domain.at(i)), i < 2^(eval - trace), then bit-reversed
  // (component_prover.rs:101-108). V of CanonicCoset(t).coset at p is pi^(t-1)(p.x).
  const uint32_t log_expand = eval_log - trace_log, n_den = 1u << log_expand;
  uint32_t den[1u << kMaxExpand];
  for (uint32_t i = 0; i < n_den; i++) {
    const uint32_t idx = (subgroup_gen(eval_log + 1) + i * subgroup_gen(eval_log - 1)) & 0x7fffffffu;
    uint32_t x = point_of(idx).x;
    for (uint32_t k = 1; k < trace_log; k++) x = m31_sub(m31_add(m31_sqr(x), m31_sqr(x)), 1);
    den[i] = m31_inv(x);
  }
  for (uint32_t i = 0; i < n_den; i++) {
    uint32_t j = 0;
    for (uint32_t b = 0; b < log_expand; b++) j |= ((i >> b) & 1u) << (log_expand - 1 - b);
    p.den[j] = den[i];
  }
  for (int c = 0; c < 4; c++) CS_CHECK_ARG(h_accum[c] != nullptr, "wide_fib_composition: null accumulator");
  const uint32_t n = 1u << eval_log;
  const uint32_t blocks = std::max(1u, std::min((n + 255) / 256, 152u * 8));
  wide_fib_composition_kernel<<<blocks, 256, 0, to_stream(stream)>>>(p, h_accum[0], h_accum[1], h_accum[2],
                                                                     h_accum[3]);
  CS_LAUNCHED("wide_fib_composition_kernel");
  return CS_OK;
}

extern "C" cs_status cs_wide_fib_trace(const uint32_t* d_a, const uint32_t* d_b, uint32_t log_n, uint32_t n_cols,
                                       uint32_t* const* h_cols, cs_stream stream) {
  CS_CHECK_ARG(d_a != nullptr && d_b != nullptr && h_cols != nullptr, "wide_fib_trace: null pointer");
  CS_CHECK_ARG(n_cols >= 2 && n_cols <= kMaxFibCols && log_n <= 30, "wide_fib_trace: bad sizes");
  static thread_local FibTraceCols out;
  for (uint32_t k = 0; k < n_cols; k++) {
    CS_CHECK_ARG(h_cols[k] != nullptr, "wide_fib_trace: column %u is null", k);
    out.cols[k] = h_cols[k];
  }
  const uint32_t n = 1u << log_n;
  const uint32_t blocks = std::max(1u, std::min((n + 255) / 256, 152u * 8));
  wide_fib_trace_kernel<<<blocks, 256, 0, to_stream(stream)>>>(d_a, d_b, log_n, n_cols, out);
  CS_LAUNCHED("wide_fib_trace_kernel");
  return CS_OK;
}
