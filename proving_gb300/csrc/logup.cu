// LogUp interaction columns on the device: the last column of
// LogupTraceGenerator (crates/constraint-framework/src/prover/logup.rs:50-130)
// for fractions 1 / (z - v_i): claimed_sum = sum_i 1 / (z - v_i), each
// fraction shifted by claimed_sum / n, then the inclusive prefix sum in coset
// order (inclusive_prefix_sum, crates/stwo/src/prover/backend/simd/prefix_sum.rs:20-149),
// values stored in bit-reversed circle-domain order. Coset index k lives at
// circle-domain index k / 2 (k even) or n/2 + (n - 1 - k) / 2 (k odd)
// (crates/stwo/src/core/utils.rs:177-188), stored at its bit reversal.
//
// Kernels: fractions (one QM31 inverse per row); claimed sum (one block);
// block scans of 1024 coset-ordered values with the shift applied, writing
// block totals; a scan of the totals; the block offsets added back.
#include <algorithm>

#include "common.cuh"
#include "field.cuh"
#include "logup.cuh"
#include "rows.cuh"

namespace cs {

namespace {

constexpr uint32_t kScanBlock = 1024;

__device__ __forceinline__ uint32_t coset_pos(uint32_t k, uint32_t log_n) {
  const uint32_t n = 1u << log_n;
  const uint32_t c = (k & 1) ? (n >> 1) + ((n - 1 - k) >> 1) : (k >> 1);
  return __brev(c) >> (32 - log_n);
}

__global__ void fractions_kernel(const uint32_t* __restrict__ v, uint32_t n, qm31 z, Q4 out) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const qm31 f = qm31_inv(qm31_sub(z, qm31_make(v[i], 0, 0, 0)));
    out.c[0][i] = f.a.a;
    out.c[1][i] = f.a.b;
    out.c[2][i] = f.b.a;
    out.c[3][i] = f.b.b;
  }
}

__global__ void sum_kernel(Q4 in, uint32_t n, uint32_t* sum_out) {
  __shared__ uint64_t sh[32];
  for (int k = 0; k < 4; k++) {
    uint64_t acc = 0;
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) acc += in.c[k][i];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
      uint64_t t = 0;
      for (uint32_t w = 0; w < blockDim.x / 32; w++) t += sh[w];
      sum_out[k] = (uint32_t)(t % P);
    }
    __syncthreads();
  }
}

// Inclusive scan of one M31 value per thread across a 1024-thread block.
__device__ __forceinline__ uint32_t block_scan(uint32_t x, uint32_t* sh) {
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= (uint32_t)o) x = m31_add(x, y);
  }
  if (lane == 31) sh[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t t = lane < (blockDim.x >> 5) ? sh[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= (uint32_t)o) t = m31_add(t, y);
    }
    sh[lane] = t;
  }
  __syncthreads();
  if (warp > 0) x = m31_add(x, sh[warp - 1]);
  __syncthreads();
  return x;
}

__global__ void __launch_bounds__(kScanBlock) block_scan_kernel(Q4 io, uint32_t log_n, qm31 shift,
                                                                uint32_t* totals) {
  __shared__ uint32_t sh[32];
  const uint32_t k = blockIdx.x * kScanBlock + threadIdx.x;
  const uint32_t pos = coset_pos(k, log_n);
  const uint32_t s[4] = {shift.a.a, shift.a.b, shift.b.a, shift.b.b};
  for (int c = 0; c < 4; c++) {
    const uint32_t x = block_scan(m31_sub(io.c[c][pos], s[c]), sh);
    io.c[c][pos] = x;
    if (threadIdx.x == kScanBlock - 1) totals[4 * blockIdx.x + c] = x;
  }
}

// Exclusive scan of the block totals (one block, sequential chunks).
__global__ void __launch_bounds__(kScanBlock) totals_scan_kernel(uint32_t* totals, uint32_t n_blocks) {
  __shared__ uint32_t sh[32];
  for (int c = 0; c < 4; c++) {
    uint32_t carry = 0;
    for (uint32_t base = 0; base < n_blocks; base += kScanBlock) {
      const uint32_t i = base + threadIdx.x;
      const uint32_t x = i < n_blocks ? totals[4 * i + c] : 0;
      const uint32_t inc = block_scan(x, sh);
      if (i < n_blocks) totals[4 * i + c] = m31_add(m31_sub(inc, x), carry);  // exclusive + carry
      __shared__ uint32_t last;
      if (threadIdx.x == kScanBlock - 1) last = inc;
      __syncthreads();
      carry = m31_add(carry, last);
      __syncthreads();
    }
  }
}

__global__ void add_offsets_kernel(Q4 io, uint32_t log_n, const uint32_t* offsets) {
  const uint32_t k = blockIdx.x * kScanBlock + threadIdx.x;
  const uint32_t pos = coset_pos(k, log_n);
  for (int c = 0; c < 4; c++) io.c[c][pos] = m31_add(io.c[c][pos], offsets[4 * blockIdx.x + c]);
}

struct LookupCompParams {
  const uint32_t* values;  // the trace column on the evaluation domain
  const uint32_t* inter[4];
  qm31 z, shift, rc;
  uint32_t den[32];
  uint32_t eval_log, trace_log;
};

// Quotient of a single-column LogUp component's one constraint
// (cur - prev + shift) (v - z) + 1, weighted by rc, per evaluation row.
__global__ void lookup_composition_kernel(const LookupCompParams p, uint32_t* a0, uint32_t* a1, uint32_t* a2,
                                          uint32_t* a3) {
  const uint32_t n = 1u << p.eval_log;
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    const uint32_t pr = prev_row(r, p.trace_log, p.eval_log);
    const qm31 cur = qm31_make(__ldg(p.inter[0] + r), __ldg(p.inter[1] + r), __ldg(p.inter[2] + r),
                               __ldg(p.inter[3] + r));
    const qm31 prev = qm31_make(__ldg(p.inter[0] + pr), __ldg(p.inter[1] + pr), __ldg(p.inter[2] + pr),
                                __ldg(p.inter[3] + pr));
    const qm31 shifted = qm31_add(qm31_sub(cur, prev), p.shift);
    const qm31 cons = qm31_add(qm31_mul(shifted, qm31_sub(qm31_make(__ldg(p.values + r), 0, 0, 0), p.z)),
                               qm31_make(1, 0, 0, 0));
    const qm31 v = qm31_mul_m31(qm31_mul(p.rc, cons), p.den[r >> p.trace_log]);
    a0[r] = m31_add(a0[r], v.a.a);
    a1[r] = m31_add(a1[r], v.a.b);
    a2[r] = m31_add(a2[r], v.b.a);
    a3[r] = m31_add(a3[r], v.b.b);
  }
}

cpoint lookup_point_at(uint32_t idx) {
  cpoint r{1, 0}, cur{2u, 1268011823u};
  while (idx) {
    if (idx & 1) r = cpoint_add(r, cur);
    cur = cpoint_add(cur, cur);
    idx >>= 1;
  }
  return r;
}

// Columns shorter than one scan block: one thread, in coset order.
__global__ void small_scan_kernel(Q4 io, uint32_t log_n, qm31 shift) {
  const uint32_t n = 1u << log_n;
  qm31 run = qm31_make(0, 0, 0, 0);
  for (uint32_t k = 0; k < n; k++) {
    const uint32_t pos = coset_pos(k, log_n);
    run = qm31_add(run, qm31_sub(qm31_make(io.c[0][pos], io.c[1][pos], io.c[2][pos], io.c[3][pos]), shift));
    io.c[0][pos] = run.a.a;
    io.c[1][pos] = run.a.b;
    io.c[2][pos] = run.b.a;
    io.c[3][pos] = run.b.b;
  }
}

}  // namespace

cs_status logup_finalize_last(Q4 col, uint32_t log_size, uint32_t claimed_sum_out[4], cudaStream_t st) {
  const uint32_t n = 1u << log_size, n_blocks = n / kScanBlock;
  uint32_t* scratch = nullptr;  // 4 words of sum, then 4 words per scan block
  CS_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&scratch), sizeof(uint32_t) * 4 * (1 + n_blocks), st));
  cs_status result = CS_OK;
  do {
    sum_kernel<<<1, 1024, 0, st>>>(col, n, scratch);
    note_launch();
    uint32_t sum[4];
    cudaError_t e = cudaMemcpyAsync(sum, scratch, sizeof(sum), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      result = from_cuda(e, "logup finalize");
      break;
    }
    for (int c = 0; c < 4; c++) claimed_sum_out[c] = sum[c];
    // shift = claimed_sum / n, 1/n = 2^(31 - log_size)
    const qm31 shift = qm31_mul_m31(qm31_make(sum[0], sum[1], sum[2], sum[3]), 1u << (31 - log_size));
    if (n_blocks == 0) {
      small_scan_kernel<<<1, 1, 0, st>>>(col, log_size, shift);
      note_launch();
      e = cudaGetLastError();
      if (e != cudaSuccess) result = from_cuda(e, "logup finalize launch");
      break;
    }
    uint32_t* totals = scratch + 4;
    block_scan_kernel<<<n_blocks, kScanBlock, 0, st>>>(col, log_size, shift, totals);
    note_launch();
    totals_scan_kernel<<<1, kScanBlock, 0, st>>>(totals, n_blocks);
    note_launch();
    add_offsets_kernel<<<n_blocks, kScanBlock, 0, st>>>(col, log_size, totals);
    note_launch();
    e = cudaGetLastError();
    if (e != cudaSuccess) result = from_cuda(e, "logup finalize launch");
  } while (false);
  cudaError_t e = cudaFreeAsync(scratch, st);
  if (result == CS_OK && e != cudaSuccess) return from_cuda(e, "cudaFreeAsync");
  return result;
}

}  // namespace cs

using namespace cs;

extern "C" cs_status cs_logup_running_sum(const uint32_t* d_values, uint32_t log_size, const uint32_t z[4],
                                          uint32_t* const h_out[4], uint32_t claimed_sum_out[4], cs_stream stream) {
  CS_CHECK_ARG(d_values != nullptr && z != nullptr && h_out != nullptr && claimed_sum_out != nullptr,
               "logup_running_sum: null pointer");
  CS_CHECK_ARG(log_size >= 1 && log_size <= 28, "logup_running_sum: log size %u outside [1, 28]", log_size);
  Q4 out;
  for (int c = 0; c < 4; c++) {
    CS_CHECK_ARG(h_out[c] != nullptr, "logup_running_sum: null output coordinate");
    out.c[c] = h_out[c];
  }
  cudaStream_t st = to_stream(stream);
  const uint32_t n = 1u << log_size;
  fractions_kernel<<<std::min<uint32_t>((n + 255) / 256, 152 * 16), 256, 0, st>>>(
      d_values, n, qm31_make(z[0], z[1], z[2], z[3]), out);
  note_launch();
  CS_CUDA(cudaGetLastError());
  return logup_finalize_last(out, log_size, claimed_sum_out, st);
}

extern "C" cs_status cs_logup_composition(const uint32_t* d_values, const uint32_t* const h_inter[4], uint32_t eval_log,
                                          uint32_t trace_log, const uint32_t z[4], const uint32_t claimed_sum[4],
                                          const uint32_t rc[4], uint32_t* const h_accum[4], cs_stream stream) {
  CS_CHECK_ARG(d_values != nullptr && h_inter != nullptr && z != nullptr && claimed_sum != nullptr && rc != nullptr &&
                   h_accum != nullptr,
               "logup_composition: null pointer");
  CS_CHECK_ARG(trace_log >= 1 && eval_log >= trace_log && eval_log - trace_log <= 5 && eval_log <= 30,
               "logup_composition: bad sizes eval %u trace %u", eval_log, trace_log);
  LookupCompParams p;
  p.values = d_values;
  for (int c = 0; c < 4; c++) {
    CS_CHECK_ARG(h_inter[c] != nullptr && h_accum[c] != nullptr, "logup_composition: null column");
    p.inter[c] = h_inter[c];
  }
  p.z = qm31_make(z[0], z[1], z[2], z[3]);
  p.rc = qm31_make(rc[0], rc[1], rc[2], rc[3]);
  // cumsum_shift = claimed_sum / 2^trace_log (LogupAtRow::new, crates/constraint-framework/src/logup.rs:32-40)
  p.shift = qm31_mul_m31(qm31_make(claimed_sum[0], claimed_sum[1], claimed_sum[2], claimed_sum[3]),
                         1u << (31 - trace_log));
  p.eval_log = eval_log;
  p.trace_log = trace_log;
  const uint32_t log_expand = eval_log - trace_log, n_den = 1u << log_expand;
  if (log_expand == 0) {
    p.den[0] = 1;
  } else {
    // 1 / V_trace(eval_domain.at(i)), bit-reversed (component_prover.rs:101-108)
    for (uint32_t i = 0; i < n_den; i++) {
      const uint32_t idx = (subgroup_gen(eval_log + 1) + i * subgroup_gen(eval_log - 1)) & 0x7fffffffu;
      uint32_t x = lookup_point_at(idx).x;
      for (uint32_t k = 1; k < trace_log; k++) x = m31_sub(m31_add(m31_sqr(x), m31_sqr(x)), 1);
      uint32_t j = 0;
      for (uint32_t b = 0; b < log_expand; b++) j |= ((i >> b) & 1u) << (log_expand - 1 - b);
      p.den[j] = m31_inv(x);
    }
  }
  const uint32_t n = 1u << eval_log;
  const uint32_t blocks = std::max(1u, std::min((n + 255) / 256, 152u * 8));
  lookup_composition_kernel<<<blocks, 256, 0, to_stream(stream)>>>(p, h_accum[0], h_accum[1], h_accum[2],
                                                                    h_accum[3]);
  CS_LAUNCHED("lookup_composition_kernel");
  return CS_OK;
}
