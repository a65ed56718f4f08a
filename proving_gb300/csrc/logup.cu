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
  CS_CHECK_ARG(log_size >= 10 && log_size <= 28, "logup_running_sum: log size %u outside [10, 28]", log_size);
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
