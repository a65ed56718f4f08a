// Twiddle-tree precompute and column bit reversal.
//
// precompute_twiddles: crates/stwo/src/prover/backend/cpu/circle.rs:240-285
// (slow_precompute_twiddles) — per doubling j of the root coset, the
// x-coordinates of the first half of the coset, bit-reversed, concatenated,
// plus one pad word 1. Every word is computed independently on the device:
// the point of index idx is sum_b [bit b of idx] * (2^b G), with the 31 powers
// 2^b G passed in as a kernel parameter; itwiddles are Fermat inverses.
#include <algorithm>

#include "common.cuh"
#include "field.cuh"

namespace cs {

namespace {

struct GenPowers {
  cpoint p[31];  // (2^b) * M31_CIRCLE_GEN
};

GenPowers make_gen_powers() {
  GenPowers g;
  cpoint cur{2u, 1268011823u};
  for (int b = 0; b < 31; b++) {
    g.p[b] = cur;
    cur = cpoint_add(cur, cur);
  }
  return g;
}

__device__ __forceinline__ cpoint point_of_index(const GenPowers& g, uint32_t idx) {
  cpoint r{1, 0};
#pragma unroll 1
  for (int b = 0; b < 31; b++)
    if ((idx >> b) & 1) r = cpoint_add(r, g.p[b]);
  return r;
}

__global__ void twiddles_kernel(const GenPowers g, uint32_t initial_index, uint32_t K, uint32_t* tw, uint32_t* itw) {
  const uint32_t n = 1u << K;
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    uint32_t x;
    if (t == n - 1) {
      x = 1;  // pad
    } else {
      // layer j occupies [2^K - 2^(K-j), 2^K - 2^(K-j-1)); rem = 2^K - t in (2^(K-j-1), 2^(K-j)]
      const uint32_t rem = n - t;
      const uint32_t ceil_log = 32 - __clz(rem - 1);
      const uint32_t j = K - ceil_log;
      const uint32_t layer_log = K - j - 1;  // log of the half coset size at layer j
      const uint32_t i = t - (n - (1u << (K - j)));
      const uint32_t br = layer_log == 0 ? 0 : (__brev(i) >> (32 - layer_log));
      const uint32_t init = (initial_index << j) & 0x7fffffffu;
      const uint32_t step = (1u << (31 - K)) << j;  // subgroup_gen(K) doubled j times
      const uint32_t idx = (init + br * step) & 0x7fffffffu;
      x = point_of_index(g, idx).x;
    }
    tw[t] = x;
    if (itw) itw[t] = m31_inv(x);
  }
}

__global__ void bit_reverse_kernel(uint32_t* col, uint32_t log_n) {
  const uint32_t n = 1u << log_n;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t j = __brev(i) >> (32 - log_n);
    if (j > i) {
      const uint32_t a = col[i];
      col[i] = col[j];
      col[j] = a;
    }
  }
}

}  // namespace
}  // namespace cs

using namespace cs;

extern "C" cs_status cs_precompute_twiddles(uint32_t root_initial_index, uint32_t root_log_size,
                                            uint32_t* d_twiddles, uint32_t* d_itwiddles, cs_stream stream) {
  CS_CHECK_ARG(d_twiddles != nullptr, "precompute_twiddles: null output");
  CS_CHECK_ARG(root_log_size >= 1 && root_log_size <= 29, "precompute_twiddles: log size %u out of range",
               root_log_size);
  static const GenPowers g = make_gen_powers();
  const uint32_t n = 1u << root_log_size;
  const uint32_t blocks = std::min<uint32_t>((n + 255) / 256, 152 * 16);
  twiddles_kernel<<<blocks, 256, 0, to_stream(stream)>>>(g, root_initial_index & 0x7fffffffu, root_log_size,
                                                          d_twiddles, d_itwiddles);
  CS_LAUNCHED("twiddles_kernel");
  return CS_OK;
}

extern "C" cs_status cs_bit_reverse_m31(uint32_t* d_col, uint32_t log_size, cs_stream stream) {
  CS_CHECK_ARG(d_col != nullptr, "bit_reverse: null column");
  CS_CHECK_ARG(log_size <= 30, "bit_reverse: log size %u too large", log_size);
  if (log_size == 0) return CS_OK;
  const uint32_t n = 1u << log_size;
  const uint32_t blocks = std::min<uint32_t>((n + 255) / 256, 152 * 16);
  bit_reverse_kernel<<<blocks, 256, 0, to_stream(stream)>>>(d_col, log_size);
  CS_LAUNCHED("bit_reverse_kernel");
  return CS_OK;
}
