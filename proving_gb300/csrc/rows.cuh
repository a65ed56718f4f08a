// Row arithmetic of bit-reversed evaluation domains shared by the AIR kernels.
#pragma once
#include <cstdint>

namespace cs {

// The row one trace step before row r:
// offset_bit_reversed_circle_domain_index (crates/stwo/src/core/utils.rs:144-160)
// on a larger evaluation domain, the coset-order predecessor on the trace domain.
__device__ __forceinline__ uint32_t prev_row(uint32_t r, uint32_t trace_log, uint32_t eval_log) {
  const uint32_t n = 1u << eval_log, half = n >> 1;
  uint32_t i = __brev(r) >> (32 - eval_log);
  if (eval_log > trace_log) {
    const uint32_t step = 1u << (eval_log - trace_log - 1);
    i = i < half ? (i + half - step) & (half - 1) : ((i - half + step) & (half - 1)) + half;
  } else {
    uint32_t k = i < half ? 2 * i : 2 * (n - 1 - i) + 1;
    k = (k + n - 1) & (n - 1);
    i = (k & 1) ? half + ((n - 1 - k) >> 1) : (k >> 1);
  }
  return __brev(i) >> (32 - eval_log);
}

}  // namespace cs
