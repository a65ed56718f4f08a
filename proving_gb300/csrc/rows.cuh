// Row arithmetic of bit-reversed evaluation domains shared by the AIR kernels.
#pragma once
#include <cstdint>

namespace cs {

// The row `offset` trace steps from row r (a mask offset of the constraint framework).
// On an evaluation domain larger than the trace this is
// offset_bit_reversed_circle_domain_index (crates/stwo/src/core/utils.rs:144-160): in natural
// order the first half of the domain steps forward by offset * 2^(eval_log - trace_log - 1)
// and the second half backward, each modulo the half. On the trace domain itself it is the
// coset-order neighbour (crates/constraint-framework/src/prover/assert.rs:58-66): the row's
// coset index plus offset, modulo the domain. Both wrap modulo a power of two that divides 2^32,
// so the arithmetic runs on unsigned words with the offset's two's complement.
__device__ __forceinline__ uint32_t offset_row(uint32_t r, int32_t offset, uint32_t trace_log,
                                               uint32_t eval_log) {
  const uint32_t n = 1u << eval_log, half = n >> 1;
  uint32_t i = __brev(r) >> (32 - eval_log);
  if (eval_log > trace_log) {
    const uint32_t step = (uint32_t)offset << (eval_log - trace_log - 1);
    i = i < half ? (i + step) & (half - 1) : ((i - half - step) & (half - 1)) + half;
  } else {
    uint32_t k = i < half ? 2 * i : 2 * (n - 1 - i) + 1;
    k = (k + (uint32_t)offset) & (n - 1);
    i = (k & 1) ? half + ((n - 1 - k) >> 1) : (k >> 1);
  }
  return __brev(i) >> (32 - eval_log);
}

// The row one trace step before row r.
__device__ __forceinline__ uint32_t prev_row(uint32_t r, uint32_t trace_log, uint32_t eval_log) {
  return offset_row(r, -1, trace_log, eval_log);
}

}  // namespace cs
