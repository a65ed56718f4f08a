// Shared pieces of the proof-of-work search (grind.cu).
#pragma once
#include <cstdint>

#include "common.cuh"

namespace cs {

// Blake2s chaining value = digest words of H(0x12345678 || digest || pow_bits).
struct GrindPrefix {
  uint32_t w[8];
};

GrindPrefix grind_prefix(const uint8_t digest[32], uint32_t pow_bits);

__global__ void grind_kernel(const GrindPrefix pre, uint32_t pow_bits, uint64_t base, uint32_t tries,
                             unsigned long long* best);

// Runs the search with a caller-provided 8-byte device slot; synchronous on st.
cs_status grind_with_slot(const uint8_t digest[32], uint32_t pow_bits, uint64_t max_nonce, uint64_t* nonce_out,
                          unsigned long long* d_best, cudaStream_t st);

}  // namespace cs
