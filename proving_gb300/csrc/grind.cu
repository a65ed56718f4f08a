// Proof-of-work grinding for the Blake2s channel, smallest nonce first.
//
// Spec: crates/stwo/src/core/channel/blake2s.rs:100-117 — prefixed =
// Blake2s(0x12345678_le || digest || pow_bits_le); a nonce passes when
// Blake2s(prefixed || nonce_le64) has >= pow_bits trailing zero bits in its
// low 128 bits (for pow_bits <= 32 that is the first digest word). The
// 40-byte message is a single final Blake2s block, as in the SIMD grind
// (crates/stwo/src/prover/backend/simd/grind.rs:65-92).
//
// Thread t of a launch tries nonces base + t, base + t + T, ... in increasing
// order and stops as soon as its next nonce is not below the best nonce found
// so far (an atomicMin'd 64-bit slot). Every nonce below the final answer is
// therefore tried, so the answer is the smallest qualifying nonce, like the
// reference's sequential CpuBackend::grind (cpu/grind.rs:5-15). The host
// relaunches over the next nonce range until one is found or max_nonce is
// reached. On GB300 the slot's update reaches some SMs late (a relaxed,
// acquire or volatile load; about one SM in eight polled the old value for
// dozens of hashes), so the early exit only trims work: the first launch
// tries one nonce per thread (2^18.2 nonces, enough for the 16-bit OODS and
// 10-bit FRI work almost always) and each relaunch doubles the tries per
// thread, up to 64.
#include <algorithm>

#include "blake2s.cuh"
#include "common.cuh"
#include "grind.cuh"

namespace cs {

__global__ void grind_kernel(const GrindPrefix pre, uint32_t pow_bits, uint64_t base, uint32_t tries,
                             unsigned long long* best) {
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t mask = pow_bits >= 32 ? 0xffffffffu : ((1u << pow_bits) - 1u);
  uint64_t nonce = base + tid;
  for (uint32_t k = 0; k < tries; k++, nonce += stride) {
    if (nonce >= *reinterpret_cast<volatile unsigned long long*>(best)) return;
    uint32_t m[16];
#pragma unroll
    for (int w = 0; w < 8; w++) m[w] = pre.w[w];
    m[8] = (uint32_t)nonce;
    m[9] = (uint32_t)(nonce >> 32);
#pragma unroll
    for (int w = 10; w < 16; w++) m[w] = 0;
    uint32_t h[8];
    b2s_init(h);
    b2s_compress(h, m, 40, 0, true);
    if ((h[0] & mask) == 0) {
      atomicMin(best, (unsigned long long)nonce);
      return;
    }
  }
}

GrindPrefix grind_prefix(const uint8_t digest[32], uint32_t pow_bits) {
  // One 40-byte final block: prefix word, 8 digest words, pow_bits.
  uint32_t m[16] = {0};
  m[0] = 0x12345678u;
  for (int w = 0; w < 8; w++)
    m[1 + w] = (uint32_t)digest[4 * w] | ((uint32_t)digest[4 * w + 1] << 8) | ((uint32_t)digest[4 * w + 2] << 16) |
               ((uint32_t)digest[4 * w + 3] << 24);
  m[9] = pow_bits;
  GrindPrefix pre;
  b2s_init(pre.w);
  b2s_compress(pre.w, m, 40, 0, true);
  return pre;
}

cs_status grind_with_slot(const uint8_t digest[32], uint32_t pow_bits, uint64_t max_nonce, uint64_t* nonce_out,
                          unsigned long long* d_best, cudaStream_t st) {
  const GrindPrefix pre = grind_prefix(digest, pow_bits);
  const uint32_t blocks = 152 * 8, threads = 256;
  unsigned long long best = ~0ull;
  uint32_t tries = 1;
  for (uint64_t base = 0; base < max_nonce;) {
    const uint64_t span = (uint64_t)blocks * threads * tries;
    CS_CUDA(cudaMemsetAsync(d_best, 0xff, sizeof(unsigned long long), st));
    grind_kernel<<<blocks, threads, 0, st>>>(pre, pow_bits, base, tries, d_best);
    CS_LAUNCHED("grind_kernel");
    CS_CUDA(cudaMemcpyAsync(&best, d_best, sizeof(best), cudaMemcpyDeviceToHost, st));
    CS_CUDA(cudaStreamSynchronize(st));
    if (best != ~0ull && best < max_nonce) {
      *nonce_out = best;
      return CS_OK;
    }
    if (base + span < base) break;  // wrapped
    base += span;
    tries = std::min(64u, 2 * tries);
  }
  set_error("grind: no nonce below %llu has %u trailing zero bits", (unsigned long long)max_nonce, pow_bits);
  return CS_ERR_TIMEOUT;
}

}  // namespace cs

using namespace cs;

extern "C" cs_status cs_grind_blake2s(const uint8_t digest[32], uint32_t pow_bits, uint64_t max_nonce,
                                      uint64_t* nonce_out, cs_stream stream) {
  CS_CHECK_ARG(digest != nullptr && nonce_out != nullptr, "grind: null digest or output");
  CS_CHECK_ARG(pow_bits <= 32, "grind: pow_bits %u > 32 is not supported", pow_bits);
  cudaStream_t st = to_stream(stream);
  unsigned long long* d_best = nullptr;
  CS_CUDA(stream_alloc(reinterpret_cast<void**>(&d_best), sizeof(unsigned long long), st));
  cs_status s = grind_with_slot(digest, pow_bits, max_nonce, nonce_out, d_best, st);
  cudaError_t e = cudaFreeAsync(d_best, st);
  if (s == CS_OK && e != cudaSuccess) return from_cuda(e, "cudaFreeAsync");
  return s;
}
