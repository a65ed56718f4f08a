// The device side of the Blake2s Fiat-Shamir channel (Blake2sChannel,
// crates/stwo/src/core/channel/blake2s.rs:16-118) on a 9-word state: the 32-byte digest as 8
// little-endian words, then the draw counter. Shared by the one-thread channel kernels
// (channel.cu) and the fused FRI tail (fri.cu).
#pragma once
#include <cstdint>

#include "blake2s.cuh"
#include "field.cuh"

namespace cs {

// Blake2sMerkleChannel::mix_hash (crates/stwo/src/core/vcs_lifted/blake2_merkle.rs:56-58):
// digest <- Blake2s(digest || root), one 64-byte final block; the draw counter restarts
// (Blake2sChannel::update_digest, blake2s.rs:27-30).
__device__ __forceinline__ void channel_mix_message(const uint32_t state[9], const uint32_t root[8], uint32_t m[16]) {
#pragma unroll
  for (int i = 0; i < 8; i++) {
    m[i] = state[i];
    m[8 + i] = root[i];
  }
}
constexpr uint32_t kChannelMixBytes = 64;
__device__ __forceinline__ void channel_after_mix(uint32_t state[9], const uint32_t h[8]) {
#pragma unroll
  for (int i = 0; i < 8; i++) state[i] = h[i];
  state[8] = 0;
}

// draw_secure_felt (blake2s.rs:69-74): the draw Blake2s(digest || n_draws as 4 LE bytes || 0x00)
// (draw_u32s, blake2s.rs:79-97) gives 8 words, each reduced mod P (draw_base_felts), and
// coordinate i is f[2i] + 2 f[2i+1].
__device__ __forceinline__ void channel_draw_message(const uint32_t state[9], uint32_t m[16]) {
#pragma unroll
  for (int i = 0; i < 8; i++) m[i] = state[i];
  m[8] = state[8];
#pragma unroll
  for (int i = 9; i < 16; i++) m[i] = 0;  // the 0x00 domain-separation byte, then padding
}
constexpr uint32_t kChannelDrawBytes = 37;
__device__ __forceinline__ void channel_after_draw(uint32_t state[9], const uint32_t h[8], uint32_t felt[4]) {
  state[8] += 1;
  uint32_t f[8];
#pragma unroll
  for (int i = 0; i < 8; i++) {
    uint32_t w = h[i];
    if (w >= 2 * P) w -= 2 * P;  // w < 2^32 = 2P + 2
    f[i] = m31_reduce_once(w);
  }
#pragma unroll
  for (int i = 0; i < 4; i++) felt[i] = m31_add(f[2 * i], m31_add(f[2 * i + 1], f[2 * i + 1]));
}

__device__ __forceinline__ void channel_mix_root(uint32_t state[9], const uint32_t root[8]) {
  uint32_t m[16], h[8];
  channel_mix_message(state, root, m);
  b2s_init(h);
  b2s_compress(h, m, kChannelMixBytes, 0, true);
  channel_after_mix(state, h);
}

__device__ __forceinline__ void channel_draw_felt(uint32_t state[9], uint32_t felt[4]) {
  uint32_t m[16], h[8];
  channel_draw_message(state, m);
  b2s_init(h);
  b2s_compress(h, m, kChannelDrawBytes, 0, true);
  channel_after_draw(state, h, felt);
}

}  // namespace cs
