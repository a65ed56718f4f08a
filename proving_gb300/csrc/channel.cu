// The Blake2s Fiat-Shamir channel with its state in device memory, so that the
// FRI commit loop (commit a layer, mix its root, draw the folding challenge,
// fold) runs without a round trip to the host per layer. The state is 9 words:
// the 32-byte digest as 8 little-endian words, then the draw counter
// (Blake2sChannel, crates/stwo/src/core/channel/blake2s.rs:16-118).
#include "blake2s.cuh"
#include "common.cuh"
#include "field.cuh"

namespace cs {
namespace {

// Blake2sMerkleChannel::mix_hash (crates/stwo/src/core/vcs_lifted/blake2_merkle.rs:56-58):
// digest <- Blake2s(digest || root), one 64-byte final block; the draw counter restarts
// (Blake2sChannel::update_digest, blake2s.rs:27-30).
__global__ void channel_mix_root_kernel(uint32_t* state, const uint32_t* root) {
  uint32_t m[16], h[8];
#pragma unroll
  for (int i = 0; i < 8; i++) {
    m[i] = state[i];
    m[8 + i] = root[i];
  }
  b2s_init(h);
  b2s_compress(h, m, 64, 0, true);
#pragma unroll
  for (int i = 0; i < 8; i++) state[i] = h[i];
  state[8] = 0;
}

// draw_secure_felt (blake2s.rs:69-74): the draw Blake2s(digest || n_draws as 4 LE bytes || 0x00)
// (draw_u32s, blake2s.rs:79-97) gives 8 words, each reduced mod P (draw_base_felts), and
// coordinate i is f[2i] + 2 f[2i+1].
__global__ void channel_draw_felt_kernel(uint32_t* state, uint32_t* felt) {
  uint32_t m[16], h[8];
#pragma unroll
  for (int i = 0; i < 8; i++) m[i] = state[i];
  m[8] = state[8];
#pragma unroll
  for (int i = 9; i < 16; i++) m[i] = 0;  // the 0x00 domain-separation byte, then padding
  b2s_init(h);
  b2s_compress(h, m, 37, 0, true);
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

}  // namespace
}  // namespace cs

using namespace cs;

extern "C" cs_status cs_channel_mix_root(uint32_t* d_state, const uint32_t* d_root, cs_stream stream) {
  CS_CHECK_ARG(d_state != nullptr && d_root != nullptr, "channel_mix_root: null pointer");
  channel_mix_root_kernel<<<1, 1, 0, to_stream(stream)>>>(d_state, d_root);
  CS_LAUNCHED("channel_mix_root_kernel");
  return CS_OK;
}

extern "C" cs_status cs_channel_draw_secure_felt(uint32_t* d_state, uint32_t* d_felt, cs_stream stream) {
  CS_CHECK_ARG(d_state != nullptr && d_felt != nullptr, "channel_draw_secure_felt: null pointer");
  channel_draw_felt_kernel<<<1, 1, 0, to_stream(stream)>>>(d_state, d_felt);
  CS_LAUNCHED("channel_draw_felt_kernel");
  return CS_OK;
}
