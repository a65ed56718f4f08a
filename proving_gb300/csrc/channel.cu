// The Blake2s Fiat-Shamir channel with its state in device memory, so that the
// FRI commit loop (commit a layer, mix its root, draw the folding challenge,
// fold) runs without a round trip to the host per layer. The state is 9 words:
// the 32-byte digest as 8 little-endian words, then the draw counter
// (Blake2sChannel, crates/stwo/src/core/channel/blake2s.rs:16-118).
#include "channel.cuh"
#include "common.cuh"

namespace cs {
namespace {

__global__ void channel_mix_root_kernel(uint32_t* state, const uint32_t* root) {
  uint32_t s[9], r[8];
#pragma unroll
  for (int i = 0; i < 9; i++) s[i] = state[i];
#pragma unroll
  for (int i = 0; i < 8; i++) r[i] = root[i];
  channel_mix_root(s, r);
#pragma unroll
  for (int i = 0; i < 9; i++) state[i] = s[i];
}

__global__ void channel_draw_felt_kernel(uint32_t* state, uint32_t* felt) {
  uint32_t s[9], f[4];
#pragma unroll
  for (int i = 0; i < 9; i++) s[i] = state[i];
  channel_draw_felt(s, f);
  state[8] = s[8];
#pragma unroll
  for (int i = 0; i < 4; i++) felt[i] = f[i];
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
