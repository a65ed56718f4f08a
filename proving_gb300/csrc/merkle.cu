// Lifted Blake2s Merkle trees on sm_103a.
//
// Leaves: crates/stwo/src/prover/backend/cpu/merkle_lifted.rs:46-90 — leaf i
// hashes, in column order (columns sorted by length), the LE bytes of
// col[(i >> (L - l + 1) << 1) + (i & 1)]; 16 columns fill one 64-byte Blake2s
// block. One thread per leaf: a warp reads 32 consecutive words of a column
// (coalesced), the 16 words of a block are loaded before the block is
// compressed, and the chaining value stays in registers.
// Nodes: merkle_lifted.rs:92-97 / crates/stwo/src/core/vcs_lifted/blake2_merkle.rs:29-36,
// node = Blake2s(left || right), one 64-byte final block per node.
#include <algorithm>
#include <numeric>
#include <vector>

#include "blake2s.cuh"
#include "common.cuh"

namespace cs {

namespace {

constexpr uint32_t kMaxLeafCols = 2048;
constexpr int kLeafThreads = 128;

struct LeafParams {
  const uint32_t* cols[kMaxLeafCols];
  uint8_t shift[kMaxLeafCols];  // L - l + 1
  uint32_t n_cols;
  uint32_t log_leaves;
  uint32_t one;  // 1, opaque to the compiler (see b2s_compress)
};

__global__ void __launch_bounds__(kLeafThreads) merkle_leaves_kernel(const __grid_constant__ LeafParams p,
                                                                     uint32_t* __restrict__ out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (1u << p.log_leaves)) return;
  uint32_t h[8];
  b2s_init(h);
  uint32_t m[16];
  const uint32_t n_cols = p.n_cols;
  if (n_cols == 0) {
#pragma unroll
    for (int k = 0; k < 16; k++) m[k] = 0;
    b2s_compress(h, m, 0, 0, true);
  } else {
    const uint32_t n_blocks = (n_cols + 15) >> 4;
    for (uint32_t b = 0; b < n_blocks; b++) {
      const uint32_t base = b << 4;
      const bool last = b + 1 == n_blocks;
      const uint32_t cnt = last ? n_cols - base : 16;
#pragma unroll
      for (int k = 0; k < 16; k++) {
        uint32_t v = 0;
        if ((uint32_t)k < cnt) {
          const uint32_t c = base + k;
          const uint32_t s = p.shift[c];
          const uint32_t idx = ((i >> s) << 1) | (i & 1);
          v = __ldg(p.cols[c] + idx);
        }
        m[k] = v;
      }
      b2s_compress(h, m, (base + cnt) * 4, 0, last, p.one);
    }
  }
  uint4* o = reinterpret_cast<uint4*>(out + (size_t)i * 8);
  o[0] = make_uint4(h[0], h[1], h[2], h[3]);
  o[1] = make_uint4(h[4], h[5], h[6], h[7]);
}

__global__ void merkle_node_kernel(const uint32_t* __restrict__ prev, uint32_t log_out, uint32_t* __restrict__ out,
                                   uint32_t one) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (1u << log_out)) return;
  const uint4* src = reinterpret_cast<const uint4*>(prev + (size_t)i * 16);
  uint32_t m[16];
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const uint4 q = __ldg(src + k);
    m[4 * k] = q.x;
    m[4 * k + 1] = q.y;
    m[4 * k + 2] = q.z;
    m[4 * k + 3] = q.w;
  }
  uint32_t h[8];
  b2s_init(h);
  b2s_compress(h, m, 64, 0, true, one);
  uint4* o = reinterpret_cast<uint4*>(out + (size_t)i * 8);
  o[0] = make_uint4(h[0], h[1], h[2], h[3]);
  o[1] = make_uint4(h[4], h[5], h[6], h[7]);
}

}  // namespace

cs_status merkle_leaves(const uint32_t* const* cols, const uint32_t* log_sizes, uint32_t n_cols, uint32_t L,
                        uint32_t* d_leaves, cudaStream_t st) {
  CS_CHECK_ARG(n_cols <= kMaxLeafCols, "build_leaves: %u columns exceed the limit of %u", n_cols, kMaxLeafCols);
  CS_CHECK_ARG(n_cols > 0 || L == 0, "build_leaves: an empty tree must have lifting_log_size 0 (got %u)", L);
  CS_CHECK_ARG(L <= 30, "build_leaves: lifting_log_size %u too large", L);
  CS_CHECK_ARG(d_leaves != nullptr, "build_leaves: null output");
  static thread_local LeafParams p;
  p.n_cols = n_cols;
  p.log_leaves = n_cols == 0 ? 0 : L;
  p.one = 1;
  uint32_t prev = 0;
  for (uint32_t c = 0; c < n_cols; c++) {
    CS_CHECK_ARG(cols[c] != nullptr, "build_leaves: column %u is null", c);
    const uint32_t l = log_sizes[c];
    CS_CHECK_ARG(l >= 1 && l <= L, "build_leaves: column %u has log size %u outside [1, %u]", c, l, L);
    CS_CHECK_ARG(l >= prev, "build_leaves: columns must be sorted by length (column %u)", c);
    prev = l;
    p.cols[c] = cols[c];
    p.shift[c] = (uint8_t)(L - l + 1);
  }
  const uint32_t n = 1u << p.log_leaves;
  merkle_leaves_kernel<<<(n + kLeafThreads - 1) / kLeafThreads, kLeafThreads, 0, st>>>(p, d_leaves);
  CS_LAUNCHED("merkle_leaves_kernel");
  return CS_OK;
}

cs_status merkle_next_layer(const uint32_t* d_prev, uint32_t log_out, uint32_t* d_out, cudaStream_t st) {
  CS_CHECK_ARG(d_prev != nullptr && d_out != nullptr, "build_next_layer: null buffer");
  CS_CHECK_ARG(log_out <= 29, "build_next_layer: log size %u too large", log_out);
  const uint32_t n = 1u << log_out;
  const uint32_t threads = 128;
  merkle_node_kernel<<<(n + threads - 1) / threads, threads, 0, st>>>(d_prev, log_out, d_out, 1u);
  CS_LAUNCHED("merkle_node_kernel");
  return CS_OK;
}

}  // namespace cs

using namespace cs;

extern "C" cs_status cs_merkle_build_leaves(const uint32_t* const* h_cols, const uint32_t* h_log_sizes,
                                            uint32_t n_cols, uint32_t lifting_log_size, uint32_t* d_leaves,
                                            cs_stream stream) {
  CS_CHECK_ARG(n_cols == 0 || (h_cols != nullptr && h_log_sizes != nullptr), "build_leaves: null column table");
  return merkle_leaves(h_cols, h_log_sizes, n_cols, lifting_log_size, d_leaves, to_stream(stream));
}

extern "C" cs_status cs_merkle_build_next_layer(const uint32_t* d_prev, uint32_t out_log_size, uint32_t* d_out,
                                                cs_stream stream) {
  return merkle_next_layer(d_prev, out_log_size, d_out, to_stream(stream));
}

extern "C" cs_status cs_merkle_commit(const uint32_t* const* h_cols, const uint32_t* h_log_sizes, uint32_t n_cols,
                                      uint32_t lifting_log_size, uint32_t* d_layers, cs_stream stream) {
  CS_CHECK_ARG(n_cols == 0 || (h_cols != nullptr && h_log_sizes != nullptr), "commit: null column table");
  CS_CHECK_ARG(n_cols <= kMaxLeafCols, "commit: %u columns exceed the limit of %u", n_cols, kMaxLeafCols);
  // Stable sort by length (crates/stwo/src/prover/vcs_lifted/prover.rs:68).
  std::vector<uint32_t> order(n_cols);
  std::iota(order.begin(), order.end(), 0u);
  std::stable_sort(order.begin(), order.end(),
                   [&](uint32_t a, uint32_t b) { return h_log_sizes[a] < h_log_sizes[b]; });
  std::vector<const uint32_t*> cols(n_cols);
  std::vector<uint32_t> logs(n_cols);
  for (uint32_t i = 0; i < n_cols; i++) {
    cols[i] = h_cols[order[i]];
    logs[i] = h_log_sizes[order[i]];
  }
  cudaStream_t st = to_stream(stream);
  cs_status s = merkle_leaves(cols.data(), logs.data(), n_cols, lifting_log_size, d_layers, st);
  if (s != CS_OK) return s;
  uint32_t* cur = d_layers;
  for (uint32_t k = lifting_log_size; k >= 1; k--) {
    uint32_t* next = cur + ((size_t)8 << k);
    s = merkle_next_layer(cur, k - 1, next, st);
    if (s != CS_OK) return s;
    cur = next;
  }
  return CS_OK;
}
