// Lifted Blake2s Merkle trees on sm_103a.
//
// Leaves: crates/stwo/src/prover/backend/cpu/merkle_lifted.rs:46-90 — leaf i
// hashes, in column order (columns sorted by length), the LE bytes of
// col[(i >> (L - l + 1) << 1) + (i & 1)]; 16 columns fill one 64-byte Blake2s
// block. The lift of a leaf index to a shorter column is the composition of
// the lifts through every intermediate size, so the chaining value after a
// prefix of blocks whose columns are all of log size <= l depends only on the
// leaf's lift to size l. Blocks are therefore compressed at the smallest size
// that determines them (the largest log size among their 16 columns; the
// final block at the tree height): one launch per such size, one thread per
// index at that size, chaining values handed up through a pair of state
// buffers (the same prefix sharing as blake2s_lifted.rs:46-200 in the SIMD
// backend). A warp reads 32 consecutive words of a column of its own size
// (coalesced), shorter columns through the cache. With columns of one size
// this is a single launch at the tree height.
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
  uint8_t log[kMaxLeafCols];  // column log sizes (sorted)
  uint32_t n_cols;
  uint32_t level_log;            // the blocks of this launch are determined by the lift to this size
  uint32_t prev_log;             // size of prev_state's indices
  uint32_t block0, block1;       // blocks [block0, block1) of 16 columns
  uint32_t is_final;             // block1 - 1 is the message's final block; out receives digests
  const uint32_t* prev_state;    // chaining values after blocks [0, block0), or null (initial value)
  uint32_t one;                  // 1, opaque to the compiler (see b2s_compress)
};

// Index of leaf-lift x (at log size `from`) in a column or state of log size `to` <= from.
__device__ __forceinline__ uint32_t lift_index(uint32_t x, uint32_t from, uint32_t to) {
  return from == to ? x : (((x >> (from - to + 1)) << 1) | (x & 1));
}

__global__ void __launch_bounds__(kLeafThreads) merkle_leaves_kernel(const __grid_constant__ LeafParams p,
                                                                     uint32_t* __restrict__ out) {
  const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= (1u << p.level_log)) return;
  uint32_t h[8];
  uint32_t m[16];
  if (p.n_cols == 0) {
    b2s_init(h);
#pragma unroll
    for (int k = 0; k < 16; k++) m[k] = 0;
    b2s_compress(h, m, 0, 0, true);
  } else {
    if (p.prev_state != nullptr) {
      const uint4* src = reinterpret_cast<const uint4*>(p.prev_state + (size_t)lift_index(x, p.level_log, p.prev_log) * 8);
      const uint4 a = __ldg(src), b = __ldg(src + 1);
      h[0] = a.x; h[1] = a.y; h[2] = a.z; h[3] = a.w;
      h[4] = b.x; h[5] = b.y; h[6] = b.z; h[7] = b.w;
    } else {
      b2s_init(h);
    }
    for (uint32_t b = p.block0; b < p.block1; b++) {
      const uint32_t base = b << 4;
      const bool last = p.is_final && b + 1 == p.block1;
      const uint32_t cnt = min(16u, p.n_cols - base);
#pragma unroll
      for (int k = 0; k < 16; k++) {
        uint32_t v = 0;
        if ((uint32_t)k < cnt) {
          const uint32_t c = base + k;
          v = __ldg(p.cols[c] + lift_index(x, p.level_log, p.log[c]));
        }
        m[k] = v;
      }
      b2s_compress(h, m, (base + cnt) * 4, 0, last, p.one);
    }
  }
  uint4* o = reinterpret_cast<uint4*>(out + (size_t)x * 8);
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

// The top layers of a tree in one launch: one block builds layers log_in - 1 down to 0 from the
// layer of 2^log_in digests at `layer`, each written right after the one before it (the layout of
// cs_merkle_commit), with a barrier between layers. Plain loads, since each layer reads what the
// block wrote for the previous one; the barrier makes those stores visible to the block.
constexpr uint32_t kTopLayersLog = 10;  // layers of up to 2^10 nodes

__global__ void __launch_bounds__(1024) merkle_top_kernel(uint32_t* layer, uint32_t log_in, uint32_t one) {
  const uint32_t* prev = layer;
  uint32_t* out = layer + ((size_t)8 << log_in);
  for (int k = (int)log_in - 1; k >= 0; k--) {
    for (uint32_t i = threadIdx.x; i < (1u << k); i += blockDim.x) {
      const uint4* src = reinterpret_cast<const uint4*>(prev + (size_t)i * 16);
      uint32_t m[16];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const uint4 w = src[q];
        m[4 * q] = w.x;
        m[4 * q + 1] = w.y;
        m[4 * q + 2] = w.z;
        m[4 * q + 3] = w.w;
      }
      uint32_t h[8];
      b2s_init(h);
      b2s_compress(h, m, 64, 0, true, one);
      uint4* o = reinterpret_cast<uint4*>(out + (size_t)i * 8);
      o[0] = make_uint4(h[0], h[1], h[2], h[3]);
      o[1] = make_uint4(h[4], h[5], h[6], h[7]);
    }
    __syncthreads();
    prev = out;
    out += (size_t)8 << k;
  }
}

}  // namespace

cs_status merkle_leaves(const uint32_t* const* cols, const uint32_t* log_sizes, uint32_t n_cols, uint32_t L,
                        uint32_t* d_leaves, cudaStream_t st) {
  CS_CHECK_ARG(n_cols <= kMaxLeafCols, "build_leaves: %u columns exceed the limit of %u", n_cols, kMaxLeafCols);
  CS_CHECK_ARG(n_cols > 0 || L == 0, "build_leaves: an empty tree must have lifting_log_size 0 (got %u)", L);
  CS_CHECK_ARG(L <= 30, "build_leaves: lifting_log_size %u too large", L);
  CS_CHECK_ARG(d_leaves != nullptr, "build_leaves: null output");
  CS_CHECK_ARG(aligned16(d_leaves), "build_leaves: output not 16-byte aligned (digests are written as 16-byte words)");
  static thread_local LeafParams p;
  p.n_cols = n_cols;
  p.one = 1;
  uint32_t prev = 0;
  for (uint32_t c = 0; c < n_cols; c++) {
    CS_CHECK_ARG(cols[c] != nullptr, "build_leaves: column %u is null", c);
    const uint32_t l = log_sizes[c];
    CS_CHECK_ARG(l >= 1 && l <= L, "build_leaves: column %u has log size %u outside [1, %u]", c, l, L);
    CS_CHECK_ARG(l >= prev, "build_leaves: columns must be sorted by length (column %u)", c);
    prev = l;
    p.cols[c] = cols[c];
    p.log[c] = (uint8_t)l;
  }
  // launches: runs of non-final blocks by the size that determines them (the log size of their
  // last column), then the final block (and any non-final blocks of the tree height) at L
  const uint32_t n_blocks = n_cols == 0 ? 1 : (n_cols + 15) / 16;
  struct Run {
    uint32_t level, b0, b1;
  };
  std::vector<Run> runs;
  for (uint32_t b = 0; b + 1 < n_blocks; b++) {
    const uint32_t level = log_sizes[16 * b + 15];
    if (level == L) break;
    if (!runs.empty() && runs.back().level == level)
      runs.back().b1 = b + 1;
    else
      runs.push_back({level, b, b + 1});
  }
  const uint32_t top_b0 = runs.empty() ? 0 : runs.back().b1;
  uint32_t* states = nullptr;
  size_t half = 0;  // words per state buffer
  if (!runs.empty()) {
    uint32_t max_level = 0;
    for (const Run& r : runs) max_level = std::max(max_level, r.level);
    half = (size_t)8 << max_level;
    CS_CUDA(stream_alloc(reinterpret_cast<void**>(&states), sizeof(uint32_t) * 2 * half, st));
  }
  cs_status result = CS_OK;
  const uint32_t* prev_state = nullptr;
  uint32_t prev_log = 0;
  for (size_t r = 0; r <= runs.size() && result == CS_OK; r++) {
    const bool top = r == runs.size();
    p.level_log = top ? (n_cols == 0 ? 0 : L) : runs[r].level;
    p.block0 = top ? top_b0 : runs[r].b0;
    p.block1 = top ? n_blocks : runs[r].b1;
    p.is_final = top ? 1 : 0;
    p.prev_state = prev_state;
    p.prev_log = prev_log;
    uint32_t* dst = top ? d_leaves : states + (r & 1) * half;
    const uint32_t n = 1u << p.level_log;
    merkle_leaves_kernel<<<(n + kLeafThreads - 1) / kLeafThreads, kLeafThreads, 0, st>>>(p, dst);
    note_launch();
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) result = from_cuda(e, "merkle_leaves_kernel");
    prev_state = dst;
    prev_log = p.level_log;
  }
  if (states != nullptr) {
    const cudaError_t e = cudaFreeAsync(states, st);
    if (result == CS_OK && e != cudaSuccess) return from_cuda(e, "cudaFreeAsync");
  }
  return result;
}

cs_status merkle_next_layer(const uint32_t* d_prev, uint32_t log_out, uint32_t* d_out, cudaStream_t st) {
  CS_CHECK_ARG(d_prev != nullptr && d_out != nullptr, "build_next_layer: null buffer");
  CS_CHECK_ARG(log_out <= 29, "build_next_layer: log size %u too large", log_out);
  CS_CHECK_ARG(aligned16(d_prev) && aligned16(d_out),
               "build_next_layer: layers must be 16-byte aligned (digests move as 16-byte words)");
  const uint32_t n = 1u << log_out;
  const uint32_t threads = 128;
  merkle_node_kernel<<<(n + threads - 1) / threads, threads, 0, st>>>(d_prev, log_out, d_out, 1u);
  CS_LAUNCHED("merkle_node_kernel");
  return CS_OK;
}

// Every node layer above the 2^L leaves at d_layers, each right after the one before (leaves
// first, root last): one launch per layer of more than 2^10 nodes, then the rest in one.
cs_status merkle_layers(uint32_t* d_layers, uint32_t L, cudaStream_t st) {
  uint32_t* cur = d_layers;
  for (uint32_t k = L; k >= 1; k--) {
    if (k - 1 <= kTopLayersLog) {
      const uint32_t threads = std::max(32u, std::min(1024u, 1u << (k - 1)));
      merkle_top_kernel<<<1, threads, 0, st>>>(cur, k, 1u);
      CS_LAUNCHED("merkle_top_kernel");
      break;
    }
    uint32_t* next = cur + ((size_t)8 << k);
    const cs_status s = merkle_next_layer(cur, k - 1, next, st);
    if (s != CS_OK) return s;
    cur = next;
  }
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

extern "C" cs_status cs_merkle_build_layers(uint32_t* d_layers, uint32_t lifting_log_size, cs_stream stream) {
  CS_CHECK_ARG(d_layers != nullptr, "build_layers: null buffer");
  CS_CHECK_ARG(lifting_log_size <= 30, "build_layers: log size %u too large", lifting_log_size);
  CS_CHECK_ARG(aligned16(d_layers), "build_layers: layers must be 16-byte aligned (digests move as 16-byte words)");
  return merkle_layers(d_layers, lifting_log_size, to_stream(stream));
}

extern "C" cs_status cs_merkle_commit(const uint32_t* const* h_cols, const uint32_t* h_log_sizes, uint32_t n_cols,
                                      uint32_t lifting_log_size, uint32_t* d_layers, cs_stream stream) {
  CS_CHECK_ARG(n_cols == 0 || (h_cols != nullptr && h_log_sizes != nullptr), "commit: null column table");
  CS_CHECK_ARG(n_cols <= kMaxLeafCols, "commit: %u columns exceed the limit of %u", n_cols, kMaxLeafCols);
  CS_CHECK_ARG(d_layers != nullptr && aligned16(d_layers),
               "commit: layers must be non-null and 16-byte aligned (digests move as 16-byte words)");
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
  return merkle_layers(d_layers, lifting_log_size, st);
}
