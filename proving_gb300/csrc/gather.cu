// Batched reads of device words for decommitment: every value and hash the
// proof reveals after the queries are drawn, in one launch and one copy back.
// The reference reads them one at a time through Column::at
// (MerkleProverLifted::decommit, crates/stwo/src/prover/vcs_lifted/prover.rs:97-162;
// compute_decommitment_positions_and_witness_evals, crates/stwo/src/prover/fri.rs:408-438).
//
// Request k reads word index[k] of table entry slot[k]. Slots and indices are
// checked against the table's lengths on the host before anything is copied,
// so the kernel only makes in-bounds reads.
#include <algorithm>
#include <cstring>
#include <vector>

#include "common.cuh"

namespace cs {
namespace {

__global__ void gather_kernel(const uint32_t* const* __restrict__ table, const uint32_t* __restrict__ slot,
                              const uint32_t* __restrict__ index, uint32_t n, uint32_t* __restrict__ out) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
    out[k] = table[slot[k]][index[k]];
}

__global__ void gather_runs_kernel(const uint32_t* const* __restrict__ table, const uint32_t* __restrict__ slot,
                                   const uint32_t* __restrict__ index, const uint32_t* __restrict__ offset,
                                   uint32_t n, uint32_t* __restrict__ out) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const uint32_t* src = table[slot[k]] + index[k];
    for (uint32_t o = offset[k], w = 0; o < offset[k + 1]; o++, w++) out[o] = src[w];
  }
}

// This thread's pinned staging buffer of at least `bytes` (grown by doubling, kept across calls):
// the request tables go up and the words come back by DMA from page-locked memory, and a proof's
// decommitment does not fault in fresh host pages each time.
struct PinnedStage {
  uint8_t* p = nullptr;
  size_t cap = 0;
  ~PinnedStage() {
    if (p != nullptr) cudaFreeHost(p);
  }
};

uint8_t* pinned_stage(size_t bytes) {
  thread_local PinnedStage s;
  if (s.cap < bytes) {
    const size_t cap = std::max(bytes, std::max<size_t>(2 * s.cap, 1u << 20));
    if (s.p != nullptr) cudaFreeHost(s.p);
    s.p = nullptr;
    s.cap = 0;
    void* q = nullptr;
    if (cudaMallocHost(&q, cap) != cudaSuccess) return nullptr;
    s.p = static_cast<uint8_t*>(q);
    s.cap = cap;
  }
  return s.p;
}

}  // namespace
}  // namespace cs

using namespace cs;

extern "C" cs_status cs_gather_u32(const uint32_t* const* h_table, const uint64_t* h_lengths, uint32_t n_table,
                                   const uint32_t* h_slot, const uint32_t* h_index, uint32_t n, uint32_t* h_out,
                                   cs_stream stream) {
  if (n == 0) return CS_OK;
  CS_CHECK_ARG(h_table != nullptr && h_lengths != nullptr && h_slot != nullptr && h_index != nullptr &&
                   h_out != nullptr,
               "gather: null pointer");
  CS_CHECK_ARG(n_table > 0, "gather: empty table");
  for (uint32_t t = 0; t < n_table; t++) CS_CHECK_ARG(h_table[t] != nullptr, "gather: table entry %u is null", t);
  for (uint32_t k = 0; k < n; k++) {
    CS_CHECK_ARG(h_slot[k] < n_table, "gather: request %u names slot %u of %u", k, h_slot[k], n_table);
    CS_CHECK_ARG(h_index[k] < h_lengths[h_slot[k]], "gather: request %u reads word %u of a %llu-word entry", k,
                 h_index[k], (unsigned long long)h_lengths[h_slot[k]]);
  }
  // one staging buffer: the table, then slots, indices and results
  const size_t table_bytes = sizeof(void*) * n_table, req_bytes = sizeof(uint32_t) * (size_t)n;
  const size_t in_bytes = table_bytes + 2 * req_bytes;
  uint8_t* host = pinned_stage(in_bytes + req_bytes);
  if (host == nullptr) return from_cuda(cudaErrorMemoryAllocation, "gather: pinned staging buffer");
  std::memcpy(host, h_table, table_bytes);
  std::memcpy(host + table_bytes, h_slot, req_bytes);
  std::memcpy(host + table_bytes + req_bytes, h_index, req_bytes);
  cudaStream_t st = to_stream(stream);
  uint8_t* dev = nullptr;
  CS_CUDA(stream_alloc(reinterpret_cast<void**>(&dev), in_bytes + req_bytes, st));
  cudaError_t e = cudaMemcpyAsync(dev, host, in_bytes, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    const uint32_t blocks = (n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024;
    gather_kernel<<<blocks, 256, 0, st>>>(reinterpret_cast<const uint32_t* const*>(dev),
                                          reinterpret_cast<const uint32_t*>(dev + table_bytes),
                                          reinterpret_cast<const uint32_t*>(dev + table_bytes + req_bytes), n,
                                          reinterpret_cast<uint32_t*>(dev + in_bytes));
    note_launch();
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(host + in_bytes, dev + in_bytes, req_bytes, cudaMemcpyDeviceToHost, st);
  const cudaError_t ef = cudaFreeAsync(dev, st);
  if (e == cudaSuccess) e = ef;
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return from_cuda(e, "gather");
  std::memcpy(h_out, host + in_bytes, req_bytes);
  return CS_OK;
}

namespace cs {

cs_status gather_runs(const uint32_t* const* h_table, const uint64_t* h_lengths, uint32_t n_table,
                      const uint32_t* h_slot, const uint32_t* h_index, const uint32_t* h_offset, uint32_t n,
                      uint32_t* h_out, cudaStream_t st) {
  if (n == 0) return CS_OK;
  CS_CHECK_ARG(n_table > 0 && h_offset[0] == 0, "gather_runs: empty table or offsets not starting at 0");
  for (uint32_t t = 0; t < n_table; t++) CS_CHECK_ARG(h_table[t] != nullptr, "gather_runs: table entry %u is null", t);
  for (uint32_t k = 0; k < n; k++) {
    CS_CHECK_ARG(h_slot[k] < n_table && h_offset[k + 1] >= h_offset[k], "gather_runs: request %u is malformed", k);
    CS_CHECK_ARG((uint64_t)h_index[k] + (h_offset[k + 1] - h_offset[k]) <= h_lengths[h_slot[k]],
                 "gather_runs: request %u reads past its %llu-word entry", k,
                 (unsigned long long)h_lengths[h_slot[k]]);
  }
  const size_t table_bytes = sizeof(void*) * n_table, req_bytes = sizeof(uint32_t) * (size_t)n;
  const size_t off_bytes = sizeof(uint32_t) * ((size_t)n + 1), out_bytes = sizeof(uint32_t) * (size_t)h_offset[n];
  const size_t in_bytes = table_bytes + 2 * req_bytes + off_bytes;
  uint8_t* host = pinned_stage(in_bytes + out_bytes);
  if (host == nullptr) return from_cuda(cudaErrorMemoryAllocation, "gather_runs: pinned staging buffer");
  std::memcpy(host, h_table, table_bytes);
  std::memcpy(host + table_bytes, h_slot, req_bytes);
  std::memcpy(host + table_bytes + req_bytes, h_index, req_bytes);
  std::memcpy(host + table_bytes + 2 * req_bytes, h_offset, off_bytes);
  uint8_t* dev = nullptr;
  CS_CUDA(stream_alloc(reinterpret_cast<void**>(&dev), in_bytes + out_bytes, st));
  cudaError_t e = cudaMemcpyAsync(dev, host, in_bytes, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    const uint32_t blocks = (n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024;
    gather_runs_kernel<<<blocks, 256, 0, st>>>(reinterpret_cast<const uint32_t* const*>(dev),
                                               reinterpret_cast<const uint32_t*>(dev + table_bytes),
                                               reinterpret_cast<const uint32_t*>(dev + table_bytes + req_bytes),
                                               reinterpret_cast<const uint32_t*>(dev + table_bytes + 2 * req_bytes),
                                               n, reinterpret_cast<uint32_t*>(dev + in_bytes));
    note_launch();
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(host + in_bytes, dev + in_bytes, out_bytes, cudaMemcpyDeviceToHost, st);
  const cudaError_t ef = cudaFreeAsync(dev, st);
  if (e == cudaSuccess) e = ef;
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return from_cuda(e, "gather_runs");
  std::memcpy(h_out, host + in_bytes, out_bytes);
  return CS_OK;
}

}  // namespace cs
