// Batched reads of device words for decommitment: every value and hash the
// proof reveals after the queries are drawn, in one launch and one copy back.
// The reference reads them one at a time through Column::at
// (MerkleProverLifted::decommit, crates/stwo/src/prover/vcs_lifted/prover.rs:97-162;
// compute_decommitment_positions_and_witness_evals, crates/stwo/src/prover/fri.rs:408-438).
//
// Request k reads word index[k] of table entry slot[k]. Slots and indices are
// checked against the table's lengths on the host before anything is copied,
// so the kernel only makes in-bounds reads.
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
  std::vector<uint8_t> host(in_bytes);
  std::memcpy(host.data(), h_table, table_bytes);
  std::memcpy(host.data() + table_bytes, h_slot, req_bytes);
  std::memcpy(host.data() + table_bytes + req_bytes, h_index, req_bytes);
  cudaStream_t st = to_stream(stream);
  uint8_t* dev = nullptr;
  CS_CUDA(stream_alloc(reinterpret_cast<void**>(&dev), in_bytes + req_bytes, st));
  cudaError_t e = cudaMemcpyAsync(dev, host.data(), in_bytes, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    const uint32_t blocks = (n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024;
    gather_kernel<<<blocks, 256, 0, st>>>(reinterpret_cast<const uint32_t* const*>(dev),
                                          reinterpret_cast<const uint32_t*>(dev + table_bytes),
                                          reinterpret_cast<const uint32_t*>(dev + table_bytes + req_bytes), n,
                                          reinterpret_cast<uint32_t*>(dev + in_bytes));
    note_launch();
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(h_out, dev + in_bytes, req_bytes, cudaMemcpyDeviceToHost, st);
  const cudaError_t ef = cudaFreeAsync(dev, st);
  if (e == cudaSuccess) e = ef;
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return from_cuda(e, "gather");
  return CS_OK;
}
