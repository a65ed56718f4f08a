// Shared helpers for the C-ABI: status codes, the per-thread error message,
// launch checks and the batch size of column-pointer tables passed by value.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <string>

#include "stwo_cuda.h"

namespace cs {

// Column-pointer tables travel as kernel parameters (no device allocation);
// larger batches are split into several launches by the host wrappers.
constexpr int kMaxBatch = 256;
// Per-device set-up flags (kernel attributes, pool settings) are kept for this many ordinals.
constexpr int kMaxDevices = 64;

// 16-byte alignment of a device pointer, for kernels that move whole digests or tiles as uint4.
inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

void set_error(const char* fmt, ...);
// Counts kernel launches made by this library (reported by cs_kernel_launch_count).
void note_launch();
cs_status from_cuda(cudaError_t e, const char* what);
// cudaMallocAsync from the device's default pool, which first (once per device) is set to keep
// the memory freed back to it instead of returning it to the driver at every synchronisation:
// the scratch and proof buffers of one call are reused by the next without remapping.
cudaError_t stream_alloc(void** ptr, size_t bytes, cudaStream_t st);

inline cudaStream_t to_stream(cs_stream s) { return reinterpret_cast<cudaStream_t>(s); }

// Reads of runs of device words in one launch and one copy back (gather.cu): request k copies
// words [index[k], index[k] + offset[k+1] - offset[k]) of table entry slot[k] to out[offset[k] ..];
// offset has n + 1 entries, offset[n] words in all. Every run is checked against its entry's length
// on the host first. Synchronous on st.
cs_status gather_runs(const uint32_t* const* h_table, const uint64_t* h_lengths, uint32_t n_table,
                      const uint32_t* h_slot, const uint32_t* h_index, const uint32_t* h_offset, uint32_t n,
                      uint32_t* h_out, cudaStream_t st);

inline uint32_t subgroup_gen(uint32_t log_size) { return 1u << (31 - log_size); }

}  // namespace cs

#define CS_CHECK_ARG(cond, ...)            \
  do {                                     \
    if (!(cond)) {                         \
      cs::set_error(__VA_ARGS__);          \
      return CS_ERR_INVALID_ARG;           \
    }                                      \
  } while (0)

#define CS_CUDA(call)                                         \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) return cs::from_cuda(e_, #call);   \
  } while (0)

#define CS_LAUNCHED(name)                                           \
  do {                                                              \
    cs::note_launch();                                              \
    cudaError_t e_ = cudaGetLastError();                            \
    if (e_ != cudaSuccess) return cs::from_cuda(e_, "launch " name); \
  } while (0)
