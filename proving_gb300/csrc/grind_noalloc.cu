// Proof-of-work search that allocates no device memory.
//
// cs_grind_blake2s takes an 8-byte best-nonce slot from the stream-ordered
// allocator on every call. Some callers cannot allocate: a prover embedded in
// a service whose device memory is carved up front into a fixed arena (where
// any cudaMalloc may fail or stall the device), or code that must not
// introduce allocation calls into a stream it does not own. This variant
// keeps its slots in a file-scope __device__ array instead, so a call makes
// no cudaMalloc, cudaFree, cudaMallocAsync or allocating library call.
//
// The array holds kNoAllocMaxDigests slots (512 bytes) and stays resident on
// every GPU that loads this library until the process exits. Host code cannot
// use the array's name as a device address, so the first call on each device
// (with that device current) looks the address up with cudaGetSymbolAddress
// and caches it; make that first call before any stream capture. The cached
// address belongs to the device's current context: cudaDeviceReset unloads
// this module, so after a reset of a device the process must not call this
// entry point on that device again. Every call
// shares the array and re-initialises the slots it uses before each search
// round, so calls that overlap on the GPU (e.g. on two streams) race on it.
#include <mutex>

#include "common.cuh"
#include "grind.cuh"

namespace cs {

namespace {

constexpr uint32_t kNoAllocMaxDigests = 64;

__device__ __align__(256) unsigned long long g_grind_slots[kNoAllocMaxDigests];

std::mutex g_slot_mutex;
unsigned long long* g_slot_ptr[kMaxDevices] = {};

cs_status slots_on_current_device(unsigned long long** out) {
  int dev = -1;
  CS_CUDA(cudaGetDevice(&dev));
  CS_CHECK_ARG(dev >= 0 && dev < kMaxDevices, "grind_noalloc: device ordinal %d not supported", dev);
  std::lock_guard<std::mutex> lock(g_slot_mutex);
  if (g_slot_ptr[dev] == nullptr) {
    void* p = nullptr;
    CS_CUDA(cudaGetSymbolAddress(&p, g_grind_slots));
    g_slot_ptr[dev] = static_cast<unsigned long long*>(p);
  }
  *out = g_slot_ptr[dev];
  return CS_OK;
}

}  // namespace
}  // namespace cs

using namespace cs;

extern "C" cs_status cs_grind_blake2s_noalloc(const uint8_t* digests, uint32_t n_digests, uint32_t pow_bits,
                                              uint64_t max_nonce, uint64_t* nonces_out, cs_stream stream) {
  CS_CHECK_ARG(digests != nullptr && nonces_out != nullptr, "grind_noalloc: null digests or output");
  CS_CHECK_ARG(n_digests >= 1 && n_digests <= kNoAllocMaxDigests,
               "grind_noalloc: %u digests requested, the static scratch holds at most %u", n_digests,
               kNoAllocMaxDigests);
  CS_CHECK_ARG(pow_bits <= 32, "grind_noalloc: pow_bits %u > 32 is not supported", pow_bits);
  unsigned long long* slots = nullptr;
  cs_status s = slots_on_current_device(&slots);
  if (s != CS_OK) return s;
  cudaStream_t st = to_stream(stream);
  for (uint32_t i = 0; i < n_digests; i++) {
    s = grind_with_slot(digests + 32 * (size_t)i, pow_bits, max_nonce, nonces_out + i, slots + i, st);
    if (s != CS_OK) return s;
  }
  return CS_OK;
}
