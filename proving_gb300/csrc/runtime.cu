// Runtime part of the C ABI: error reporting, device memory and copies.
#include <atomic>
#include <cstdint>
#include <mutex>
#include <cstdarg>
#include <cstdio>
#include <string>

#include "common.cuh"

namespace cs {

namespace {
thread_local std::string g_last_error;
std::atomic<uint64_t> g_launches{0};
}

void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

cudaError_t stream_alloc(void** ptr, size_t bytes, cudaStream_t st) {
  static std::mutex mu;
  static bool done[64] = {false};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev >= 0 && dev < 64) {
    std::lock_guard<std::mutex> lock(mu);
    if (!done[dev]) {
      cudaMemPool_t pool;
      if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        uint64_t keep = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
      }
      done[dev] = true;
    }
  }
  return cudaMallocAsync(ptr, bytes, st);
}

void set_error(const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
}

cs_status from_cuda(cudaError_t e, const char* what) {
  set_error("%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
  if (e == cudaErrorMemoryAllocation) return CS_ERR_OOM;
  if (e == cudaErrorInvalidValue) return CS_ERR_INVALID_ARG;
  return CS_ERR_DEVICE;
}

const char* last_error() { return g_last_error.c_str(); }

}  // namespace cs

using namespace cs;

extern "C" const char* cs_last_error(void) { return last_error(); }

extern "C" const char* cs_version(void) { return "stwo-cuda 0.1 sm_103a"; }

extern "C" uint64_t cs_kernel_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

extern "C" cs_status cs_malloc(void** d_ptr, size_t bytes) {
  CS_CHECK_ARG(d_ptr != nullptr, "malloc: null output pointer");
  *d_ptr = nullptr;
  if (bytes == 0) return CS_OK;
  CS_CUDA(cudaMalloc(d_ptr, bytes));
  return CS_OK;
}

extern "C" cs_status cs_free(void* d_ptr) {
  if (d_ptr == nullptr) return CS_OK;
  CS_CUDA(cudaFree(d_ptr));
  return CS_OK;
}

extern "C" cs_status cs_memset_zero(void* d_ptr, size_t bytes, cs_stream stream) {
  if (bytes == 0) return CS_OK;
  CS_CHECK_ARG(d_ptr != nullptr, "memset: null pointer");
  CS_CUDA(cudaMemsetAsync(d_ptr, 0, bytes, to_stream(stream)));
  return CS_OK;
}

extern "C" cs_status cs_memcpy_h2d(void* d_dst, const void* h_src, size_t bytes, cs_stream stream) {
  if (bytes == 0) return CS_OK;
  CS_CHECK_ARG(d_dst != nullptr && h_src != nullptr, "memcpy_h2d: null pointer");
  CS_CUDA(cudaMemcpyAsync(d_dst, h_src, bytes, cudaMemcpyHostToDevice, to_stream(stream)));
  return CS_OK;
}

extern "C" cs_status cs_memcpy_d2h(void* h_dst, const void* d_src, size_t bytes, cs_stream stream) {
  if (bytes == 0) return CS_OK;
  CS_CHECK_ARG(h_dst != nullptr && d_src != nullptr, "memcpy_d2h: null pointer");
  CS_CUDA(cudaMemcpyAsync(h_dst, d_src, bytes, cudaMemcpyDeviceToHost, to_stream(stream)));
  return CS_OK;
}

extern "C" cs_status cs_memcpy_d2d(void* d_dst, const void* d_src, size_t bytes, cs_stream stream) {
  if (bytes == 0) return CS_OK;
  CS_CHECK_ARG(d_dst != nullptr && d_src != nullptr, "memcpy_d2d: null pointer");
  CS_CUDA(cudaMemcpyAsync(d_dst, d_src, bytes, cudaMemcpyDeviceToDevice, to_stream(stream)));
  return CS_OK;
}

extern "C" cs_status cs_stream_synchronize(cs_stream stream) {
  CS_CUDA(cudaStreamSynchronize(to_stream(stream)));
  return CS_OK;
}
