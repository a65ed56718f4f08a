// Throughput probe of the integer pipes: the measured denominator for the
// kernels of this library that are bound by integer instructions (the FFT
// butterflies and the Blake2s compressions), next to the measured HBM and
// tensor peaks. Each thread runs 8 independent chains of one operation kind;
// every operation reads another chain's register, so none can be folded away.
//   kind 0: 3-input add (IADD3)      kind 1: 3-input logic (LOP3)
//   kind 2: funnel shift (SHF)       kind 3: multiply-add (IMAD, FMA pipe)
#include "common.cuh"

namespace cs {
namespace {

template <int KIND>
__global__ void __launch_bounds__(256) int_peak_kernel(uint32_t iters, uint32_t x, uint32_t y, uint32_t* out) {
  uint32_t r[8];
#pragma unroll
  for (int j = 0; j < 8; j++) r[j] = threadIdx.x * 0x9e3779b9u + j * 0x85ebca6bu + blockIdx.x;
  for (uint32_t i = 0; i < iters; i++) {
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const uint32_t o = r[(j + 1) & 7];
      if (KIND == 0) r[j] = r[j] + o + x;
      if (KIND == 1) r[j] = (r[j] ^ o) & (x | o);
      if (KIND == 2) r[j] = __funnelshift_l(r[j], o, 7);
      if (KIND == 3) r[j] = r[j] * x + o;
    }
  }
  uint32_t acc = y;
#pragma unroll
  for (int j = 0; j < 8; j++) acc ^= r[j];
  out[blockIdx.x * blockDim.x + threadIdx.x] = acc;
}

}  // namespace
}  // namespace cs

using namespace cs;

extern "C" cs_status cs_int_peak_probe(uint32_t kind, uint32_t blocks, uint32_t iters, uint32_t* d_out,
                                       cs_stream stream) {
  CS_CHECK_ARG(kind <= 3, "int_peak_probe: kind %u outside [0, 3]", kind);
  CS_CHECK_ARG(d_out != nullptr && blocks > 0 && blocks <= 65535, "int_peak_probe: bad arguments");
  cudaStream_t st = to_stream(stream);
  switch (kind) {
    case 0: int_peak_kernel<0><<<blocks, 256, 0, st>>>(iters, 0x3u, 0x5u, d_out); break;
    case 1: int_peak_kernel<1><<<blocks, 256, 0, st>>>(iters, 0x0f0f0f0fu, 0x5u, d_out); break;
    case 2: int_peak_kernel<2><<<blocks, 256, 0, st>>>(iters, 0x3u, 0x5u, d_out); break;
    default: int_peak_kernel<3><<<blocks, 256, 0, st>>>(iters, 0x2545f491u, 0x5u, d_out); break;
  }
  CS_LAUNCHED("int_peak_kernel");
  return CS_OK;
}
