// The last LogUp interaction column, shared by the LogUp producers.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

#include "stwo_cuda.h"

namespace cs {

// A QM31 column as its four coordinate arrays.
struct Q4 {
  uint32_t* c[4];
};

// LogupTraceGenerator::finalize_last (crates/constraint-framework/src/prover/logup.rs:96-130)
// in place on `col`, which holds each row's fraction total (2^log_size values, bit-reversed
// circle-domain order, log_size >= 1): claimed_sum = the sum of the column (returned on the
// host, the call synchronizes `st` once), then every value minus claimed_sum / n,
// inclusive-prefix-summed in coset order. Uses stream-ordered device scratch.
cs_status logup_finalize_last(Q4 col, uint32_t log_size, uint32_t claimed_sum_out[4], cudaStream_t st);

}  // namespace cs
