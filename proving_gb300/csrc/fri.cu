// FRI folds and leaf packing on sm_103a. Pure HBM streaming: each thread reads
// one (f(x), f(-x)) pair per coordinate as an 8-byte load and writes one QM31.
//
// fold_line: crates/stwo/src/prover/backend/cpu/fri.rs:66-91 — on the line
// domain x(half_odds(n)), pair i sits at x = domain.at(bitrev(2i, n)); its
// inverse is itwiddle tree word 2^K - 2^n + i (the tree layer of that coset).
// fold_circle_into_line: cpu/fri.rs:94-116 — pair i is (p, -p) with
// p = domain.at(bitrev(2i, n)); 1/p.y is the circle-layer itwiddle of the
// domain: from line layer 1 (tree offset 2^K - 2^(n-1)) pick
// [1/y, -1/y, -1/x, 1/x][i & 3] of pair (i >> 2)
// (circle_twiddles_from_line_twiddles, cpu/circle.rs:306-323).
#include <algorithm>

#include "common.cuh"
#include "field.cuh"

namespace cs {

namespace {

struct Coords {
  const uint32_t* in[4];
  uint32_t* out[4];
};

__device__ __forceinline__ qm31 load_pair(const Coords& c, uint32_t i, qm31& f1) {
  uint2 a = __ldg(reinterpret_cast<const uint2*>(c.in[0]) + i);
  uint2 b = __ldg(reinterpret_cast<const uint2*>(c.in[1]) + i);
  uint2 cc = __ldg(reinterpret_cast<const uint2*>(c.in[2]) + i);
  uint2 d = __ldg(reinterpret_cast<const uint2*>(c.in[3]) + i);
  f1 = qm31_make(a.y, b.y, cc.y, d.y);
  return qm31_make(a.x, b.x, cc.x, d.x);
}

__device__ __forceinline__ void store(const Coords& c, uint32_t i, qm31 v) {
  c.out[0][i] = v.a.a;
  c.out[1][i] = v.a.b;
  c.out[2][i] = v.b.a;
  c.out[3][i] = v.b.b;
}

__device__ __forceinline__ void qm31_ibfly(qm31& v0, qm31& v1, uint32_t t) {
  const qm31 tmp = v0;
  v0 = qm31_add(tmp, v1);
  v1 = qm31_mul_m31(qm31_sub(tmp, v1), t);
}

// alpha_dev: when not null, the folding challenge is read from device memory (4 words), where a
// device-resident channel drew it; otherwise `alpha` is used.
__device__ __forceinline__ qm31 challenge(qm31 alpha, const uint32_t* alpha_dev) {
  return alpha_dev ? qm31_make(__ldg(alpha_dev), __ldg(alpha_dev + 1), __ldg(alpha_dev + 2), __ldg(alpha_dev + 3))
                   : alpha;
}

__global__ void fold_line_kernel(const Coords c, uint32_t half, const uint32_t* __restrict__ itw_layer, qm31 alpha_h,
                                 const uint32_t* alpha_dev) {
  const qm31 alpha = challenge(alpha_h, alpha_dev);
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < half; i += gridDim.x * blockDim.x) {
    qm31 f1;
    qm31 f0 = load_pair(c, i, f1);
    qm31_ibfly(f0, f1, __ldg(itw_layer + i));
    store(c, i, qm31_add(f0, qm31_mul(alpha, f1)));
  }
}

__global__ void fold_circle_kernel(const Coords c, uint32_t half, const uint32_t* __restrict__ lt1, qm31 alpha_h,
                                   const uint32_t* alpha_dev) {
  const qm31 alpha = challenge(alpha_h, alpha_dev);
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < half; i += gridDim.x * blockDim.x) {
    const uint32_t pair = (i >> 2) << 1;
    const uint32_t ix = __ldg(lt1 + pair), iy = __ldg(lt1 + pair + 1);
    uint32_t t;
    switch (i & 3) {
      case 0: t = iy; break;
      case 1: t = m31_neg(iy); break;
      case 2: t = m31_neg(ix); break;
      default: t = ix; break;
    }
    qm31 f1;
    qm31 f0 = load_pair(c, i, f1);
    qm31_ibfly(f0, f1, t);
    store(c, i, qm31_add(qm31_mul(alpha, f1), f0));
  }
}

struct Pack {
  const uint32_t* in[4];
  uint32_t* out[16];
};

__global__ void pack_leaves_kernel(const Pack p, uint32_t n_rows) {
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n_rows; r += gridDim.x * blockDim.x) {
#pragma unroll
    for (int coord = 0; coord < 4; coord++) {
      const uint4 q = __ldg(reinterpret_cast<const uint4*>(p.in[coord]) + r);
      p.out[coord + 0][r] = q.x;
      p.out[coord + 4][r] = q.y;
      p.out[coord + 8][r] = q.z;
      p.out[coord + 12][r] = q.w;
    }
  }
}

uint32_t grid_for(uint32_t n, uint32_t threads) { return std::max(1u, std::min<uint32_t>((n + threads - 1) / threads, 152 * 8)); }

}  // namespace
}  // namespace cs

using namespace cs;

static cs_status check_coords(const uint32_t* const src[4], uint32_t* const dst[4]) {
  CS_CHECK_ARG(src != nullptr && dst != nullptr, "fold: null coordinate table");
  for (int k = 0; k < 4; k++) {
    CS_CHECK_ARG(src[k] != nullptr && dst[k] != nullptr, "fold: coordinate %d is null", k);
    CS_CHECK_ARG((reinterpret_cast<uintptr_t>(src[k]) & 7) == 0, "fold: coordinate %d is not 8-byte aligned", k);
  }
  return CS_OK;
}

namespace cs {
namespace {

cs_status fold_line_impl(const uint32_t* const h_src[4], uint32_t log_size, qm31 alpha, const uint32_t* alpha_dev,
                         uint32_t* const h_dst[4], const uint32_t* d_itwiddles, uint32_t twiddle_log_size,
                         cs_stream stream) {
  cs_status s = check_coords(h_src, h_dst);
  if (s != CS_OK) return s;
  CS_CHECK_ARG(d_itwiddles != nullptr, "fold_line: null twiddles");
  CS_CHECK_ARG(log_size >= 1 && log_size <= twiddle_log_size,
               "fold_line: line domain of log %u is not covered by a tree of log %u", log_size, twiddle_log_size);
  Coords c;
  for (int k = 0; k < 4; k++) {
    c.in[k] = h_src[k];
    c.out[k] = h_dst[k];
  }
  const uint32_t half = 1u << (log_size - 1);
  const uint32_t* layer = d_itwiddles + ((1u << twiddle_log_size) - (1u << log_size));
  fold_line_kernel<<<grid_for(half, 256), 256, 0, to_stream(stream)>>>(c, half, layer, alpha, alpha_dev);
  CS_LAUNCHED("fold_line_kernel");
  return CS_OK;
}

cs_status fold_circle_impl(const uint32_t* const h_src[4], uint32_t log_size, qm31 alpha, const uint32_t* alpha_dev,
                           uint32_t* const h_dst[4], const uint32_t* d_itwiddles, uint32_t twiddle_log_size,
                           cs_stream stream) {
  cs_status s = check_coords(h_src, h_dst);
  if (s != CS_OK) return s;
  CS_CHECK_ARG(d_itwiddles != nullptr, "fold_circle_into_line: null twiddles");
  CS_CHECK_ARG(log_size >= 3 && log_size <= twiddle_log_size + 1,
               "fold_circle_into_line: circle domain of log %u is not covered by a tree of log %u (min log 3)",
               log_size, twiddle_log_size);
  Coords c;
  for (int k = 0; k < 4; k++) {
    c.in[k] = h_src[k];
    c.out[k] = h_dst[k];
  }
  const uint32_t half = 1u << (log_size - 1);
  const uint32_t* lt1 = d_itwiddles + ((1u << twiddle_log_size) - (1u << (log_size - 1)));
  fold_circle_kernel<<<grid_for(half, 256), 256, 0, to_stream(stream)>>>(c, half, lt1, alpha, alpha_dev);
  CS_LAUNCHED("fold_circle_kernel");
  return CS_OK;
}

}  // namespace
}  // namespace cs

extern "C" cs_status cs_fold_line(const uint32_t* const h_src[4], uint32_t log_size, const uint32_t alpha[4],
                                  uint32_t* const h_dst[4], const uint32_t* d_itwiddles, uint32_t twiddle_log_size,
                                  cs_stream stream) {
  CS_CHECK_ARG(alpha != nullptr, "fold_line: null alpha");
  return fold_line_impl(h_src, log_size, qm31_make(alpha[0], alpha[1], alpha[2], alpha[3]), nullptr, h_dst,
                        d_itwiddles, twiddle_log_size, stream);
}

extern "C" cs_status cs_fold_line_device_alpha(const uint32_t* const h_src[4], uint32_t log_size,
                                               const uint32_t* d_alpha, uint32_t* const h_dst[4],
                                               const uint32_t* d_itwiddles, uint32_t twiddle_log_size,
                                               cs_stream stream) {
  CS_CHECK_ARG(d_alpha != nullptr, "fold_line: null device alpha");
  return fold_line_impl(h_src, log_size, qm31_make(0, 0, 0, 0), d_alpha, h_dst, d_itwiddles, twiddle_log_size,
                        stream);
}

extern "C" cs_status cs_fold_circle_into_line(const uint32_t* const h_src[4], uint32_t log_size,
                                              const uint32_t alpha[4], uint32_t* const h_dst[4],
                                              const uint32_t* d_itwiddles, uint32_t twiddle_log_size,
                                              cs_stream stream) {
  CS_CHECK_ARG(alpha != nullptr, "fold_circle_into_line: null alpha");
  return fold_circle_impl(h_src, log_size, qm31_make(alpha[0], alpha[1], alpha[2], alpha[3]), nullptr, h_dst,
                          d_itwiddles, twiddle_log_size, stream);
}

extern "C" cs_status cs_fold_circle_into_line_device_alpha(const uint32_t* const h_src[4], uint32_t log_size,
                                                           const uint32_t* d_alpha, uint32_t* const h_dst[4],
                                                           const uint32_t* d_itwiddles, uint32_t twiddle_log_size,
                                                           cs_stream stream) {
  CS_CHECK_ARG(d_alpha != nullptr, "fold_circle_into_line: null device alpha");
  return fold_circle_impl(h_src, log_size, qm31_make(0, 0, 0, 0), d_alpha, h_dst, d_itwiddles, twiddle_log_size,
                          stream);
}

extern "C" cs_status cs_pack_leaves_input(const uint32_t* const h_in[4], uint32_t log_size, uint32_t* const h_out[16],
                                          cs_stream stream) {
  CS_CHECK_ARG(h_in != nullptr && h_out != nullptr, "pack_leaves_input: null table");
  CS_CHECK_ARG(log_size >= 2 && log_size <= 30, "pack_leaves_input: log size %u out of range", log_size);
  Pack p;
  for (int k = 0; k < 4; k++) {
    CS_CHECK_ARG(h_in[k] != nullptr && (reinterpret_cast<uintptr_t>(h_in[k]) & 15) == 0,
                 "pack_leaves_input: input %d null or not 16-byte aligned", k);
    p.in[k] = h_in[k];
  }
  for (int k = 0; k < 16; k++) {
    CS_CHECK_ARG(h_out[k] != nullptr, "pack_leaves_input: output %d null", k);
    p.out[k] = h_out[k];
  }
  const uint32_t rows = 1u << (log_size - 2);
  pack_leaves_kernel<<<grid_for(rows, 256), 256, 0, to_stream(stream)>>>(p, rows);
  CS_LAUNCHED("pack_leaves_kernel");
  return CS_OK;
}
