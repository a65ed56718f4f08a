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

// Several folds of a line evaluation in one pass (FriOps::fold_line with k challenges,
// crates/stwo/src/prover/fri.rs:27-45; CpuBackend folds one at a time, cpu/fri.rs:15-28): fold j
// pairs values 2p, 2p+1 of the j-times folded evaluation, so 2^T consecutive values fold to
// 2^(T-k) without touching any other. A block stages such a tile of the four coordinates in
// shared memory, folds it there with one pair per thread, and writes the result: the input is
// read once and the intermediate layers never reach HBM.
constexpr uint32_t kFoldTileLog = 10;
constexpr uint32_t kFoldThreads = 1u << (kFoldTileLog - 1);

struct FoldSteps {
  qm31_const alpha[kFoldTileLog];  // each challenge as its product table
};

template <bool VEC>
__global__ void __launch_bounds__(kFoldThreads) fold_line_tile_kernel(const Coords c, uint32_t log_size,
                                                                       uint32_t tile_log, uint32_t n_folds,
                                                                       const uint32_t* __restrict__ itw,
                                                                       uint32_t twiddle_log_size, const FoldSteps steps) {
  __shared__ uint32_t s[4][1u << kFoldTileLog];
  __shared__ uint32_t tw[1u << kFoldTileLog];  // fold j's inverse x-coordinates at n_tile - (n_tile >> j)
  const uint32_t tile = blockIdx.x;
  const uint32_t n_tile = 1u << tile_log;
  // Every load of the tile -- its twiddles for all folds and its values -- is issued before the
  // first store to shared memory, so a block waits for HBM once, not once per loop trip.
  const uint32_t p = threadIdx.x;
  uint32_t tv[kFoldTileLog];
#pragma unroll
  for (uint32_t j = 0; j < kFoldTileLog; j++) {
    const uint32_t m = n_tile >> (j + 1);
    if (j < n_folds && p < m)
      tv[j] = __ldg(itw + ((1u << twiddle_log_size) - (1u << (log_size - j))) + (size_t)tile * m + p);
  }
  constexpr uint32_t kPer = 2;  // 16-byte words per thread: 4 coordinates x 2^(T-2) <= 2 x kFoldThreads
  uint4 v[kPer];
  uint32_t sv[8];
  if constexpr (VEC) {
    const uint32_t per_log = tile_log - 2;
#pragma unroll
    for (uint32_t r = 0; r < kPer; r++) {
      const uint32_t q = p + r * kFoldThreads;
      if (q < (4u << per_log))
        v[r] = __ldg(reinterpret_cast<const uint4*>(c.in[q >> per_log] + ((size_t)tile << tile_log)) +
                     (q & ((1u << per_log) - 1)));
    }
  } else {
#pragma unroll
    for (uint32_t r = 0; r < 8; r++) {
      const uint32_t q = p + r * kFoldThreads;
      if (q < (4u << tile_log)) sv[r] = __ldg(c.in[q >> tile_log] + ((size_t)tile << tile_log) + (q & (n_tile - 1)));
    }
  }
#pragma unroll
  for (uint32_t j = 0, off = 0; j < kFoldTileLog; j++) {
    const uint32_t m = n_tile >> (j + 1);
    if (j < n_folds && p < m) tw[off + p] = tv[j];
    off += m;
  }
  if constexpr (VEC) {
    const uint32_t per_log = tile_log - 2;
#pragma unroll
    for (uint32_t r = 0; r < kPer; r++) {
      const uint32_t q = p + r * kFoldThreads;
      if (q < (4u << per_log)) {
        uint32_t* d = &s[q >> per_log][4 * (q & ((1u << per_log) - 1))];
        d[0] = v[r].x, d[1] = v[r].y, d[2] = v[r].z, d[3] = v[r].w;
      }
    }
  } else {
#pragma unroll
    for (uint32_t r = 0; r < 8; r++) {
      const uint32_t q = p + r * kFoldThreads;
      if (q < (4u << tile_log)) s[q >> tile_log][q & (n_tile - 1)] = sv[r];
    }
  }
  __syncthreads();
  uint32_t off = 0;
#pragma unroll
  for (uint32_t j = 0; j < kFoldTileLog; j++) {
    if (j == n_folds) break;  // the same for the whole block
    const uint32_t m = n_tile >> (j + 1);  // pairs of this tile at fold j
    qm31 r;
    if (p < m) {
      qm31 f0 = qm31_make(s[0][2 * p], s[1][2 * p], s[2][2 * p], s[3][2 * p]);
      qm31 f1 = qm31_make(s[0][2 * p + 1], s[1][2 * p + 1], s[2][2 * p + 1], s[3][2 * p + 1]);
      qm31_ibfly(f0, f1, tw[off + p]);
      r = qm31_add(f0, qm31_mul_const(f1, steps.alpha[j]));
    }
    __syncthreads();
    if (p < m) {
      s[0][p] = r.a.a;
      s[1][p] = r.a.b;
      s[2][p] = r.b.a;
      s[3][p] = r.b.b;
    }
    off += m;
    __syncthreads();
  }
  const uint32_t n_out = n_tile >> n_folds;
  for (uint32_t q = threadIdx.x; q < 4 * n_out; q += blockDim.x) {
    const uint32_t k = q / n_out, i = q % n_out;
    c.out[k][(size_t)tile * n_out + i] = s[k][i];
  }
}

// Asynchronous global -> shared copies (cp.async, completed by commit / wait groups).
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const uint32_t s = static_cast<uint32_t>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
  const uint32_t s = static_cast<uint32_t>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// fold_line_tile_kernel as a persistent loop over tiles with two shared-memory buffers: while a
// block folds tile i, the asynchronous copies of tile i + gridDim.x -- its values and the
// twiddles of all its folds -- are in flight, so HBM stays busy through the folds. 256 threads,
// two pairs each at the first fold. Needs 16-byte aligned coordinates and tile_log >= 2.
constexpr uint32_t kStreamThreads = 256;

__global__ void __launch_bounds__(kStreamThreads, 4) fold_line_stream_kernel(const Coords c, uint32_t log_size,
                                                                          uint32_t tile_log, uint32_t n_folds,
                                                                          const uint32_t* __restrict__ itw,
                                                                          uint32_t twiddle_log_size, uint32_t n_tiles,
                                                                          const FoldSteps steps) {
  __shared__ __align__(16) uint32_t s[2][4][1u << kFoldTileLog];
  __shared__ uint32_t tw[2][1u << kFoldTileLog];
  const uint32_t p = threadIdx.x;
  const uint32_t n_tile = 1u << tile_log;
  const uint32_t per_log = tile_log - 2;  // 16-byte words per coordinate
  const uint32_t per_mask = (1u << per_log) - 1;
  auto issue = [&](uint32_t tile, uint32_t b) {
#pragma unroll
    for (uint32_t r = 0; r < 4; r++) {  // 4 coordinates x 2^(T-2) <= 4 x 256 words of 16 bytes
      const uint32_t q = p + r * kStreamThreads;
      if (q < (4u << per_log))
        cp_async16(&s[b][q >> per_log][4 * (q & per_mask)],
                   c.in[q >> per_log] + ((size_t)tile << tile_log) + 4 * (q & per_mask));
    }
    uint32_t off = 0;
#pragma unroll
    for (uint32_t j = 0; j < kFoldTileLog; j++) {
      if (j < n_folds) {
        const uint32_t m = n_tile >> (j + 1);
        const uint32_t* layer = itw + ((1u << twiddle_log_size) - (1u << (log_size - j))) + (size_t)tile * m;
#pragma unroll
        for (uint32_t r = 0; r < 2; r++)
          if (p + r * kStreamThreads < m) cp_async4(&tw[b][off + p + r * kStreamThreads], layer + p + r * kStreamThreads);
        off += m;
      }
    }
    cp_async_commit();
  };
  uint32_t tile = blockIdx.x;
  if (tile >= n_tiles) return;  // the same for the whole block
  issue(tile, 0);
  for (uint32_t i = 0; tile < n_tiles; i++, tile += gridDim.x) {
    const uint32_t b = i & 1;
    if (tile + gridDim.x < n_tiles) {
      issue(tile + gridDim.x, b ^ 1);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    uint32_t off = 0;
#pragma unroll
    for (uint32_t j = 0; j < kFoldTileLog; j++) {
      if (j == n_folds) break;  // the same for the whole block
      const uint32_t m = n_tile >> (j + 1);
      qm31 r[2];
#pragma unroll
      for (uint32_t h = 0; h < 2; h++) {
        const uint32_t q = p + h * kStreamThreads;
        if (q < m) {
          qm31 f0 = qm31_make(s[b][0][2 * q], s[b][1][2 * q], s[b][2][2 * q], s[b][3][2 * q]);
          qm31 f1 = qm31_make(s[b][0][2 * q + 1], s[b][1][2 * q + 1], s[b][2][2 * q + 1], s[b][3][2 * q + 1]);
          qm31_ibfly(f0, f1, tw[b][off + q]);
          r[h] = qm31_add(f0, qm31_mul_const(f1, steps.alpha[j]));
        }
      }
      __syncthreads();
#pragma unroll
      for (uint32_t h = 0; h < 2; h++) {
        const uint32_t q = p + h * kStreamThreads;
        if (q < m) {
          s[b][0][q] = r[h].a.a;
          s[b][1][q] = r[h].a.b;
          s[b][2][q] = r[h].b.a;
          s[b][3][q] = r[h].b.b;
        }
      }
      off += m;
      __syncthreads();
    }
    const uint32_t out_log = tile_log - n_folds;
    for (uint32_t q = p; q < (4u << out_log); q += kStreamThreads) {
      const uint32_t k = q >> out_log, e = q & ((1u << out_log) - 1);
      c.out[k][((size_t)tile << out_log) + e] = s[b][k][e];
    }
    __syncthreads();  // buffer b is refilled by the next iteration's copies
  }
}

// fold_circle_kernel with four pairs per thread: values 8t .. 8t+7 of each coordinate as two
// 16-byte loads, one (1/x, 1/y) twiddle pair for the four, and one 16-byte store per coordinate.
// Needs 16-byte aligned coordinates and a multiple of 4 pairs.
__global__ void __launch_bounds__(256) fold_circle_wide_kernel(const Coords c, uint32_t quads,
                                                               const uint32_t* __restrict__ lt1,
                                                               const qm31_const alpha) {
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < quads; t += gridDim.x * blockDim.x) {
    const uint2 xy = __ldg(reinterpret_cast<const uint2*>(lt1) + t);  // (1/x, 1/y) of pair 2t
    const uint32_t tws[4] = {xy.y, m31_neg(xy.y), m31_neg(xy.x), xy.x};
    uint4 lo[4], hi[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
      lo[k] = __ldg(reinterpret_cast<const uint4*>(c.in[k]) + 2 * t);
      hi[k] = __ldg(reinterpret_cast<const uint4*>(c.in[k]) + 2 * t + 1);
    }
    uint32_t o[4][4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
      qm31 f0, f1;
      if (q == 0) f0 = qm31_make(lo[0].x, lo[1].x, lo[2].x, lo[3].x), f1 = qm31_make(lo[0].y, lo[1].y, lo[2].y, lo[3].y);
      if (q == 1) f0 = qm31_make(lo[0].z, lo[1].z, lo[2].z, lo[3].z), f1 = qm31_make(lo[0].w, lo[1].w, lo[2].w, lo[3].w);
      if (q == 2) f0 = qm31_make(hi[0].x, hi[1].x, hi[2].x, hi[3].x), f1 = qm31_make(hi[0].y, hi[1].y, hi[2].y, hi[3].y);
      if (q == 3) f0 = qm31_make(hi[0].z, hi[1].z, hi[2].z, hi[3].z), f1 = qm31_make(hi[0].w, hi[1].w, hi[2].w, hi[3].w);
      qm31_ibfly(f0, f1, tws[q]);
      const qm31 r = qm31_add(qm31_mul_const(f1, alpha), f0);
      o[0][q] = r.a.a, o[1][q] = r.a.b, o[2][q] = r.b.a, o[3][q] = r.b.b;
    }
#pragma unroll
    for (int k = 0; k < 4; k++)
      reinterpret_cast<uint4*>(c.out[k])[t] = make_uint4(o[k][0], o[k][1], o[k][2], o[k][3]);
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

// Resident blocks of fold_line_stream_kernel on the whole device (SMs x blocks per SM), once.
uint32_t stream_fold_blocks() {
  static uint32_t blocks = [] {
    int dev = 0, sms = 152, per_sm = 0;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fold_line_stream_kernel, kStreamThreads, 0) !=
            cudaSuccess ||
        per_sm < 1)
      per_sm = 1;
    return (uint32_t)(sms * per_sm);
  }();
  return blocks;
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
  bool wide = alpha_dev == nullptr;
  for (int k = 0; k < 4; k++)
    wide = wide && (reinterpret_cast<uintptr_t>(c.in[k]) & 15) == 0 && (reinterpret_cast<uintptr_t>(c.out[k]) & 15) == 0;
  if (wide) {
    fold_circle_wide_kernel<<<grid_for(half / 4, 256), 256, 0, to_stream(stream)>>>(c, half / 4, lt1,
                                                                                qm31_const_of(alpha));
    CS_LAUNCHED("fold_circle_wide_kernel");
    return CS_OK;
  }
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

extern "C" cs_status cs_fold_line_steps(const uint32_t* const h_src[4], uint32_t log_size, uint32_t n_alphas,
                                        const uint32_t* h_alphas, uint32_t* const h_dst[4],
                                        const uint32_t* d_itwiddles, uint32_t twiddle_log_size, cs_stream stream) {
  cs_status s = check_coords(h_src, h_dst);
  if (s != CS_OK) return s;
  CS_CHECK_ARG(h_alphas != nullptr && d_itwiddles != nullptr, "fold_line_steps: null pointer");
  CS_CHECK_ARG(n_alphas >= 1 && n_alphas <= log_size, "fold_line_steps: %u folds of a line domain of log %u",
               n_alphas, log_size);
  CS_CHECK_ARG(log_size <= twiddle_log_size && log_size <= 30,
               "fold_line_steps: line domain of log %u is not covered by a tree of log %u", log_size,
               twiddle_log_size);
  cudaStream_t st = to_stream(stream);
  // Launches of at most kFoldTileLog folds; the layers between two launches go to scratch.
  uint32_t* scratch = nullptr;
  const uint32_t first_tile = std::min(log_size, kFoldTileLog);
  const uint32_t first_folds = std::min(n_alphas, first_tile);
  if (first_folds < n_alphas) {
    const size_t words = (size_t)1 << (log_size - first_folds);
    CS_CUDA(stream_alloc(reinterpret_cast<void**>(&scratch), sizeof(uint32_t) * 8 * std::max<size_t>(words, 4), st));
  }
  Coords c;
  for (int k = 0; k < 4; k++) c.in[k] = h_src[k];
  uint32_t cur_log = log_size, done = 0, ping = 0;
  cudaError_t e = cudaSuccess;
  while (done < n_alphas && e == cudaSuccess) {
    const uint32_t tile_log = std::min(cur_log, kFoldTileLog);
    const uint32_t folds = std::min(n_alphas - done, tile_log);
    const bool last = done + folds == n_alphas;
    const size_t out_words = std::max<size_t>((size_t)1 << (log_size - first_folds), 4);
    for (int k = 0; k < 4; k++)
      c.out[k] = last ? h_dst[k] : scratch + (size_t)ping * 4 * out_words + (size_t)k * out_words;
    FoldSteps steps;
    for (uint32_t j = 0; j < folds; j++) {
      const uint32_t* a = h_alphas + 4 * (size_t)(done + j);
      steps.alpha[j] = qm31_const_of(qm31_make(a[0] % P, a[1] % P, a[2] % P, a[3] % P));
    }
    bool vec = tile_log >= 2;
    for (int k = 0; k < 4; k++) vec = vec && (reinterpret_cast<uintptr_t>(c.in[k]) & 15) == 0;
    const uint32_t grid = 1u << (cur_log - tile_log);
    if (vec)
      fold_line_stream_kernel<<<std::min(grid, stream_fold_blocks()), kStreamThreads, 0, st>>>(
          c, cur_log, tile_log, folds, d_itwiddles, twiddle_log_size, grid, steps);
    else
      fold_line_tile_kernel<false><<<grid, kFoldThreads, 0, st>>>(c, cur_log, tile_log, folds, d_itwiddles,
                                                                   twiddle_log_size, steps);
    note_launch();
    e = cudaGetLastError();
    for (int k = 0; k < 4; k++) c.in[k] = c.out[k];
    cur_log -= folds;
    done += folds;
    ping ^= 1;
  }
  cudaError_t ef = cudaSuccess;
  if (scratch != nullptr) ef = cudaFreeAsync(scratch, st);
  if (e != cudaSuccess) return from_cuda(e, "launch fold_line_tile_kernel");
  if (ef != cudaSuccess) return from_cuda(ef, "cudaFreeAsync");
  return CS_OK;
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
