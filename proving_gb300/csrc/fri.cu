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
#include <atomic>

#include <vector>

#include "blake2s.cuh"
#include "channel.cuh"
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

// FriOps::fold_line with F <= LOG_V + 8 challenges per launch: every 2^F consecutive values of the
// layer fold into one, with no shared-memory round trip until the last folds. A thread loads
// V = 2^LOG_V consecutive values (LOG_V 3 or 4: two or four 16-byte words per coordinate, taken in
// chunks of 8) and folds them LOG_V times in registers (its pairs are its own); the 2^(F-LOG_V)
// threads of a group fold their results over shuffles (lane l pairs with lane l + 2^k, up to five
// folds), and for F > LOG_V + 5 a group is a whole block whose warps' results meet in shared
// memory for the rest (up to three). For smaller F a block of up to 256 threads holds several
// groups. Every twiddle a thread needs is loaded before the first fold, so the chain of folds waits
// on one round of loads. Fold j of the launch pairs values (2i, 2i + 1) of its layer with the
// layer's inverse twiddle i and the challenge's product table, as fold_line_tile_kernel does.
// Needs 16-byte aligned coordinates and twiddles, F >= LOG_V, and blockDim.x * gridDim.x =
// 2^(log_size - LOG_V) with blockDim.x a multiple of 2^(F-LOG_V), equal to it for F > LOG_V + 5.
// Sixteen values a thread issue a fifth fewer folds than eight for the same layer (the shuffle
// folds, where every lane computes although half the results are read, cover fewer values) and
// halve the threads, so the largest launches fit in one wave.
constexpr uint32_t kRegFoldMax = 12;
// log2 of the values a thread of fold_line_regs_kernel folds in registers, at most (cs_fold_set_plan)
std::atomic<uint32_t> g_fold_log_values{4};
constexpr uint32_t kRegFoldThreads = 256;
struct RegFoldSteps {
  qm31_const alpha[kRegFoldMax];
};

// One pair fold, f0 + f1 + ((f0 - f1) itw) alpha (qm31_ibfly, then the challenge product), with fewer
// reductions: the sum f0 + f1 (below 2P) enters each coordinate's 64-bit accumulator of the
// challenge product unreduced (4 (P-1)^2 + 2P < 2^64), and the twiddle product takes the doubled
// twiddle 2 itw (below 2^32): the high word of d * 2 itw is (d itw) >> 31 and its low word shifted
// right by one is (d itw) mod 2^31. Canonical inputs give the canonical result of the plain form.
__device__ __forceinline__ qm31 fold_pair(const qm31& f0, const qm31& f1, uint32_t itw, const qm31_const& alpha) {
  const uint32_t t2 = itw << 1;
  const uint32_t a0[4] = {f0.a.a, f0.a.b, f0.b.a, f0.b.b};
  const uint32_t a1[4] = {f1.a.a, f1.a.b, f1.b.a, f1.b.b};
  uint32_t d[4];
#pragma unroll
  for (int j = 0; j < 4; j++) {
    const uint64_t q = (uint64_t)m31_sub(a0[j], a1[j]) * t2;
    d[j] = m31_reduce_once(((uint32_t)q >> 1) + (uint32_t)(q >> 32));
  }
  uint32_t r[4];
#pragma unroll
  for (int i = 0; i < 4; i++) {
    uint64_t acc = (uint64_t)(a0[i] + a1[i]);
#pragma unroll
    for (int j = 0; j < 4; j++) acc += (uint64_t)d[j] * alpha.k[i][j];
    r[i] = m31_reduce64(acc);
  }
  return qm31_make(r[0], r[1], r[2], r[3]);
}

__device__ __forceinline__ qm31 shfl_down_qm31(const qm31& v, uint32_t delta, uint32_t mask) {
  return qm31_make(__shfl_down_sync(mask, v.a.a, delta), __shfl_down_sync(mask, v.a.b, delta),
                   __shfl_down_sync(mask, v.b.a, delta), __shfl_down_sync(mask, v.b.b, delta));
}

template <uint32_t LOG_V>
__global__ void __launch_bounds__(kRegFoldThreads, LOG_V == 3 ? 5 : 4) fold_line_regs_kernel(
    const Coords c, uint32_t log_size, uint32_t n_folds, const uint32_t* __restrict__ itw,
    uint32_t twiddle_log_size, const RegFoldSteps steps) {
  constexpr uint32_t V = 1u << LOG_V;
  constexpr uint32_t kChunks = V / 8;
  __shared__ uint32_t part[4][8];
  const uint32_t t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const size_t tw_len = (size_t)1 << twiddle_log_size;
  // twiddles of fold j of this launch: the inverse-twiddle layer of the line domain of log (log_size - j)
  const auto layer = [&](uint32_t j) { return itw + (tw_len - ((size_t)1 << (log_size - j))); };
  const size_t g = (size_t)blockIdx.x * blockDim.x + t;  // this thread's index in layer LOG_V
  const size_t base = V * g;                             // and its first value in layer 0
  const uint32_t warp_folds = min(5u, n_folds - LOG_V);
  const uint32_t smem_folds = n_folds > LOG_V + 5 ? n_folds - LOG_V - 5 : 0;
  // every twiddle up front: chunk h's register folds (layer 0: four, layer 1: two, layer 2: one,
  // at chunk index kChunks g + h), for V = 16 the fold of the two chunks (layer 3), the shuffle
  // folds (layers LOG_V..LOG_V+4) and, for warp 0 of a block of F > LOG_V + 5, the shared-memory
  // folds (lane l takes index blockIdx.x * 2^smem_folds + l of layer LOG_V + 5, lanes past the
  // block's warps repeat lane 0)
  uint4 t0[kChunks];
  uint2 t1[kChunks];
  uint32_t t2[kChunks];
#pragma unroll
  for (uint32_t h = 0; h < kChunks; h++) {
    const size_t gc = kChunks * g + h;
    t0[h] = __ldg(reinterpret_cast<const uint4*>(layer(0) + 4 * gc));
    t1[h] = __ldg(reinterpret_cast<const uint2*>(layer(1) + 2 * gc));
    t2[h] = __ldg(layer(2) + gc);
  }
  const uint32_t t3 = LOG_V == 4 ? __ldg(layer(3) + g) : 0;
  uint32_t tw_w[5], tw_s[3];
#pragma unroll
  for (uint32_t k = 0; k < 5; k++) tw_w[k] = k < warp_folds ? __ldg(layer(LOG_V + k) + (g >> (k + 1))) : 0;
  const uint32_t n_warps = blockDim.x >> 5;
  const size_t gs = smem_folds ? ((size_t)blockIdx.x << smem_folds) + (lane < n_warps ? lane : 0) : 0;
#pragma unroll
  for (uint32_t k = 0; k < 3; k++)
    tw_s[k] = (warp == 0 && k < smem_folds) ? __ldg(layer(LOG_V + 5 + k) + (gs >> (k + 1))) : 0;
  qm31 h_out[kChunks];
#pragma unroll
  for (uint32_t h = 0; h < kChunks; h++) {
    uint32_t w[4][8];
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const uint4 lo = __ldg(reinterpret_cast<const uint4*>(c.in[k] + base + 8 * h));
      const uint4 hi = __ldg(reinterpret_cast<const uint4*>(c.in[k] + base + 8 * h) + 1);
      w[k][0] = lo.x, w[k][1] = lo.y, w[k][2] = lo.z, w[k][3] = lo.w;
      w[k][4] = hi.x, w[k][5] = hi.y, w[k][6] = hi.z, w[k][7] = hi.w;
    }
    qm31 v[8];
#pragma unroll
    for (int i = 0; i < 8; i++) v[i] = qm31_make(w[0][i], w[1][i], w[2][i], w[3][i]);
    v[0] = fold_pair(v[0], v[1], t0[h].x, steps.alpha[0]);
    v[1] = fold_pair(v[2], v[3], t0[h].y, steps.alpha[0]);
    v[2] = fold_pair(v[4], v[5], t0[h].z, steps.alpha[0]);
    v[3] = fold_pair(v[6], v[7], t0[h].w, steps.alpha[0]);
    v[0] = fold_pair(v[0], v[1], t1[h].x, steps.alpha[1]);
    v[1] = fold_pair(v[2], v[3], t1[h].y, steps.alpha[1]);
    h_out[h] = fold_pair(v[0], v[1], t2[h], steps.alpha[2]);
  }
  qm31 x = h_out[0];
  if constexpr (LOG_V == 4) x = fold_pair(h_out[0], h_out[kChunks - 1], t3, steps.alpha[3]);
  // folds over a group's lanes: lane l keeps the fold of l and l + 2^k when its index in the group is
  // a multiple of 2^(k+1); the other lanes compute values nobody reads
  const uint32_t mask = blockDim.x >= 32 ? 0xffffffffu : ((1u << blockDim.x) - 1);
#pragma unroll
  for (uint32_t k = 0; k < 5; k++) {
    if (k < warp_folds) {  // the same for the whole block
      const qm31 y = shfl_down_qm31(x, 1u << k, mask);
      x = fold_pair(x, y, tw_w[k], steps.alpha[LOG_V + k]);
    }
  }
  if (smem_folds == 0) {  // groups of 2^(F-LOG_V) lanes; the first lane of each writes its value
    if ((t & ((1u << (n_folds - LOG_V)) - 1)) == 0) {
      const size_t o = g >> (n_folds - LOG_V);
      c.out[0][o] = x.a.a;
      c.out[1][o] = x.a.b;
      c.out[2][o] = x.b.a;
      c.out[3][o] = x.b.b;
    }
    return;
  }
  // one group per block: the warps' results (layer LOG_V + 5 indices blockIdx.x * 2^smem_folds + warp) meet
  if (lane == 0) part[0][warp] = x.a.a, part[1][warp] = x.a.b, part[2][warp] = x.b.a, part[3][warp] = x.b.b;
  __syncthreads();
  if (warp != 0) return;
  const uint32_t l = lane < n_warps ? lane : 0;
  x = qm31_make(part[0][l], part[1][l], part[2][l], part[3][l]);
#pragma unroll
  for (uint32_t k = 0; k < 3; k++) {
    if (k < smem_folds) {
      const qm31 y = shfl_down_qm31(x, 1u << k, 0xffffffffu);
      x = fold_pair(x, y, tw_s[k], steps.alpha[LOG_V + 5 + k]);
    }
  }
  if (lane == 0) {
    c.out[0][blockIdx.x] = x.a.a;
    c.out[1][blockIdx.x] = x.a.b;
    c.out[2][blockIdx.x] = x.b.a;
    c.out[3][blockIdx.x] = x.b.b;
  }
}

// The small layers of FriProver::commit (crates/stwo/src/prover/fri.rs:113-207) in one block, with
// the channel on the device: for each line layer of 2^m <= 2^kFriTailMaxLog values, commit it (the
// lifted Blake2s tree of its four coordinate columns, which all have the tree's height: leaf i is
// Blake2s of the 16 bytes of value i, crates/stwo/src/prover/backend/cpu/merkle_lifted.rs:46-90;
// node = Blake2s(left || right), crates/stwo/src/core/vcs_lifted/blake2_merkle.rs:29-36), mix the
// root into the channel, draw the folding challenge and fold the layer (fold_line,
// crates/stwo/src/prover/backend/cpu/fri.rs:66-91) into the next one. Every tree, challenge and
// folded layer is written where the per-layer path (cs_merkle_commit, cs_channel_mix_root,
// cs_channel_draw_secure_felt, cs_fold_line_device_alpha) writes it; the layer being committed
// and the tree level being built stay in shared memory, so the layers cost one launch instead of
// about six each. Thread t hashes leaves 2t and 2t + 1 and their parent.
constexpr uint32_t kFriTailMaxLog = 10;
constexpr uint32_t kFriTailThreads = 1u << (kFriTailMaxLog - 1);

struct FriTail {
  uint32_t* eval[kFriTailMaxLog + 1][4];  // layer j's coordinates; j = n_layers: the last fold's output
  uint32_t* tree[kFriTailMaxLog];         // layer j's tree, leaves first and root last (16-byte aligned)
};

__device__ __forceinline__ void store_digest(uint32_t* dst, const uint32_t h[8]) {
  uint4* o = reinterpret_cast<uint4*>(dst);
  o[0] = make_uint4(h[0], h[1], h[2], h[3]);
  o[1] = make_uint4(h[4], h[5], h[6], h[7]);
}

// Every hash of the tail is one final Blake2s block from the initial chaining value (a leaf's 16
// bytes, a node's 64, the channel's 64-byte mix and 37-byte draw), so each layer is a loop of steps
// around a single compression call: the kernel holds one copy of the compression (a one-shot kernel
// whose code is otherwise fetched cold for every inlined copy).
__global__ void __launch_bounds__(kFriTailThreads) fri_tail_kernel(const __grid_constant__ FriTail T,
                                                                   uint32_t log_size, uint32_t n_layers,
                                                                   uint32_t* state, uint32_t* alphas,
                                                                   const uint32_t* __restrict__ itw,
                                                                   uint32_t twiddle_log_size, uint32_t one) {
  __shared__ uint32_t v[4][1u << kFriTailMaxLog];  // the layer being committed and folded
  __shared__ uint32_t d[kFriTailThreads][8];       // the tree level being built
  __shared__ uint32_t chan[9];
  __shared__ uint32_t alpha[4];
  const uint32_t t = threadIdx.x;
  const size_t tw_len = (size_t)1 << twiddle_log_size;
  for (uint32_t i = t; i < (4u << log_size); i += blockDim.x)
    v[i >> log_size][i & ((1u << log_size) - 1)] = T.eval[0][i >> log_size][i & ((1u << log_size) - 1)];
  if (t < 9) chan[t] = state[t];
  __syncthreads();
  for (uint32_t j = 0; j < n_layers; j++) {
    const uint32_t m = log_size - j, half = 1u << (m - 1);
    uint32_t* tree = T.tree[j];
    // steps: leaf 2t, leaf 2t + 1, their parent (node t of level m - 1), levels m - 2 .. 0, the
    // root's mix into the channel, the challenge's draw
    const uint32_t n_steps = 3 + (m - 1) + 2;
    uint32_t leaves[16];  // this thread's two leaf digests, the message of its first node
#pragma unroll 1
    for (uint32_t step = 0; step < n_steps; step++) {
      uint32_t msg[16], tlo = 64;
      bool on;
      int level = -1;  // the node level of a node step
      if (step < 2) {
        on = t < half;
        if (on) {
#pragma unroll
          for (int k = 0; k < 4; k++) msg[k] = v[k][2 * t + step];
#pragma unroll
          for (int k = 4; k < 16; k++) msg[k] = 0;
        }
        tlo = 16;
      } else if (step == 2) {
        on = t < half;
        level = (int)m - 1;
#pragma unroll
        for (int k = 0; k < 16; k++) msg[k] = leaves[k];
      } else if (step < n_steps - 2) {
        level = (int)m - 2 - (int)(step - 3);
        on = t < (1u << level);
        if (on) {
#pragma unroll
          for (int w = 0; w < 8; w++) msg[w] = d[2 * t][w], msg[8 + w] = d[2 * t + 1][w];
        }
      } else if (step == n_steps - 2) {  // mix the root (d[0]) into the channel
        on = t == 0;
        tlo = kChannelMixBytes;
        if (on) channel_mix_message(chan, d[0], msg);
      } else {  // draw the folding challenge
        on = t == 0;
        tlo = kChannelDrawBytes;
        if (on) channel_draw_message(chan, msg);
      }
      uint32_t h[8];
      if (on) {
        b2s_init(h);
        b2s_compress(h, msg, tlo, 0, true, one);
      }
      if (step < 2) {
        if (on) {
          if (step == 0) {
#pragma unroll
            for (int w = 0; w < 8; w++) leaves[w] = h[w];
          } else {
#pragma unroll
            for (int w = 0; w < 8; w++) leaves[8 + w] = h[w];
          }
          store_digest(tree + (size_t)(2 * t + step) * 8, h);
        }
      } else if (level >= 0) {
        __syncthreads();  // every read of this level's children is done
        if (on) {
#pragma unroll
          for (int w = 0; w < 8; w++) d[t][w] = h[w];
          store_digest(tree + ((size_t)(2u << m) - (2u << level) + t) * 8, h);
        }
        __syncthreads();
      } else if (step == n_steps - 2) {
        if (on) channel_after_mix(chan, h);
      } else if (on) {
        uint32_t felt[4];
        channel_after_draw(chan, h, felt);
#pragma unroll
        for (int w = 0; w < 4; w++) alpha[w] = felt[w], alphas[4 * j + w] = felt[w];
      }
    }
    __syncthreads();
    qm31 r;
    if (t < half) {  // pair (2t, 2t + 1) folds into value t of the next layer
      qm31 f0 = qm31_make(v[0][2 * t], v[1][2 * t], v[2][2 * t], v[3][2 * t]);
      qm31 f1 = qm31_make(v[0][2 * t + 1], v[1][2 * t + 1], v[2][2 * t + 1], v[3][2 * t + 1]);
      qm31_ibfly(f0, f1, __ldg(itw + (tw_len - ((size_t)1 << m)) + t));
      r = qm31_add(f0, qm31_mul(qm31_make(alpha[0], alpha[1], alpha[2], alpha[3]), f1));
      T.eval[j + 1][0][t] = r.a.a;
      T.eval[j + 1][1][t] = r.a.b;
      T.eval[j + 1][2][t] = r.b.a;
      T.eval[j + 1][3][t] = r.b.b;
    }
    __syncthreads();
    if (t < half) v[0][t] = r.a.a, v[1][t] = r.a.b, v[2][t] = r.b.a, v[3][t] = r.b.b;
    __syncthreads();
  }
  if (t < 9) state[t] = chan[t];
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

extern "C" cs_status cs_fold_set_plan(uint32_t log_values_per_thread) {
  CS_CHECK_ARG(log_values_per_thread == 3 || log_values_per_thread == 4,
               "fold_set_plan: %u (log2 of the values a thread folds: 3 or 4)", log_values_per_thread);
  cs::g_fold_log_values.store(log_values_per_thread, std::memory_order_relaxed);
  return CS_OK;
}

extern "C" cs_status cs_fold_get_plan(uint32_t* log_values_per_thread) {
  CS_CHECK_ARG(log_values_per_thread != nullptr, "fold_get_plan: null pointer");
  *log_values_per_thread = cs::g_fold_log_values.load(std::memory_order_relaxed);
  return CS_OK;
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
  // The folds in launches: of up to kRegFoldMax folds by fold_line_regs_kernel (every source
  // coordinate and the twiddle tree 16-byte aligned, at least 3 folds of a layer of at least 2^3 values),
  // otherwise of up to kFoldTileLog folds by the tile kernels; the layers between two launches go to
  // scratch.
  // (the register kernel loads 16-byte words of its source and of the twiddles and stores single
  // words, so the destination may have any 4-byte alignment; scratch layers are 16-byte aligned)
  bool aligned = (reinterpret_cast<uintptr_t>(d_itwiddles) & 15) == 0;
  for (int k = 0; k < 4; k++) aligned = aligned && (reinterpret_cast<uintptr_t>(h_src[k]) & 15) == 0;
  struct Pass {
    uint32_t folds;
    bool regs;
    uint32_t log_v;  // values per thread of the register kernel, log 3 or 4
  };
  std::vector<Pass> passes;
  size_t scratch_words = 0;
  const uint32_t log_v_max = g_fold_log_values.load(std::memory_order_relaxed);
  for (uint32_t cur = log_size, done = 0; done < n_alphas;) {
    const uint32_t left = n_alphas - done;
    Pass ps;
    ps.regs = aligned && cur >= 3 && left >= 3;
    ps.log_v = (log_v_max == 4 && cur >= 4 && left >= 4) ? 4 : 3;
    ps.folds = ps.regs ? std::min(std::min(left, ps.log_v + 8), cur) : std::min(left, std::min(cur, kFoldTileLog));
    passes.push_back(ps);
    done += ps.folds;
    cur -= ps.folds;
    if (done < n_alphas) scratch_words = std::max(scratch_words, std::max<size_t>((size_t)1 << cur, 4));
  }
  uint32_t* scratch = nullptr;
  if (scratch_words)
    CS_CUDA(stream_alloc(reinterpret_cast<void**>(&scratch), sizeof(uint32_t) * 8 * scratch_words, st));
  Coords c;
  for (int k = 0; k < 4; k++) c.in[k] = h_src[k];
  uint32_t cur_log = log_size, done = 0, ping = 0;
  cudaError_t e = cudaSuccess;
  for (size_t pi = 0; pi < passes.size() && e == cudaSuccess; pi++) {
    const uint32_t folds = passes[pi].folds;
    const bool last = pi + 1 == passes.size();
    for (int k = 0; k < 4; k++)
      c.out[k] = last ? h_dst[k] : scratch + (size_t)ping * 4 * scratch_words + (size_t)k * scratch_words;
    if (passes[pi].regs) {
      RegFoldSteps steps;
      for (uint32_t j = 0; j < folds; j++) {
        const uint32_t* a = h_alphas + 4 * (size_t)(done + j);
        steps.alpha[j] = qm31_const_of(qm31_make(a[0] % P, a[1] % P, a[2] % P, a[3] % P));
      }
      // 2^(cur_log - LOG_V) threads in groups of 2^(folds - LOG_V): for more than LOG_V + 5 folds one
      // group per block, otherwise blocks of up to kRegFoldThreads
      const uint32_t lv = passes[pi].log_v;
      const uint32_t group = 1u << (folds - lv);
      const uint32_t threads =
          folds > lv + 5 ? group : std::max(group, std::min(kRegFoldThreads, 1u << (cur_log - lv)));
      const uint32_t blocks = (1u << (cur_log - lv)) / threads;
      if (lv == 4)
        fold_line_regs_kernel<4><<<blocks, threads, 0, st>>>(c, cur_log, folds, d_itwiddles, twiddle_log_size, steps);
      else
        fold_line_regs_kernel<3><<<blocks, threads, 0, st>>>(c, cur_log, folds, d_itwiddles, twiddle_log_size, steps);
    } else {
      FoldSteps steps;
      for (uint32_t j = 0; j < folds; j++) {
        const uint32_t* a = h_alphas + 4 * (size_t)(done + j);
        steps.alpha[j] = qm31_const_of(qm31_make(a[0] % P, a[1] % P, a[2] % P, a[3] % P));
      }
      const uint32_t tile_log = std::min(cur_log, kFoldTileLog);
      bool vec = tile_log >= 2;
      for (int k = 0; k < 4; k++) vec = vec && (reinterpret_cast<uintptr_t>(c.in[k]) & 15) == 0;
      const uint32_t grid = 1u << (cur_log - tile_log);
      if (vec)
        fold_line_stream_kernel<<<std::min(grid, stream_fold_blocks()), kStreamThreads, 0, st>>>(
            c, cur_log, tile_log, folds, d_itwiddles, twiddle_log_size, grid, steps);
      else
        fold_line_tile_kernel<false><<<grid, kFoldThreads, 0, st>>>(c, cur_log, tile_log, folds, d_itwiddles,
                                                                     twiddle_log_size, steps);
    }
    note_launch();
    e = cudaGetLastError();
    for (int k = 0; k < 4; k++) c.in[k] = c.out[k];
    cur_log -= folds;
    done += folds;
    ping ^= 1;
  }
  cudaError_t ef = cudaSuccess;
  if (scratch != nullptr) ef = cudaFreeAsync(scratch, st);
  if (e != cudaSuccess) return from_cuda(e, "launch fold_line kernel");
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

extern "C" cs_status cs_fri_commit_fold_tail(uint32_t* d_state, uint32_t* d_alphas, uint32_t* const* h_evals,
                                             uint32_t* const* h_trees, uint32_t log_size, uint32_t n_layers,
                                             const uint32_t* d_itwiddles, uint32_t twiddle_log_size,
                                             cs_stream stream) {
  CS_CHECK_ARG(d_state != nullptr && d_alphas != nullptr && h_evals != nullptr && h_trees != nullptr &&
                   d_itwiddles != nullptr,
               "fri_commit_fold_tail: null pointer");
  CS_CHECK_ARG(log_size >= 1 && log_size <= kFriTailMaxLog && log_size <= twiddle_log_size,
               "fri_commit_fold_tail: layer of log %u (1..%u, covered by a tree of log %u)", log_size,
               kFriTailMaxLog, twiddle_log_size);
  CS_CHECK_ARG(n_layers >= 1 && n_layers <= log_size, "fri_commit_fold_tail: %u layers from log %u", n_layers,
               log_size);
  FriTail T;
  for (uint32_t j = 0; j <= n_layers; j++)
    for (int k = 0; k < 4; k++) {
      T.eval[j][k] = h_evals[4 * j + k];
      CS_CHECK_ARG(T.eval[j][k] != nullptr, "fri_commit_fold_tail: layer %u coordinate %d is null", j, k);
    }
  for (uint32_t j = 0; j < n_layers; j++) {
    T.tree[j] = h_trees[j];
    CS_CHECK_ARG(T.tree[j] != nullptr && aligned16(T.tree[j]),
                 "fri_commit_fold_tail: tree %u null or not 16-byte aligned", j);
  }
  const uint32_t threads = std::max(32u, 1u << (log_size - 1));
  fri_tail_kernel<<<1, threads, 0, to_stream(stream)>>>(T, log_size, n_layers, d_state, d_alphas, d_itwiddles,
                                                        twiddle_log_size, 1u);
  CS_LAUNCHED("fri_tail_kernel");
  return CS_OK;
}
