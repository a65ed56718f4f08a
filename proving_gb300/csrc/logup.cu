// LogUp interaction columns on the device: the last column of
// LogupTraceGenerator (crates/constraint-framework/src/prover/logup.rs:50-130)
// for fractions 1 / (z - v_i): claimed_sum = sum_i 1 / (z - v_i), each
// fraction shifted by claimed_sum / n, then the inclusive prefix sum in coset
// order (inclusive_prefix_sum, crates/stwo/src/prover/backend/simd/prefix_sum.rs:20-149),
// values stored in bit-reversed circle-domain order. Coset index k lives at
// circle-domain index k / 2 (k even) or n/2 + (n - 1 - k) / 2 (k odd)
// (crates/stwo/src/core/utils.rs:177-188), stored at its bit reversal.
//
// Several columns of any sizes go through three launches per batch, with no
// host round trip between them and with every HBM access coalesced. With
// c the natural circle-domain index of storage position p (c = bitrev(p)),
// P the inclusive prefix sum of the fractions g in natural order and
// T = P(n - 1), the unshifted coset-order running sum at p is
//   c < n/2 (p even, k = 2c):             P(c) + T - P(n - 1 - c)
//   c >= n/2 (p odd, k = 2n - 1 - 2c):    P(n - 1 - c) + T - P(c) + g(c)
// (the even coset indices walk the first half forward, the odd ones the
// second half backward), and the mirror n - 1 - c sits at storage n - 1 - p.
// The shift is applied last: sum_{j<=k} (f_j - s) = F_k - (k + 1) s.
// Natural order is reached through 32 x 32 tiles: with c = (h, m, lo) (5, l - 10
// and 5 bits), tile m holds 32 natural runs of 32 (one per h) and 32 storage
// runs of 32 (one per lo).
//   1. runs: per tile, the fractions (stored in place in the output) and the
//      32 natural run totals;
//   2. run offsets: one block per column scans its run totals into exclusive
//      offsets (within 32 segments, plus the segment offsets); their sum is
//      the claimed sum, kept in device memory;
//   3. outputs: per pair of mirror tiles (m, ~m), the natural prefixes of both
//      and then every output of both.
// Columns of at most 2^9 rows are done by one block in the first launch.
#include <algorithm>
#include <vector>

#include "common.cuh"
#include "field.cuh"
#include "logup.cuh"
#include "rows.cuh"

namespace cs {

namespace {

constexpr uint32_t kSumBatch = 48;  // columns per launch (their pointers travel as kernel parameters)
constexpr uint32_t kSmallLog = 9;   // columns up to 2^9 rows: one block each
constexpr uint32_t kThreads = 1024;

struct SumBatch {
  const uint32_t* values[kSumBatch];  // the looked-up values (fractions 1 / (z - v)), or null:
                                      // the fractions are already in `out`
  uint32_t* out[kSumBatch][4];
  uint32_t log_size[kSumBatch];
  uint32_t tile0[kSumBatch + 1];  // first launch-1 block of each column (one per tile; one if small)
  uint32_t pair0[kSumBatch + 1];  // first launch-3 block of each column (none if small)
  uint32_t run0[kSumBatch];       // first run total of each column in `runs` (4 words each)
  uint32_t hoff0[kSumBatch];      // the column's 32 segment offsets in `runs`
  uint32_t n_cols;
  uint32_t* runs;     // 4 words per natural run of 32
  uint32_t* claimed;  // 4 words per column
  qm31 z;
};

__device__ __forceinline__ uint32_t rev5(uint32_t x) { return __brev(x) >> 27; }
__device__ __forceinline__ uint32_t rev_bits(uint32_t x, uint32_t bits) { return bits ? __brev(x) >> (32 - bits) : 0; }

// The column owning a block of a launch whose per-column first blocks are `first` (linear search
// over at most kSumBatch entries of the parameter table).
__device__ __forceinline__ uint32_t block_column(const uint32_t* first, uint32_t n_cols, uint32_t blk) {
  uint32_t c = 0;
  while (c + 1 < n_cols && first[c + 1] <= blk) c++;
  return c;
}

__device__ __forceinline__ qm31 load_fraction(const SumBatch& b, uint32_t col, uint32_t p) {
  if (b.values[col] != nullptr) return qm31_inv(qm31_sub(b.z, qm31_make(b.values[col][p], 0, 0, 0)));
  return qm31_make(b.out[col][0][p], b.out[col][1][p], b.out[col][2][p], b.out[col][3][p]);
}

__device__ __forceinline__ void store4(const SumBatch& b, uint32_t col, uint32_t p, const qm31& v) {
  b.out[col][0][p] = v.a.a;
  b.out[col][1][p] = v.a.b;
  b.out[col][2][p] = v.b.a;
  b.out[col][3][p] = v.b.b;
}

// The shifted running sum at storage position p of natural index c, from the natural prefixes at c
// (qp) and at its mirror (qm), the fraction g at c and the total t.
__device__ __forceinline__ qm31 running_value(uint32_t c, uint32_t log_n, const qm31& qp, const qm31& qm,
                                              const qm31& g, const qm31& t) {
  const uint32_t n = 1u << log_n;
  const bool first_half = c < (n >> 1);
  qm31 v = first_half ? qm31_sub(qm31_add(qp, t), qm) : qm31_add(qm31_sub(qm31_add(qm, t), qp), g);
  const uint32_t k = first_half ? 2 * c : 2 * n - 1 - 2 * c;
  // shift = t / n, 1 / n = 2^(31 - log_n) in M31
  const qm31 shift = qm31_mul_m31(t, 1u << (31 - log_n));
  return qm31_sub(v, qm31_mul_m31(shift, k + 1));
}

// Inclusive scan of four M31 values per thread across the block.
__device__ __forceinline__ void block_scan4(uint32_t x[4], uint32_t (*sh)[32]) {
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
#pragma unroll
    for (int c = 0; c < 4; c++) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x[c], o);
      if (lane >= (uint32_t)o) x[c] = m31_add(x[c], y);
    }
  }
  if (lane == 31) {
#pragma unroll
    for (int c = 0; c < 4; c++) sh[c][warp] = x[c];
  }
  __syncthreads();
  if (warp < 4) {
    uint32_t t = lane < (blockDim.x >> 5) ? sh[warp][lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= (uint32_t)o) t = m31_add(t, y);
    }
    sh[warp][lane] = t;
  }
  __syncthreads();
  if (warp > 0) {
#pragma unroll
    for (int c = 0; c < 4; c++) x[c] = m31_add(x[c], sh[c][warp - 1]);
  }
  __syncthreads();
}

// Inclusive scan of four M31 values over the lanes of a warp.
__device__ __forceinline__ void warp_scan4(uint32_t x[4]) {
  const uint32_t lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
#pragma unroll
    for (int c = 0; c < 4; c++) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x[c], o);
      if (lane >= (uint32_t)o) x[c] = m31_add(x[c], y);
    }
  }
}

// A column of at most 2^9 rows, all in one block (at least 2^9 threads).
__device__ void small_column(const SumBatch& b, uint32_t col, uint32_t* flat, uint32_t (*sh)[32]) {
  const uint32_t log_n = b.log_size[col], n = 1u << log_n, t = threadIdx.x;
  qm31 g = qm31_make(0, 0, 0, 0);
  uint32_t c = 0;
  if (t < n) {
    g = load_fraction(b, col, t);
    c = rev_bits(t, log_n);
    flat[c] = g.a.a;
    flat[512 + c] = g.a.b;
    flat[1024 + c] = g.b.a;
    flat[1536 + c] = g.b.b;
  }
  __syncthreads();
  uint32_t x[4];
#pragma unroll
  for (int k = 0; k < 4; k++) x[k] = t < n ? flat[512 * k + t] : 0;
  block_scan4(x, sh);
  if (t < n) {
#pragma unroll
    for (int k = 0; k < 4; k++) flat[512 * k + t] = x[k];
  }
  __syncthreads();
  const qm31 total = qm31_make(flat[n - 1], flat[512 + n - 1], flat[1024 + n - 1], flat[1536 + n - 1]);
  if (t < n) {
    const uint32_t mc = n - 1 - c;
    const qm31 qp = qm31_make(flat[c], flat[512 + c], flat[1024 + c], flat[1536 + c]);
    const qm31 qm = qm31_make(flat[mc], flat[512 + mc], flat[1024 + mc], flat[1536 + mc]);
    store4(b, col, t, running_value(c, log_n, qp, qm, g, total));
  }
  if (t < 4) b.claimed[4 * col + t] = t == 0 ? total.a.a : t == 1 ? total.a.b : t == 2 ? total.b.a : total.b.b;
}

// 1 / (z - v0) and 1 / (z - v1) with one M31 inversion (Montgomery's trick on the norms): for
// x = a + b u, 1 / x = (a - b u) / (a^2 - (2 + i) b^2), and 1 / d = conj(d) / |d|^2 for d in CM31.
__device__ __forceinline__ void fraction_pair(const qm31& z, uint32_t v0, uint32_t v1, qm31& f0, qm31& f1) {
  const qm31 x0 = qm31_sub(z, qm31_make(v0, 0, 0, 0)), x1 = qm31_sub(z, qm31_make(v1, 0, 0, 0));
  const auto denom = [](const qm31& x) {
    const cm31 b2 = cm31_mul(x.b, x.b);
    const cm31 ib2 = {m31_neg(b2.b), b2.a};
    return cm31_sub(cm31_mul(x.a, x.a), cm31_add(cm31_add(b2, b2), ib2));
  };
  const cm31 d0 = denom(x0), d1 = denom(x1);
  const uint32_t n0 = m31_add(m31_sqr(d0.a), m31_sqr(d0.b)), n1 = m31_add(m31_sqr(d1.a), m31_sqr(d1.b));
  const uint32_t prod = m31_mul(n0, n1);
  uint32_t i0, i1;
  if (prod != 0) {
    const uint32_t inv = m31_inv(prod);
    i0 = m31_mul(inv, n1);
    i1 = m31_mul(inv, n0);
  } else {  // z = v for one of them: each inverted alone (the inverse of 0 taken as 0, as in qm31_inv)
    i0 = m31_inv(n0);
    i1 = m31_inv(n1);
  }
  const cm31 di0 = {m31_mul(d0.a, i0), m31_mul(m31_neg(d0.b), i0)};
  const cm31 di1 = {m31_mul(d1.a, i1), m31_mul(m31_neg(d1.b), i1)};
  f0 = {cm31_mul(x0.a, di0), cm31_mul(cm31_neg(x0.b), di0)};
  f1 = {cm31_mul(x1.a, di1), cm31_mul(cm31_neg(x1.b), di1)};
}

// Launch 1 (512 threads): per tile m of a column of 2^10 or more rows, thread (w, t) (w < 16) takes
// the storage positions (rev5(lo) << (l - 5)) | (rev(m) << 5) | t for lo = w and w + 16, i.e.
// natural (h = rev5(t), m, lo); their two fractions share one M31 inversion.
__global__ void __launch_bounds__(kThreads / 2) runs_kernel(const SumBatch b) {
  __shared__ uint32_t tile[4][32][33];
  __shared__ uint32_t sh[4][32];
  const uint32_t col = block_column(b.tile0, b.n_cols, blockIdx.x);
  const uint32_t log_n = b.log_size[col];
  if (log_n <= kSmallLog) {
    small_column(b, col, &tile[0][0][0], sh);
    return;
  }
  const uint32_t mb = log_n - 10, m = blockIdx.x - b.tile0[col];
  const uint32_t w = threadIdx.x >> 5, t = threadIdx.x & 31, h = rev5(t);
  const uint32_t mid = (rev_bits(m, mb) << 5) | t;
  const uint32_t p0 = (rev5(w) << (log_n - 5)) | mid, p1 = (rev5(w + 16) << (log_n - 5)) | mid;
  qm31 g[2];
  if (b.values[col] != nullptr) {
    fraction_pair(b.z, b.values[col][p0], b.values[col][p1], g[0], g[1]);
    store4(b, col, p0, g[0]);
    store4(b, col, p1, g[1]);
  } else {
    g[0] = load_fraction(b, col, p0);
    g[1] = load_fraction(b, col, p1);
  }
#pragma unroll
  for (int q = 0; q < 2; q++) {
    const uint32_t lo = w + 16 * q;
    tile[0][lo][h] = g[q].a.a;
    tile[1][lo][h] = g[q].a.b;
    tile[2][lo][h] = g[q].b.a;
    tile[3][lo][h] = g[q].b.b;
  }
  __syncthreads();
  // warp w sums natural runs (h' = w and w + 16, m): lanes are lo
#pragma unroll
  for (int q = 0; q < 2; q++) {
    const uint32_t hh = w + 16 * q;
    uint32_t x[4];
#pragma unroll
    for (int k = 0; k < 4; k++) x[k] = tile[k][t][hh];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
      for (int k = 0; k < 4; k++) x[k] = m31_add(x[k], __shfl_xor_sync(0xffffffffu, x[k], o));
    }
    if (t < 4) b.runs[4 * (b.run0[col] + ((hh << mb) | m)) + t] = x[t];
  }
}

// Launch 2: one block per column of 2^10 or more rows. The natural runs (h, m) are ordered h-major,
// so warp h owns the contiguous runs [h 2^mb, (h + 1) 2^mb): it turns them into exclusive offsets
// within its segment (coalesced, 32 runs per step), and the block turns the 32 segment totals into
// the segment offsets `hoff` (added by launch 3); the grand total is the claimed sum.
__global__ void __launch_bounds__(kThreads) run_offsets_kernel(const SumBatch b) {
  __shared__ uint32_t seg_total[4][32];
  const uint32_t col = blockIdx.x;
  const uint32_t log_n = b.log_size[col];
  if (log_n <= kSmallLog) return;
  const uint32_t seg = 1u << (log_n - 10);
  const uint32_t h = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint4* r = reinterpret_cast<uint4*>(b.runs) + b.run0[col] + (size_t)h * seg;
  uint32_t carry[4] = {0, 0, 0, 0};
  for (uint32_t base = 0; base < seg; base += 32) {
    const bool live = base + lane < seg;
    const uint4 v = live ? r[base + lane] : make_uint4(0, 0, 0, 0);
    uint32_t x[4] = {v.x, v.y, v.z, v.w};
    warp_scan4(x);
    if (live)
      r[base + lane] = make_uint4(m31_add(m31_sub(x[0], v.x), carry[0]), m31_add(m31_sub(x[1], v.y), carry[1]),
                                  m31_add(m31_sub(x[2], v.z), carry[2]), m31_add(m31_sub(x[3], v.w), carry[3]));
#pragma unroll
    for (int k = 0; k < 4; k++) carry[k] = m31_add(carry[k], __shfl_sync(0xffffffffu, x[k], 31));
  }
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < 4; k++) seg_total[k][h] = carry[k];
  }
  __syncthreads();
  if (h == 0) {
    uint32_t x[4];
#pragma unroll
    for (int k = 0; k < 4; k++) x[k] = seg_total[k][lane];
    uint32_t own[4] = {x[0], x[1], x[2], x[3]};
    warp_scan4(x);
    uint4* hoff = reinterpret_cast<uint4*>(b.runs) + b.hoff0[col];
    hoff[lane] = make_uint4(m31_sub(x[0], own[0]), m31_sub(x[1], own[1]), m31_sub(x[2], own[2]),
                            m31_sub(x[3], own[3]));
    if (lane == 31) {
#pragma unroll
      for (int k = 0; k < 4; k++) b.claimed[4 * col + k] = x[k];
    }
  }
}

// Launch 3: per mirror pair of tiles (m, m' = ~m) of a column of 2^10 or more rows.
__global__ void __launch_bounds__(kThreads) outputs_kernel(const SumBatch b) {
  __shared__ uint32_t tiles[2][4][32][33];
  const uint32_t col = block_column(b.pair0, b.n_cols, blockIdx.x);
  const uint32_t log_n = b.log_size[col];
  const uint32_t mb = log_n - 10;
  const uint32_t m = blockIdx.x - b.pair0[col], mm = ((1u << mb) - 1) - m;
  const uint32_t n_tiles = m == mm ? 1 : 2;
  const uint32_t w = threadIdx.x >> 5, t = threadIdx.x & 31, h = rev5(t);
  const uint32_t ms[2] = {m, mm};
  qm31 g[2];
  uint32_t pos[2];
  for (uint32_t q = 0; q < n_tiles; q++) {
    pos[q] = (rev5(w) << (log_n - 5)) | (rev_bits(ms[q], mb) << 5) | t;
    const uint32_t p = pos[q];
    g[q] = qm31_make(b.out[col][0][p], b.out[col][1][p], b.out[col][2][p], b.out[col][3][p]);
    tiles[q][0][w][h] = g[q].a.a;
    tiles[q][1][w][h] = g[q].a.b;
    tiles[q][2][w][h] = g[q].b.a;
    tiles[q][3][w][h] = g[q].b.b;
  }
  __syncthreads();
  const uint32_t* r = b.runs + 4 * (size_t)b.run0[col];
  const uint32_t* hoff = b.runs + 4 * (size_t)b.hoff0[col] + 4 * w;  // segment h = w
  for (uint32_t q = 0; q < n_tiles; q++) {
    // warp w: natural run (h = w, ms[q]); lanes are lo
    uint32_t x[4];
#pragma unroll
    for (int k = 0; k < 4; k++) x[k] = tiles[q][k][t][w];
    warp_scan4(x);
    const uint32_t run = (w << mb) | ms[q];
#pragma unroll
    for (int k = 0; k < 4; k++) tiles[q][k][t][w] = m31_add(m31_add(x[k], r[4 * run + k]), hoff[k]);
  }
  __syncthreads();
  const qm31 total = qm31_make(b.claimed[4 * col], b.claimed[4 * col + 1], b.claimed[4 * col + 2],
                               b.claimed[4 * col + 3]);
  for (uint32_t q = 0; q < n_tiles; q++) {
    // element (h, ms[q], lo = w); its mirror (31 - h, ms[1 - q], 31 - w) is in the other tile
    // (the same one when m = m')
    const uint32_t o = n_tiles == 1 ? 0 : 1 - q;
    const qm31 qp = qm31_make(tiles[q][0][w][h], tiles[q][1][w][h], tiles[q][2][w][h], tiles[q][3][w][h]);
    const qm31 qm = qm31_make(tiles[o][0][31 - w][31 - h], tiles[o][1][31 - w][31 - h], tiles[o][2][31 - w][31 - h],
                              tiles[o][3][31 - w][31 - h]);
    const uint32_t c = (h << (log_n - 5)) | (ms[q] << 5) | w;
    store4(b, col, pos[q], running_value(c, log_n, qp, qm, g[q], total));
  }
}

// Runs the three launches over columns [0, n) of the tables; claimed sums to d_claimed (4 words each).
cs_status scan_columns(const uint32_t* const* values, const Q4* outs, const uint32_t* log_sizes, uint32_t n,
                       const qm31& z, uint32_t* d_claimed, cudaStream_t st) {
  uint64_t all_runs = 0;  // run totals, then 32 segment offsets, per column of 2^10 or more rows
  for (uint32_t i = 0; i < n; i++)
    if (log_sizes[i] > kSmallLog) all_runs += (1ull << (log_sizes[i] - 5)) + 32;
  uint32_t* runs = nullptr;
  CS_CUDA(stream_alloc(reinterpret_cast<void**>(&runs), sizeof(uint32_t) * 4 * std::max<uint64_t>(1, all_runs), st));
  cs_status result = CS_OK;
  uint64_t run_base = 0;
  for (uint32_t b0 = 0; b0 < n && result == CS_OK; b0 += kSumBatch) {
    SumBatch b;
    b.n_cols = std::min<uint32_t>(kSumBatch, n - b0);
    b.z = z;
    b.claimed = d_claimed + 4 * b0;
    b.runs = runs;
    uint32_t tiles = 0, pairs = 0;
    for (uint32_t i = 0; i < b.n_cols; i++) {
      const uint32_t l = log_sizes[b0 + i];
      b.values[i] = values != nullptr ? values[b0 + i] : nullptr;
      for (int c = 0; c < 4; c++) b.out[i][c] = outs[b0 + i].c[c];
      b.log_size[i] = l;
      b.tile0[i] = tiles;
      b.pair0[i] = pairs;
      b.run0[i] = (uint32_t)run_base;
      b.hoff0[i] = 0;
      if (l <= kSmallLog) {
        tiles += 1;
      } else {
        tiles += 1u << (l - 10);
        pairs += l == 10 ? 1 : 1u << (l - 11);
        b.hoff0[i] = (uint32_t)(run_base + (1ull << (l - 5)));
        run_base += (1ull << (l - 5)) + 32;
      }
    }
    b.tile0[b.n_cols] = tiles;
    b.pair0[b.n_cols] = pairs;
    runs_kernel<<<tiles, kThreads / 2, 0, st>>>(b);
    note_launch();
    if (pairs > 0) {
      run_offsets_kernel<<<b.n_cols, kThreads, 0, st>>>(b);
      note_launch();
      outputs_kernel<<<pairs, kThreads, 0, st>>>(b);
      note_launch();
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) result = from_cuda(e, "logup running sum launch");
  }
  cudaError_t e = cudaFreeAsync(runs, st);
  if (result == CS_OK && e != cudaSuccess) return from_cuda(e, "cudaFreeAsync");
  return result;
}

constexpr uint32_t kCompBatch = 24;  // LogUp components per launch

// rc ((cur - prev + shift)(v - z) + 1) = (v rc - rc z)(cur - prev + shift) + rc: per component the
// weight rc and rc z, per launch the sum of the weights.
struct LookupCompParams {
  const uint32_t* values[kCompBatch];  // each component's trace column on the evaluation domain
  const uint32_t* inter[kCompBatch][4];
  qm31 shift[kCompBatch], rc[kCompBatch], rcz[kCompBatch];
  qm31 rc_sum;
  uint32_t den[32];
  uint32_t n_comp, eval_log, trace_log;
};

// Quotients of single-column LogUp components of one size: per evaluation row, the sum over the
// components of rc (cur - prev + shift) (v - z) + 1, over V_trace, added to the accumulator once.
// Components go in pairs whose 18 loads are issued before either is evaluated.
struct LookupRow {
  uint32_t v, cur[4], prev[4];
};

__device__ __forceinline__ void load_lookup_row(const LookupCompParams& p, uint32_t k, uint32_t r, uint32_t pr,
                                                LookupRow& o) {
  const uint32_t* const* in = p.inter[k];
  o.v = __ldg(p.values[k] + r);
#pragma unroll
  for (int c = 0; c < 4; c++) {
    o.cur[c] = __ldg(in[c] + r);
    o.prev[c] = __ldg(in[c] + pr);
  }
}

// (v rc - rc z)(cur - prev + shift); the rc term is added once per launch (rc_sum).
__device__ __forceinline__ qm31 lookup_term(const LookupCompParams& p, uint32_t k, const LookupRow& o) {
  const qm31 cur = qm31_make(o.cur[0], o.cur[1], o.cur[2], o.cur[3]);
  const qm31 prev = qm31_make(o.prev[0], o.prev[1], o.prev[2], o.prev[3]);
  const qm31 shifted = qm31_add(qm31_sub(cur, prev), p.shift[k]);
  return qm31_mul(qm31_sub(qm31_mul_m31(p.rc[k], o.v), p.rcz[k]), shifted);
}

__global__ void lookup_composition_kernel(const __grid_constant__ LookupCompParams p, uint32_t* a0, uint32_t* a1,
                                          uint32_t* a2, uint32_t* a3) {
  const uint32_t n = 1u << p.eval_log;
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    const uint32_t pr = prev_row(r, p.trace_log, p.eval_log);
    qm31 acc = p.rc_sum;
    uint32_t k = 0;
    for (; k + 2 <= p.n_comp; k += 2) {
      LookupRow x, y;
      load_lookup_row(p, k, r, pr, x);
      load_lookup_row(p, k + 1, r, pr, y);
      acc = qm31_add(acc, qm31_add(lookup_term(p, k, x), lookup_term(p, k + 1, y)));
    }
    if (k < p.n_comp) {
      LookupRow x;
      load_lookup_row(p, k, r, pr, x);
      acc = qm31_add(acc, lookup_term(p, k, x));
    }
    const qm31 v = qm31_mul_m31(acc, p.den[r >> p.trace_log]);
    a0[r] = m31_add(a0[r], v.a.a);
    a1[r] = m31_add(a1[r], v.a.b);
    a2[r] = m31_add(a2[r], v.b.a);
    a3[r] = m31_add(a3[r], v.b.b);
  }
}

cpoint lookup_point_at(uint32_t idx) {
  cpoint r{1, 0}, cur{2u, 1268011823u};
  while (idx) {
    if (idx & 1) r = cpoint_add(r, cur);
    cur = cpoint_add(cur, cur);
    idx >>= 1;
  }
  return r;
}

// LookupElements::combine (crates/constraint-framework/src/logup.rs:80-94) per row over up to
// kCombineBatch value columns: den = sum_i alpha^i values_i - z; later batches of a call add on.
constexpr uint32_t kCombineBatch = 32;
struct CombineBatch {
  const uint32_t* values[kCombineBatch];
  qm31 alpha[kCombineBatch];
  uint32_t n;
  uint32_t first;  // the first batch: subtract z and store; otherwise add to the output
  qm31 z;
};

__global__ void logup_combine_kernel(const __grid_constant__ CombineBatch b, uint32_t n_rows, uint32_t* o0,
                                     uint32_t* o1, uint32_t* o2, uint32_t* o3) {
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n_rows; r += gridDim.x * blockDim.x) {
    qm31 acc = b.first ? qm31_neg(b.z) : qm31_make(o0[r], o1[r], o2[r], o3[r]);
    for (uint32_t i = 0; i < b.n; i++) acc = qm31_add(acc, qm31_mul_m31(b.alpha[i], __ldg(b.values[i] + r)));
    o0[r] = acc.a.a;
    o1[r] = acc.a.b;
    o2[r] = acc.b.a;
    o3[r] = acc.b.b;
  }
}

// LogupColGenerator::write_frac for every row, then finalize_col (crates/constraint-framework/src/
// prover/logup.rs:133-196): out = num / den + prev, the inverse per row (qm31_inv; the reference's
// batch inversion gives the same values), num QM31 (num0..3) or M31 (num_m31), prev optional.
struct FracCol {
  const uint32_t* num[4];
  const uint32_t* num_m31;
  const uint32_t* den[4];
  const uint32_t* prev[4];
  uint32_t* out[4];
};

__global__ void logup_frac_kernel(const FracCol f, uint32_t n_rows) {
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n_rows; r += gridDim.x * blockDim.x) {
    const qm31 den = qm31_make(__ldg(f.den[0] + r), __ldg(f.den[1] + r), __ldg(f.den[2] + r), __ldg(f.den[3] + r));
    const qm31 inv = qm31_inv(den);
    qm31 v = f.num_m31 != nullptr
                 ? qm31_mul_m31(inv, __ldg(f.num_m31 + r))
                 : qm31_mul(qm31_make(__ldg(f.num[0] + r), __ldg(f.num[1] + r), __ldg(f.num[2] + r),
                                      __ldg(f.num[3] + r)),
                            inv);
    if (f.prev[0] != nullptr)
      v = qm31_add(v, qm31_make(__ldg(f.prev[0] + r), __ldg(f.prev[1] + r), __ldg(f.prev[2] + r),
                                __ldg(f.prev[3] + r)));
    f.out[0][r] = v.a.a;
    f.out[1][r] = v.a.b;
    f.out[2][r] = v.b.a;
    f.out[3][r] = v.b.b;
  }
}

uint32_t rows_grid(uint32_t n) { return std::max(1u, std::min<uint32_t>((n + 255) / 256, 152 * 8)); }

}  // namespace

cs_status logup_finalize_last(Q4 col, uint32_t log_size, uint32_t claimed_sum_out[4], cudaStream_t st) {
  uint32_t* d_claimed = nullptr;
  CS_CUDA(stream_alloc(reinterpret_cast<void**>(&d_claimed), sizeof(uint32_t) * 4, st));
  cs_status result = scan_columns(nullptr, &col, &log_size, 1, qm31_make(0, 0, 0, 0), d_claimed, st);
  if (result == CS_OK) {
    cudaError_t e = cudaMemcpyAsync(claimed_sum_out, d_claimed, sizeof(uint32_t) * 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) result = from_cuda(e, "logup finalize");
  }
  cudaError_t e = cudaFreeAsync(d_claimed, st);
  if (result == CS_OK && e != cudaSuccess) return from_cuda(e, "cudaFreeAsync");
  return result;
}

}  // namespace cs

using namespace cs;

extern "C" cs_status cs_logup_running_sum(const uint32_t* d_values, uint32_t log_size, const uint32_t z[4],
                                          uint32_t* const h_out[4], uint32_t claimed_sum_out[4], cs_stream stream) {
  CS_CHECK_ARG(d_values != nullptr && z != nullptr && h_out != nullptr && claimed_sum_out != nullptr,
               "logup_running_sum: null pointer");
  CS_CHECK_ARG(log_size >= 1 && log_size <= 28, "logup_running_sum: log size %u outside [1, 28]", log_size);
  Q4 out;
  for (int c = 0; c < 4; c++) {
    CS_CHECK_ARG(h_out[c] != nullptr, "logup_running_sum: null output coordinate");
    out.c[c] = h_out[c];
  }
  cudaStream_t st = to_stream(stream);
  uint32_t* d_claimed = nullptr;
  CS_CUDA(stream_alloc(reinterpret_cast<void**>(&d_claimed), sizeof(uint32_t) * 4, st));
  cs_status result = scan_columns(&d_values, &out, &log_size, 1, qm31_make(z[0], z[1], z[2], z[3]), d_claimed, st);
  if (result == CS_OK) {
    cudaError_t e = cudaMemcpyAsync(claimed_sum_out, d_claimed, sizeof(uint32_t) * 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) result = from_cuda(e, "logup_running_sum");
  }
  cudaError_t e = cudaFreeAsync(d_claimed, st);
  if (result == CS_OK && e != cudaSuccess) return from_cuda(e, "cudaFreeAsync");
  return result;
}

extern "C" cs_status cs_logup_running_sums(uint32_t n_cols, const uint32_t* const* h_values,
                                           const uint32_t* h_log_sizes, const uint32_t z[4],
                                           uint32_t* const* h_out, uint32_t* d_claimed, cs_stream stream) {
  CS_CHECK_ARG(n_cols == 0 || (h_values != nullptr && h_log_sizes != nullptr && h_out != nullptr),
               "logup_running_sums: null table");
  CS_CHECK_ARG(z != nullptr && (n_cols == 0 || d_claimed != nullptr), "logup_running_sums: null pointer");
  std::vector<Q4> outs(n_cols);
  for (uint32_t i = 0; i < n_cols; i++) {
    CS_CHECK_ARG(h_values[i] != nullptr, "logup_running_sums: column %u has no values", i);
    CS_CHECK_ARG(h_log_sizes[i] >= 1 && h_log_sizes[i] <= 28, "logup_running_sums: column %u log size %u outside "
                 "[1, 28]", i, h_log_sizes[i]);
    for (int c = 0; c < 4; c++) {
      CS_CHECK_ARG(h_out[4 * i + c] != nullptr, "logup_running_sums: column %u coordinate %d is null", i, c);
      outs[i].c[c] = h_out[4 * i + c];
    }
  }
  if (n_cols == 0) return CS_OK;
  return scan_columns(h_values, outs.data(), h_log_sizes, n_cols, qm31_make(z[0], z[1], z[2], z[3]), d_claimed,
                      to_stream(stream));
}

extern "C" cs_status cs_logup_compositions(uint32_t n_comp, const uint32_t* const* h_values,
                                           const uint32_t* const* h_inter, uint32_t eval_log, uint32_t trace_log,
                                           const uint32_t z[4], const uint32_t* claimed_sums, const uint32_t* rcs,
                                           uint32_t* const h_accum[4], cs_stream stream) {
  CS_CHECK_ARG(z != nullptr && h_accum != nullptr, "logup_compositions: null pointer");
  CS_CHECK_ARG(n_comp == 0 || (h_values != nullptr && h_inter != nullptr && claimed_sums != nullptr && rcs != nullptr),
               "logup_compositions: null table");
  CS_CHECK_ARG(trace_log >= 1 && eval_log >= trace_log && eval_log - trace_log <= 5 && eval_log <= 30,
               "logup_compositions: bad sizes eval %u trace %u", eval_log, trace_log);
  for (int c = 0; c < 4; c++) CS_CHECK_ARG(h_accum[c] != nullptr, "logup_compositions: null accumulator");
  for (uint32_t k = 0; k < n_comp; k++) {
    CS_CHECK_ARG(h_values[k] != nullptr, "logup_compositions: component %u has no values", k);
    for (int c = 0; c < 4; c++)
      CS_CHECK_ARG(h_inter[4 * k + c] != nullptr, "logup_compositions: component %u coordinate %d is null", k, c);
  }
  static thread_local LookupCompParams p;
  const qm31 zz = qm31_make(z[0], z[1], z[2], z[3]);
  p.eval_log = eval_log;
  p.trace_log = trace_log;
  const uint32_t log_expand = eval_log - trace_log, n_den = 1u << log_expand;
  if (log_expand == 0) {
    p.den[0] = 1;
  } else {
    // 1 / V_trace(eval_domain.at(i)), bit-reversed (component_prover.rs:101-108)
    for (uint32_t i = 0; i < n_den; i++) {
      const uint32_t idx = (subgroup_gen(eval_log + 1) + i * subgroup_gen(eval_log - 1)) & 0x7fffffffu;
      uint32_t x = lookup_point_at(idx).x;
      for (uint32_t k = 1; k < trace_log; k++) x = m31_sub(m31_add(m31_sqr(x), m31_sqr(x)), 1);
      uint32_t j = 0;
      for (uint32_t b = 0; b < log_expand; b++) j |= ((i >> b) & 1u) << (log_expand - 1 - b);
      p.den[j] = m31_inv(x);
    }
  }
  const uint32_t n = 1u << eval_log;
  const uint32_t blocks = std::max(1u, std::min((n + 255) / 256, 152u * 8));
  for (uint32_t k0 = 0; k0 < n_comp; k0 += kCompBatch) {
    p.n_comp = std::min(kCompBatch, n_comp - k0);
    p.rc_sum = qm31_make(0, 0, 0, 0);
    for (uint32_t i = 0; i < p.n_comp; i++) {
      const uint32_t k = k0 + i;
      p.values[i] = h_values[k];
      for (int c = 0; c < 4; c++) p.inter[i][c] = h_inter[4 * k + c];
      p.rc[i] = qm31_make(rcs[4 * k] % P, rcs[4 * k + 1] % P, rcs[4 * k + 2] % P, rcs[4 * k + 3] % P);
      p.rcz[i] = qm31_mul(p.rc[i], zz);
      p.rc_sum = qm31_add(p.rc_sum, p.rc[i]);
      // cumsum_shift = claimed_sum / 2^trace_log (LogupAtRow::new, crates/constraint-framework/src/logup.rs:32-40)
      p.shift[i] = qm31_mul_m31(qm31_make(claimed_sums[4 * k], claimed_sums[4 * k + 1], claimed_sums[4 * k + 2],
                                          claimed_sums[4 * k + 3]),
                                1u << (31 - trace_log));
    }
    lookup_composition_kernel<<<blocks, 256, 0, to_stream(stream)>>>(p, h_accum[0], h_accum[1], h_accum[2],
                                                                      h_accum[3]);
    CS_LAUNCHED("lookup_composition_kernel");
  }
  return CS_OK;
}

extern "C" cs_status cs_logup_composition(const uint32_t* d_values, const uint32_t* const h_inter[4], uint32_t eval_log,
                                          uint32_t trace_log, const uint32_t z[4], const uint32_t claimed_sum[4],
                                          const uint32_t rc[4], uint32_t* const h_accum[4], cs_stream stream) {
  CS_CHECK_ARG(d_values != nullptr && h_inter != nullptr && claimed_sum != nullptr && rc != nullptr,
               "logup_composition: null pointer");
  return cs_logup_compositions(1, &d_values, h_inter, eval_log, trace_log, z, claimed_sum, rc, h_accum, stream);
}

extern "C" cs_status cs_logup_combine(const uint32_t* const* h_values, uint32_t n_values, uint32_t log_size,
                                      const uint32_t* alpha_powers, const uint32_t z[4], uint32_t* const h_den[4],
                                      cs_stream stream) {
  CS_CHECK_ARG(h_values != nullptr && alpha_powers != nullptr && z != nullptr && h_den != nullptr,
               "logup_combine: null pointer");
  CS_CHECK_ARG(n_values >= 1, "logup_combine: no values");
  CS_CHECK_ARG(log_size <= 30, "logup_combine: log size %u", log_size);
  for (int c = 0; c < 4; c++) CS_CHECK_ARG(h_den[c] != nullptr, "logup_combine: null output coordinate");
  cudaStream_t st = to_stream(stream);
  const uint32_t n = 1u << log_size;
  for (uint32_t b0 = 0; b0 < n_values; b0 += kCombineBatch) {
    CombineBatch b;
    b.n = std::min(kCombineBatch, n_values - b0);
    b.first = b0 == 0;
    b.z = qm31_make(z[0] % P, z[1] % P, z[2] % P, z[3] % P);
    for (uint32_t i = 0; i < b.n; i++) {
      CS_CHECK_ARG(h_values[b0 + i] != nullptr, "logup_combine: value column %u is null", b0 + i);
      b.values[i] = h_values[b0 + i];
      const uint32_t* a = alpha_powers + 4 * (size_t)(b0 + i);
      b.alpha[i] = qm31_make(a[0] % P, a[1] % P, a[2] % P, a[3] % P);
    }
    logup_combine_kernel<<<rows_grid(n), 256, 0, st>>>(b, n, h_den[0], h_den[1], h_den[2], h_den[3]);
    CS_LAUNCHED("logup_combine_kernel");
  }
  return CS_OK;
}

extern "C" cs_status cs_logup_gen_col(const uint32_t* const* h_num, const uint32_t* d_num_m31,
                                      const uint32_t* const h_den[4], const uint32_t* const* h_prev,
                                      uint32_t log_size, uint32_t* const h_out[4], cs_stream stream) {
  CS_CHECK_ARG(h_den != nullptr && h_out != nullptr, "logup_gen_col: null pointer");
  CS_CHECK_ARG((h_num != nullptr) != (d_num_m31 != nullptr),
               "logup_gen_col: give exactly one numerator (QM31 coordinates or an M31 column)");
  CS_CHECK_ARG(log_size <= 30, "logup_gen_col: log size %u", log_size);
  FracCol f;
  for (int c = 0; c < 4; c++) {
    CS_CHECK_ARG(h_den[c] != nullptr && h_out[c] != nullptr, "logup_gen_col: null coordinate");
    f.num[c] = h_num != nullptr ? h_num[c] : nullptr;
    CS_CHECK_ARG(h_num == nullptr || f.num[c] != nullptr, "logup_gen_col: null numerator coordinate");
    f.den[c] = h_den[c];
    f.prev[c] = h_prev != nullptr ? h_prev[c] : nullptr;
    CS_CHECK_ARG(h_prev == nullptr || f.prev[c] != nullptr, "logup_gen_col: null previous-column coordinate");
    f.out[c] = h_out[c];
  }
  f.num_m31 = d_num_m31;
  const uint32_t n = 1u << log_size;
  logup_frac_kernel<<<rows_grid(n), 256, 0, to_stream(stream)>>>(f, n);
  CS_LAUNCHED("logup_frac_kernel");
  return CS_OK;
}

extern "C" cs_status cs_logup_finalize_last(uint32_t* const h_col[4], uint32_t log_size, uint32_t claimed_sum_out[4],
                                            cs_stream stream) {
  CS_CHECK_ARG(h_col != nullptr && claimed_sum_out != nullptr, "logup_finalize_last: null pointer");
  CS_CHECK_ARG(log_size >= 1 && log_size <= 28, "logup_finalize_last: log size %u outside [1, 28]", log_size);
  Q4 col;
  for (int c = 0; c < 4; c++) {
    CS_CHECK_ARG(h_col[c] != nullptr, "logup_finalize_last: null coordinate");
    col.c[c] = h_col[c];
  }
  return logup_finalize_last(col, log_size, claimed_sum_out, to_stream(stream));
}
