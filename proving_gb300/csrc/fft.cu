// Circle FFT over M31 on sm_103a: interpolate (inverse) and evaluate (forward)
// on canonic circle domains, bit-reversed order, bit-exact with
// crates/stwo/src/prover/backend/cpu/circle.rs:26-79 (interpolate) and
// :187-238 (evaluate_into).
//
// Layer i (0 = the circle layer, i >= 1 line layers) pairs indices
// (g, g + 2^i) with bit i of g clear, twiddle index h = g >> (i+1)
// (fft_layer_loop, cpu/circle.rs:287-301). Line layer i reads the twiddle tree
// at tw[2^K - 2^(n-i) + h] (domain_line_twiddles_from_tree,
// crates/stwo/src/core/poly/utils.rs:98-111); the circle layer derives
// [y, -y, -x, x] from line layer 1 (cpu/circle.rs:306-323).
//
// A column of 2^n words is processed in passes. A pass owns a contiguous range
// of layers [lo, hi): every group of 2^(hi-lo) elements that differ only in
// index bits [lo, hi) is independent for those layers. A CTA stages one tile —
// such a group times 2^c neighbouring groups, chosen so global accesses are
// contiguous runs — in shared memory, runs the layers as radix-8 register
// stages, and writes the tile back. Evaluate's first pass reads each
// coefficient tile once from the (shorter) coefficient column: the
// zero-padded top layers are identities, so every blown-up replica starts
// from the same coefficients; replicas of a tile are adjacent CTAs and share
// the read through L2. Interpolate's last pass folds in the 1/n scaling.
#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "common.cuh"
#include "field.cuh"

namespace cs {

namespace {


struct FftBatch {
  uint32_t* dst[kMaxBatch];
  const uint32_t* src[kMaxBatch];
};

struct FftPass {
  uint32_t log_n;     // column log size
  uint32_t lo, hi;    // layers [lo, hi)
  uint32_t c;         // extra tile bits
  uint32_t outer;     // 1: extra bits are index bits [hi, hi + c); 0: bits [0, c) (requires lo >= c)
  uint32_t src_mask;  // source index mask: replicated reads for evaluate's first pass
  uint32_t scale;     // 0: none; else outputs are multiplied by it
  const uint32_t* tw; // twiddle (forward) or itwiddle (inverse) tree
  uint32_t tw_log;    // log2 of the tree length
  uint32_t tw_dom;    // log size of the canonic domain whose twiddle layers are used (>= log_n;
                      // larger for a subdomain, which takes the prefix of each layer)
  uint32_t vec;       // 1: every column is 16-byte aligned and the source mask keeps runs of 4,
                      // so tiles move between HBM and shared memory as 16-byte words
};

struct Tile {
  uint32_t o, ib;  // outer group and inner block (inner tiles) / first outer group (outer tiles)
};

__device__ __forceinline__ uint32_t tile_gidx(const FftPass& p, const Tile& t, uint32_t m, uint32_t e) {
  if (p.outer) return ((t.o + e) << p.hi) | m;
  return (t.o << p.hi) | (m << p.lo) | (t.ib << p.c) | e;
}

__device__ __forceinline__ void bfly(uint32_t& v0, uint32_t& v1, uint32_t t) {
  // butterfly, crates/stwo/src/core/fft.rs:5-12
  const uint32_t tmp = m31_mul(v1, t);
  v1 = m31_sub(v0, tmp);
  v0 = m31_add(v0, tmp);
}
__device__ __forceinline__ void ibfly(uint32_t& v0, uint32_t& v1, uint32_t t) {
  // ibutterfly, crates/stwo/src/core/fft.rs:14-21
  const uint32_t tmp = v0;
  v0 = m31_add(tmp, v1);
  v1 = m31_mul(m31_sub(tmp, v1), t);
}

// The tile kernels multiply by doubled twiddles t2 = 2t (at most 2^32 - 4): the 64-bit product
// a * t2 is a*t shifted left by one, so its high word is (a*t) >> 31 and its low word shifted
// right by one is (a*t) mod 2^31, which saves the masking of the plain reduction.
__device__ __forceinline__ uint32_t mul_doubled(uint32_t a, uint32_t t2) {
  const uint64_t q = (uint64_t)a * t2;
  return m31_reduce_once(((uint32_t)q >> 1) + (uint32_t)(q >> 32));
}
__device__ __forceinline__ void bfly2(uint32_t& v0, uint32_t& v1, uint32_t t2) {
  const uint32_t tmp = mul_doubled(v1, t2);
  v1 = m31_sub(v0, tmp);
  v0 = m31_add(v0, tmp);
}
__device__ __forceinline__ void ibfly2(uint32_t& v0, uint32_t& v1, uint32_t t2) {
  const uint32_t tmp = v0;
  v0 = m31_add(tmp, v1);
  v1 = mul_doubled(m31_sub(tmp, v1), t2);
}

// Shared-memory layout of a tile. Outer (contiguous) tiles hold [e][m] and
// insert one pad word per 32; inner (strided) tiles hold [m][e] with 8 values
// of e and insert 8 pad words per 256. Both make every 32-wide access of the
// two register stages and of the global load/store phase hit distinct banks,
// and keep a register group's addresses at compile-time offsets from one base.
template <bool OUTER>
__device__ __forceinline__ uint32_t pad(uint32_t L) {
  return OUTER ? L + (L >> 5) : L + ((L >> 8) << 3);
}

template <bool OUTER>
__host__ __device__ constexpr uint32_t padded_words(uint32_t n) {
  return OUTER ? n + (n >> 5) : n + ((n >> 8) << 3);
}

template <bool OUTER>
__device__ __forceinline__ uint32_t lin(uint32_t m, uint32_t e, int T, uint32_t EB) {
  return OUTER ? ((e << T) | m) : ((m << EB) | e);
}

// CNT consecutive twiddles of FFT layer `layer`, starting at twiddle index h0.
template <int CNT, bool CIRCLE>
__device__ __forceinline__ void load_twiddles(const FftPass& p, uint32_t layer, uint32_t h0, uint32_t* w) {
  const uint32_t tw_len = 1u << p.tw_log;
  if (CIRCLE) {
    // circle layer: [y, -y, -x, x] of the line-layer-1 pair (cpu/circle.rs:306-323)
    const uint32_t* lt1 = p.tw + (tw_len - (1u << (p.tw_dom - 1)));
    if (CNT >= 16) {
      // h0 is a multiple of 16: pairs (h0 >> 2) .. + 3, 8 aligned words
#pragma unroll
      for (int q8 = 0; q8 < CNT / 8; q8++) {
        const uint4 v = __ldg(reinterpret_cast<const uint4*>(lt1 + ((h0 >> 2) << 1)) + q8);
        const uint32_t xs[2] = {v.x, v.z}, ys[2] = {v.y, v.w};
#pragma unroll
        for (int k = 0; k < 2; k++) {
          w[8 * q8 + 4 * k + 0] = ys[k];
          w[8 * q8 + 4 * k + 1] = m31_neg(ys[k]);
          w[8 * q8 + 4 * k + 2] = m31_neg(xs[k]);
          w[8 * q8 + 4 * k + 3] = xs[k];
        }
      }
    } else {
#pragma unroll
      for (int q = 0; q < CNT; q++) {
        const uint32_t h = h0 + q;
        const uint32_t pair = (h >> 2) << 1;
        const uint32_t x = __ldg(lt1 + pair), y = __ldg(lt1 + pair + 1);
        const uint32_t sel = h & 3;
        const uint32_t val = sel < 2 ? y : x;
        w[q] = (sel == 1 || sel == 2) ? m31_neg(val) : val;
      }
    }
    return;
  }
  const uint32_t* lt = p.tw + (tw_len - (1u << (p.tw_dom - layer))) + h0;
  if (CNT >= 4) {
#pragma unroll
    for (int q = 0; q < CNT / 4; q++) {
      const uint4 v = __ldg(reinterpret_cast<const uint4*>(lt) + q);
      w[4 * q] = v.x;
      w[4 * q + 1] = v.y;
      w[4 * q + 2] = v.z;
      w[4 * q + 3] = v.w;
    }
  } else {
#pragma unroll
    for (int q = 0; q < CNT; q++) w[q] = __ldg(lt + q);
  }
}


// R local layers [D0, D0 + R) on the 2^R register values v, whose local index
// j maps to global index g0 + (j << (D0 + lo)). INV runs the layers upward
// with ibutterflies (interpolate), otherwise downward with butterflies. Local
// layer t needs 2^(R-1-t) consecutive twiddles. Only contiguous tiles
// (OUTER, lo = 0) contain the circle layer: local layer 0 of stage A.
template <int R>
__host__ __device__ constexpr int tw_off(int t) {
  return (1 << R) - (1 << (R - t));
}

template <bool INV, bool OUTER, int R, int D0, int K>
struct Layers {
  static __device__ __forceinline__ void run(const FftPass& p, uint32_t g0, uint32_t* v, uint32_t* w) {
    constexpr int t = INV ? K : (R - 1 - K);
    {
      const uint32_t layer = p.lo + D0 + t;
      load_twiddles<(1 << (R - 1 - t)), OUTER && D0 == 0 && t == 0>(p, layer, g0 >> (layer + 1), w + tw_off<R>(t));
#pragma unroll
      for (int q = 0; q < (1 << (R - 1 - t)); q++) w[tw_off<R>(t) + q] <<= 1;
    }
#pragma unroll
    for (int j = 0; j < (1 << R); j++) {
      if (j & (1 << t)) continue;
      if (INV)
        ibfly2(v[j], v[j | (1 << t)], w[tw_off<R>(t) + (j >> (t + 1))]);
      else
        bfly2(v[j], v[j | (1 << t)], w[tw_off<R>(t) + (j >> (t + 1))]);
    }
    Layers<INV, OUTER, R, D0, K + 1>::run(p, g0, v, w);
  }
};
template <bool INV, bool OUTER, int R, int D0>
struct Layers<INV, OUTER, R, D0, R> {
  static __device__ __forceinline__ void run(const FftPass&, uint32_t, uint32_t*, uint32_t*) {}
};

template <bool INV, bool OUTER, int R, int D0>
__device__ __forceinline__ void reg_stage(const FftPass& p, uint32_t g0, uint32_t* v) {
  uint32_t w[1 << R];  // 2^R - 1 used
  Layers<INV, OUTER, R, D0, 0>::run(p, g0, v, w);
}

// One pass over layers [lo, lo + T) of a tile of 2^T x 2^EB values: stage A
// runs local layers [0, TA) on groups m = (ma << TA) | j, stage B runs
// [TA, T) on groups m = (j << TA) | mb, with one shared-memory exchange.
template <int T, bool OUTER>
constexpr int tile_max_threads() {
  return OUTER ? 256 : (1 << (T / 2 + 3));
}
// Blocks per SM the register budget is sized for: tiles of up to 10 layers fit
// four (64 registers) without spills, larger ones two. Four blocks keep more
// tile loads in flight: the strided evaluate pass, which reads each coefficient
// tile once for its replicas, is otherwise bound by its load latency.
template <int T, bool OUTER>
constexpr int tile_min_blocks() {
  return T <= 10 ? 4 : 2;
}

template <bool INV, int T, bool OUTER>
__global__ void __launch_bounds__(tile_max_threads<T, OUTER>(), tile_min_blocks<T, OUTER>()) fft_tile_kernel(const FftBatch batch, const FftPass p) {
  constexpr int TA = T / 2, TB = T - TA;
  constexpr uint32_t M = 1u << T;
  extern __shared__ __align__(16) uint32_t s[];
  const uint32_t EB = OUTER ? p.c : 3u;  // inner tiles always hold 8 groups
  uint32_t* dst = batch.dst[blockIdx.y];
  const uint32_t* src = batch.src[blockIdx.y];
  Tile tl;
  if (OUTER) {
    tl.o = blockIdx.x << EB;
    tl.ib = 0;
  } else {
    const uint32_t outer_bits = p.log_n - p.hi;
    tl.o = blockIdx.x & ((1u << outer_bits) - 1);
    tl.ib = blockIdx.x >> outer_bits;
  }
  // every thread moves exactly 2^TB words (the tile holds 2^(T + EB) words, the block has
  // 2^(TA + EB) threads); up to 32 of a thread's loads are in flight before its first store.
  // With p.vec a thread moves four consecutive tile words at a time: four consecutive tile slots
  // are four consecutive column words in both layouts (contiguous tiles: the group index fills the
  // low bits; strided tiles: a group is 8 adjacent words), and the padding keeps the four together
  // (a 16-byte-aligned run for strided tiles; for contiguous tiles one pad word per 32 shifts each
  // 8-lane group by one bank, so the four scalar stores of a warp hit 32 distinct banks).
  constexpr bool kVecOk = TB >= 2;
  if (kVecOk && p.vec) {
    constexpr int GQ = (1 << TB) < 4 ? 1 : ((1 << TB) < 32 ? (1 << TB) : 32) / 4;  // tiles of 1 layer never get here
#pragma unroll 1
    for (int k0 = 0; k0 < (1 << TB) / 4; k0 += GQ) {
      uint4 r[GQ];
#pragma unroll
      for (int k = 0; k < GQ; k++) {
        const uint32_t L = 4 * (threadIdx.x + (k0 + k) * blockDim.x);
        const uint32_t m = OUTER ? (L & (M - 1)) : (L >> EB);
        const uint32_t e = OUTER ? (L >> T) : (L & ((1u << EB) - 1));
        r[k] = __ldg(reinterpret_cast<const uint4*>(src + (tile_gidx(p, tl, m, e) & p.src_mask)));
      }
#pragma unroll
      for (int k = 0; k < GQ; k++) {
        uint32_t* d = s + pad<OUTER>(4 * (threadIdx.x + (k0 + k) * blockDim.x));
        if (OUTER) {
          d[0] = r[k].x;
          d[1] = r[k].y;
          d[2] = r[k].z;
          d[3] = r[k].w;
        } else {
          *reinterpret_cast<uint4*>(d) = r[k];
        }
      }
    }
  } else {
    constexpr int G = (1 << TB) < 32 ? (1 << TB) : 32;
#pragma unroll 1
    for (int k0 = 0; k0 < (1 << TB); k0 += G) {
      uint32_t r[G];
#pragma unroll
      for (int k = 0; k < G; k++) {
        const uint32_t L = threadIdx.x + (k0 + k) * blockDim.x;
        const uint32_t m = OUTER ? (L & (M - 1)) : (L >> EB);
        const uint32_t e = OUTER ? (L >> T) : (L & ((1u << EB) - 1));
        r[k] = __ldg(src + (tile_gidx(p, tl, m, e) & p.src_mask));
      }
#pragma unroll
      for (int k = 0; k < G; k++) s[pad<OUTER>(threadIdx.x + (k0 + k) * blockDim.x)] = r[k];
    }
  }
  __syncthreads();
  const uint32_t t = threadIdx.x;
  for (int phase = 0; phase < 2; phase++) {
    const bool stage_a = INV ? phase == 0 : phase == 1;
    if (stage_a) {
      if (TA > 0) {
#pragma unroll 1
        for (uint32_t r = 0; r < (1u << (TB - TA)); r++) {
          const uint32_t e = OUTER ? (t >> TA) : (t & ((1u << EB) - 1));
          const uint32_t ma = (OUTER ? (t & ((1u << TA) - 1)) : (t >> EB)) + (r << TA);
          const uint32_t mbase = ma << TA;
          uint32_t v[1 << TA];
#pragma unroll
          for (int j = 0; j < (1 << TA); j++) v[j] = s[pad<OUTER>(lin<OUTER>(mbase | j, e, T, EB))];
          reg_stage<INV, OUTER, TA, 0>(p, tile_gidx(p, tl, mbase, e), v);
#pragma unroll
          for (int j = 0; j < (1 << TA); j++) s[pad<OUTER>(lin<OUTER>(mbase | j, e, T, EB))] = v[j];
        }
      }
    } else {
      const uint32_t e = OUTER ? (t >> TA) : (t & ((1u << EB) - 1));
      const uint32_t mb = OUTER ? (t & ((1u << TA) - 1)) : (t >> EB);
      uint32_t v[1 << TB];
#pragma unroll
      for (int j = 0; j < (1 << TB); j++) v[j] = s[pad<OUTER>(lin<OUTER>((j << TA) | mb, e, T, EB))];
      reg_stage<INV, OUTER, TB, TA>(p, tile_gidx(p, tl, mb, e), v);
#pragma unroll
      for (int j = 0; j < (1 << TB); j++) s[pad<OUTER>(lin<OUTER>((j << TA) | mb, e, T, EB))] = v[j];
    }
    __syncthreads();
  }
  if (kVecOk && p.vec) {
#pragma unroll 1
    for (int k0 = 0; k0 < (1 << TB) / 4; k0++) {
      const uint32_t L = 4 * (threadIdx.x + k0 * blockDim.x);
      const uint32_t m = OUTER ? (L & (M - 1)) : (L >> EB);
      const uint32_t e = OUTER ? (L >> T) : (L & ((1u << EB) - 1));
      const uint32_t* d = s + pad<OUTER>(L);
      uint4 v = OUTER ? make_uint4(d[0], d[1], d[2], d[3]) : *reinterpret_cast<const uint4*>(d);
      if (p.scale) {
        v.x = m31_mul(v.x, p.scale);
        v.y = m31_mul(v.y, p.scale);
        v.z = m31_mul(v.z, p.scale);
        v.w = m31_mul(v.w, p.scale);
      }
      *reinterpret_cast<uint4*>(dst + tile_gidx(p, tl, m, e)) = v;
    }
    return;
  }
  // stores in groups of four, which keeps the register budget of three blocks per SM
#pragma unroll 1
  for (int k0 = 0; k0 < (1 << TB); k0 += 4) {
#pragma unroll
    for (int k = 0; k < ((1 << TB) < 4 ? (1 << TB) : 4); k++) {
      const uint32_t L = threadIdx.x + (k0 + k) * blockDim.x;
      const uint32_t m = OUTER ? (L & (M - 1)) : (L >> EB);
      const uint32_t e = OUTER ? (L >> T) : (L & ((1u << EB) - 1));
      uint32_t v = s[pad<OUTER>(L)];
      if (p.scale) v = m31_mul(v, p.scale);
      dst[tile_gidx(p, tl, m, e)] = v;
    }
  }
}

// Domains of log size 1 and 2 use the half coset's first point directly
// (cpu/circle.rs:34-58 and :203-223). One thread per column.
struct SmallParams {
  uint32_t log_n;
  uint32_t log_src;
  uint32_t inverse;
  uint32_t k[4];  // precomputed constants, see small_constants()
};

__global__ void fft_small_kernel(const FftBatch batch, uint32_t n_cols, const SmallParams p) {
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n_cols) return;
  uint32_t v[4] = {0, 0, 0, 0};
  const uint32_t n = 1u << p.log_n, ns = 1u << p.log_src;
  for (uint32_t i = 0; i < ns; i++) v[i] = batch.src[c][i];
  if (p.log_n == 1) {
    if (p.inverse) {
      ibfly(v[0], v[1], p.k[0]);  // y_inv
      v[0] = m31_mul(v[0], p.k[1]);
      v[1] = m31_mul(v[1], p.k[1]);
    } else {
      bfly(v[0], v[1], p.k[0]);  // y
    }
  } else {
    if (p.inverse) {
      // k = {y_inv, x_inv, n_inv}
      ibfly(v[0], v[1], p.k[0]);
      ibfly(v[2], v[3], m31_neg(p.k[0]));
      ibfly(v[0], v[2], p.k[1]);
      ibfly(v[1], v[3], p.k[1]);
      for (int i = 0; i < 4; i++) v[i] = m31_mul(v[i], p.k[2]);
    } else {
      // k = {x, y}
      bfly(v[0], v[2], p.k[0]);
      bfly(v[1], v[3], p.k[0]);
      bfly(v[0], v[1], p.k[1]);
      bfly(v[2], v[3], m31_neg(p.k[1]));
    }
  }
  for (uint32_t i = 0; i < n; i++) batch.dst[c][i] = v[i];
}

cpoint index_to_point_host(uint32_t idx) {
  cpoint r{1, 0}, cur{2u, 1268011823u};
  while (idx) {
    if (idx & 1) r = cpoint_add(r, cur);
    cur = cpoint_add(cur, cur);
    idx >>= 1;
  }
  return r;
}

SmallParams small_constants(uint32_t log_n, uint32_t log_src, bool inverse, uint32_t tw_dom) {
  SmallParams sp{};
  sp.log_n = log_n;
  sp.log_src = log_src;
  sp.inverse = inverse ? 1 : 0;
  // The half coset of CanonicCoset(tw_dom) starts at index 2^(31 - (tw_dom + 1)); a subdomain
  // (its bit-reversed prefix) shares that first point.
  const cpoint init = index_to_point_host(subgroup_gen(tw_dom + 1));
  if (log_n == 1) {
    if (inverse) {
      const uint32_t nn = 2;
      const uint32_t yn_inv = m31_inv(m31_mul(init.y, nn));
      sp.k[0] = m31_mul(yn_inv, nn);
      sp.k[1] = m31_mul(yn_inv, init.y);
    } else {
      sp.k[0] = init.y;
    }
  } else {
    if (inverse) {
      const uint32_t nn = 4;
      const uint32_t xyn_inv = m31_inv(m31_mul(m31_mul(init.x, init.y), nn));
      sp.k[1] = m31_mul(m31_mul(xyn_inv, init.y), nn);  // x_inv
      sp.k[0] = m31_mul(m31_mul(xyn_inv, init.x), nn);  // y_inv
      sp.k[2] = m31_mul(m31_mul(xyn_inv, init.x), init.y);
    } else {
      sp.k[0] = init.x;
      sp.k[1] = init.y;
    }
  }
  return sp;
}

struct PassPlan {
  uint32_t lo, hi, c, outer;  // layers [lo, hi); c = extra tile bits
};

// Pass splits installed by an autotuner (cs_fft_set_plan), per (direction, column log size,
// number of layers); the default split below is used for every other shape.
struct PlanKey {
  uint32_t inverse, log_n, n_layers;
  bool operator<(const PlanKey& o) const {
    return std::tie(inverse, log_n, n_layers) < std::tie(o.inverse, o.log_n, o.n_layers);
  }
};
std::mutex g_plan_mutex;
std::map<PlanKey, std::vector<uint32_t>> g_plans;

constexpr uint32_t kMaxContiguousPass = 12, kMaxStridedPass = 11, kStridedC = 3;

// Splits layers [0, n_layers) of a column of log size log_n into passes of at
// most 12 layers (11 for strided passes); the first pass is contiguous.
std::vector<PassPlan> plan_passes(bool inverse, uint32_t log_n, uint32_t n_layers) {
  std::vector<PassPlan> plan;
  std::vector<uint32_t> sizes;
  {
    std::lock_guard<std::mutex> lock(g_plan_mutex);
    auto it = g_plans.find(PlanKey{inverse ? 1u : 0u, log_n, n_layers});
    if (it != g_plans.end()) sizes = it->second;
  }
  if (sizes.empty()) {
    uint32_t n_pass = 1;
    while (n_layers > kMaxContiguousPass + (n_pass - 1) * kMaxStridedPass) n_pass++;
    sizes.resize(n_pass);
    const uint32_t base = n_layers / n_pass, extra = n_layers % n_pass;
    // the contiguous first pass takes the remainder, so strided passes stay <= 11
    for (uint32_t i = 0; i < n_pass; i++) sizes[i] = base + (i < extra ? 1 : 0);
    // two passes of 17-20 layers: a 10-layer first pass (tiles of up to 10 layers run four blocks
    // per SM); measured 7-11% faster than (9, 9) at 18 layers, equal elsewhere in the range
    if (n_pass == 2 && n_layers >= 17 && n_layers <= 20) sizes = {10, n_layers - 10};
  }
  const uint32_t n_pass = (uint32_t)sizes.size();
  uint32_t lo = 0;
  for (uint32_t i = 0; i < n_pass; i++) {
    PassPlan pp;
    pp.lo = lo;
    pp.hi = lo + sizes[i];
    const uint32_t TA = sizes[i] / 2;
    if (lo == 0) {
      pp.outer = 1;  // contiguous tile, widened by outer groups to about 256 threads
      const uint32_t want = TA >= 8 ? 0 : 8 - TA;
      pp.c = std::min(want, log_n - pp.hi);
    } else {
      pp.outer = 0;  // strided tile: 8 neighbouring groups (32-byte runs in HBM)
      pp.c = kStridedC;
    }
    plan.push_back(pp);
    lo = pp.hi;
  }
  return plan;
}

template <bool INV, int T, bool OUTER>
cs_status launch_tile(const FftBatch& b, uint32_t n_cols, const FftPass& p, cudaStream_t st) {
  const size_t smem = (size_t)4 * padded_words<OUTER>(1u << (T + p.c));
  // the shared-memory limit is a per-device attribute of the kernel: raised once per device,
  // under a lock (several prover threads may launch the first FFT of a device at once)
  static std::mutex mu;
  static bool configured[kMaxDevices] = {false};
  int dev = 0;
  CS_CUDA(cudaGetDevice(&dev));
  CS_CHECK_ARG(dev >= 0 && dev < kMaxDevices, "fft: device ordinal %d out of range", dev);
  {
    std::lock_guard<std::mutex> lock(mu);
    if (!configured[dev]) {
      CS_CUDA(cudaFuncSetAttribute(fft_tile_kernel<INV, T, OUTER>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   160 * 1024));
      configured[dev] = true;
    }
  }
  const uint32_t threads = (1u << (T / 2)) << p.c;
  const uint32_t tiles = 1u << (p.log_n - T - p.c);
  dim3 grid(tiles, n_cols);
  fft_tile_kernel<INV, T, OUTER><<<grid, threads, smem, st>>>(b, p);
  CS_LAUNCHED("fft_tile_kernel");
  return CS_OK;
}

template <bool INV, bool OUTER>
cs_status dispatch_tile(const FftBatch& b, uint32_t n_cols, const FftPass& p, cudaStream_t st) {
  switch (p.hi - p.lo) {
    case 1: return launch_tile<INV, 1, OUTER>(b, n_cols, p, st);
    case 2: return launch_tile<INV, 2, OUTER>(b, n_cols, p, st);
    case 3: return launch_tile<INV, 3, OUTER>(b, n_cols, p, st);
    case 4: return launch_tile<INV, 4, OUTER>(b, n_cols, p, st);
    case 5: return launch_tile<INV, 5, OUTER>(b, n_cols, p, st);
    case 6: return launch_tile<INV, 6, OUTER>(b, n_cols, p, st);
    case 7: return launch_tile<INV, 7, OUTER>(b, n_cols, p, st);
    case 8: return launch_tile<INV, 8, OUTER>(b, n_cols, p, st);
    case 9: return launch_tile<INV, 9, OUTER>(b, n_cols, p, st);
    case 10: return launch_tile<INV, 10, OUTER>(b, n_cols, p, st);
    case 11: return launch_tile<INV, 11, OUTER>(b, n_cols, p, st);
    case 12:
      // plan_passes keeps strided passes at 11 layers or fewer
      if constexpr (OUTER) return launch_tile<INV, 12, OUTER>(b, n_cols, p, st);
      [[fallthrough]];
    default:
      set_error("fft: unsupported pass of %u layers", p.hi - p.lo);
      return CS_ERR_INVALID_ARG;
  }
}

// Constant columns (no layers): every output word is the single coefficient.
__global__ void replicate_kernel(const FftBatch batch, uint32_t log_n) {
  const uint32_t n = 1u << log_n;
  const uint32_t v = batch.src[blockIdx.y][0];
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    batch.dst[blockIdx.y][i] = v;
}

cs_status dispatch_copy(const FftBatch& b, uint32_t n_cols, const FftPass& p, cudaStream_t st) {
  const uint32_t n = 1u << p.log_n;
  dim3 grid(std::min<uint32_t>((n + 255) / 256, 64), n_cols);
  replicate_kernel<<<grid, 256, 0, st>>>(b, p.log_n);
  CS_LAUNCHED("replicate_kernel");
  return CS_OK;
}

template <bool INV>
cs_status launch_pass(const FftBatch& b, uint32_t n_cols, const FftPass& p_in, cudaStream_t st) {
  if (p_in.hi == p_in.lo) {
    // zero layers: a copy (replication of a constant column)
    return dispatch_copy(b, n_cols, p_in, st);
  }
  FftPass p = p_in;
  p.vec = p.src_mask >= 3;  // replicated reads of fewer than 4 coefficients break the runs of 4
  for (uint32_t i = 0; i < n_cols && p.vec; i++)
    p.vec = ((reinterpret_cast<uintptr_t>(b.src[i]) | reinterpret_cast<uintptr_t>(b.dst[i])) & 15) == 0;
  return p.outer ? dispatch_tile<INV, true>(b, n_cols, p, st) : dispatch_tile<INV, false>(b, n_cols, p, st);
}

// Runs the FFT over a batch of columns. inverse: interpolate in place
// (src == dst); forward: evaluate from coefficients of log_src into dst of log_n.
cs_status run_fft(const uint32_t* const* srcs, uint32_t* const* dsts, uint32_t n_cols, uint32_t log_src,
                  uint32_t log_n, bool inverse, const uint32_t* tw, uint32_t tw_log, cudaStream_t st,
                  uint32_t tw_dom = 0) {
  if (tw_dom == 0) tw_dom = log_n;
  // twiddle runs are read as 16-byte vectors
  CS_CHECK_ARG(log_n <= 2 || (reinterpret_cast<uintptr_t>(tw) & 15) == 0, "fft: twiddle buffer not 16-byte aligned");
  for (uint32_t b0 = 0; b0 < n_cols; b0 += kMaxBatch) {
    const uint32_t nb = std::min<uint32_t>(kMaxBatch, n_cols - b0);
    FftBatch batch;
    for (uint32_t i = 0; i < nb; i++) {
      batch.src[i] = srcs[b0 + i];
      batch.dst[i] = dsts[b0 + i];
    }
    if (log_n <= 2) {
      SmallParams sp = small_constants(log_n, log_src, inverse, tw_dom);
      fft_small_kernel<<<(nb + 127) / 128, 128, 0, st>>>(batch, nb, sp);
      CS_LAUNCHED("fft_small_kernel");
      continue;
    }
    const uint32_t n_layers = inverse ? log_n : log_src;
    std::vector<PassPlan> plan = plan_passes(inverse, log_n, n_layers);
    FftPass p{};
    p.log_n = log_n;
    p.tw = tw;
    p.tw_log = tw_log;
    p.tw_dom = tw_dom;
    if (inverse) {
      for (size_t k = 0; k < plan.size(); k++) {
        const PassPlan& pp = plan[k];
        p.lo = pp.lo; p.hi = pp.hi; p.c = pp.c; p.outer = pp.outer;
        p.src_mask = 0xffffffffu;
        // 1/n = 2^(31 - n) in M31 since 2^31 = 1
        p.scale = (k + 1 == plan.size()) ? (1u << (31 - log_n)) : 0;
        cs_status s = launch_pass<true>(batch, nb, p, st);
        if (s != CS_OK) return s;
        // the first pass may read a separate source; later passes work in place
        for (uint32_t i = 0; i < nb; i++) batch.src[i] = batch.dst[i];
      }
    } else {
      if (log_src == 0) {
        // constant polynomial: every evaluation is the constant coefficient
        p.lo = 0; p.hi = 0; p.c = 0; p.outer = 1;
        p.src_mask = 0;
        p.scale = 0;
        cs_status s = launch_pass<false>(batch, nb, p, st);
        if (s != CS_OK) return s;
        continue;
      }
      for (size_t k = plan.size(); k-- > 0;) {
        const PassPlan& pp = plan[k];
        p.lo = pp.lo; p.hi = pp.hi; p.c = pp.c; p.outer = pp.outer;
        p.scale = 0;
        if (k + 1 == plan.size()) {
          p.src_mask = (1u << log_src) - 1;
          FftBatch first = batch;
          cs_status s = launch_pass<false>(first, nb, p, st);
          if (s != CS_OK) return s;
          for (uint32_t i = 0; i < nb; i++) batch.src[i] = batch.dst[i];
        } else {
          p.src_mask = 0xffffffffu;
          cs_status s = launch_pass<false>(batch, nb, p, st);
          if (s != CS_OK) return s;
        }
      }
    }
  }
  return CS_OK;
}

// Side streams for the size groups of a mixed batch, per thread and device, created on first use
// (one set per calling thread, so concurrent provers never share them).
constexpr int kSideStreams = 4;
cs_status side_streams(cudaStream_t* out) {
  struct Pool {
    int dev = -1;
    cudaStream_t s[kSideStreams] = {};
    cudaEvent_t fork = nullptr, join[kSideStreams] = {};
  };
  static thread_local std::vector<Pool> pools;
  int dev = 0;
  CS_CUDA(cudaGetDevice(&dev));
  for (Pool& p : pools)
    if (p.dev == dev) {
      for (int i = 0; i < kSideStreams; i++) out[i] = p.s[i];
      return CS_OK;
    }
  Pool p;
  p.dev = dev;
  for (int i = 0; i < kSideStreams; i++) CS_CUDA(cudaStreamCreateWithFlags(&p.s[i], cudaStreamNonBlocking));
  pools.push_back(p);
  for (int i = 0; i < kSideStreams; i++) out[i] = p.s[i];
  return CS_OK;
}

// The FFT of a batch of columns of different sizes (PolyOps::interpolate_columns /
// evaluate_polynomials over a mixed batch): one batched launch sequence per size, the size groups
// spread over side streams forked from and joined back into `st` with events, so the small sizes'
// launches run beside the large ones instead of after them. Graph capture follows the fork and join.
// inverse: log_srcs[i] == log_ns[i]; forward: coefficients of log_srcs[i] evaluated on log_ns[i].
cs_status run_fft_mixed(const uint32_t* const* srcs, uint32_t* const* dsts, const uint32_t* log_srcs,
                        const uint32_t* log_ns, uint32_t n_cols, bool inverse, const uint32_t* tw, uint32_t tw_log,
                        cudaStream_t st) {
  // size groups, largest first (they take longest, so they start first)
  std::map<std::pair<uint32_t, uint32_t>, std::vector<uint32_t>, std::greater<>> groups;
  for (uint32_t i = 0; i < n_cols; i++) groups[{log_ns[i], log_srcs[i]}].push_back(i);
  if (groups.size() <= 1) {
    if (groups.empty()) return CS_OK;
    const auto& [key, idx] = *groups.begin();
    std::vector<const uint32_t*> s(idx.size());
    std::vector<uint32_t*> d(idx.size());
    for (size_t k = 0; k < idx.size(); k++) {
      s[k] = srcs[idx[k]];
      d[k] = dsts[idx[k]];
    }
    return run_fft(s.data(), d.data(), (uint32_t)idx.size(), key.second, key.first, inverse, tw, tw_log, st);
  }
  cudaStream_t side[kSideStreams];
  cs_status r = side_streams(side);
  if (r != CS_OK) return r;
  cudaEvent_t fork, join[kSideStreams];
  CS_CUDA(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
  for (int i = 0; i < kSideStreams; i++) CS_CUDA(cudaEventCreateWithFlags(&join[i], cudaEventDisableTiming));
  CS_CUDA(cudaEventRecord(fork, st));
  const int used = std::min<int>(kSideStreams, (int)groups.size());
  for (int i = 0; i < used; i++) CS_CUDA(cudaStreamWaitEvent(side[i], fork, 0));
  int g = 0;
  for (const auto& [key, idx] : groups) {
    std::vector<const uint32_t*> s(idx.size());
    std::vector<uint32_t*> d(idx.size());
    for (size_t k = 0; k < idx.size(); k++) {
      s[k] = srcs[idx[k]];
      d[k] = dsts[idx[k]];
    }
    r = run_fft(s.data(), d.data(), (uint32_t)idx.size(), key.second, key.first, inverse, tw, tw_log,
                side[g % used]);
    if (r != CS_OK) break;
    g++;
  }
  for (int i = 0; i < used; i++) {
    cudaEventRecord(join[i], side[i]);
    cudaStreamWaitEvent(st, join[i], 0);
  }
  cudaEventDestroy(fork);
  for (int i = 0; i < kSideStreams; i++) cudaEventDestroy(join[i]);
  return r;
}

}  // namespace

}  // namespace cs

using namespace cs;

extern "C" cs_status cs_interpolate_columns(uint32_t* const* h_cols, uint32_t n_cols, uint32_t log_size,
                                            const uint32_t* d_itwiddles, uint32_t twiddle_log_size,
                                            cs_stream stream) {
  CS_CHECK_ARG(n_cols == 0 || h_cols != nullptr, "interpolate: null column table");
  CS_CHECK_ARG(log_size >= 1 && log_size <= 28, "interpolate: log_size %u out of range [1, 28]", log_size);
  CS_CHECK_ARG(log_size <= 2 || (d_itwiddles != nullptr && twiddle_log_size + 1 >= log_size),
               "interpolate: twiddle tree of log %u does not cover a domain of log %u", twiddle_log_size, log_size);
  for (uint32_t i = 0; i < n_cols; i++) CS_CHECK_ARG(h_cols[i] != nullptr, "interpolate: column %u is null", i);
  return run_fft(h_cols, h_cols, n_cols, log_size, log_size, true, d_itwiddles, twiddle_log_size,
                 to_stream(stream));
}

extern "C" cs_status cs_interpolate_columns_into(const uint32_t* const* h_evals, uint32_t* const* h_coeffs,
                                                 uint32_t n_cols, uint32_t log_size, const uint32_t* d_itwiddles,
                                                 uint32_t twiddle_log_size, cs_stream stream) {
  CS_CHECK_ARG(n_cols == 0 || (h_evals != nullptr && h_coeffs != nullptr), "interpolate_into: null column table");
  CS_CHECK_ARG(log_size >= 1 && log_size <= 28, "interpolate_into: log_size %u out of range [1, 28]", log_size);
  CS_CHECK_ARG(log_size <= 2 || (d_itwiddles != nullptr && twiddle_log_size + 1 >= log_size),
               "interpolate_into: twiddle tree of log %u does not cover a domain of log %u", twiddle_log_size,
               log_size);
  for (uint32_t i = 0; i < n_cols; i++)
    CS_CHECK_ARG(h_evals[i] != nullptr && h_coeffs[i] != nullptr, "interpolate_into: column %u is null", i);
  return run_fft(h_evals, h_coeffs, n_cols, log_size, log_size, true, d_itwiddles, twiddle_log_size,
                 to_stream(stream));
}

extern "C" cs_status cs_interpolate_columns_on_subdomain(uint32_t* const* h_cols, uint32_t n_cols, uint32_t log_size,
                                                         uint32_t domain_log_size, const uint32_t* d_itwiddles,
                                                         uint32_t twiddle_log_size, cs_stream stream) {
  CS_CHECK_ARG(n_cols == 0 || h_cols != nullptr, "interpolate_on_subdomain: null column table");
  CS_CHECK_ARG(log_size >= 1 && log_size <= domain_log_size && domain_log_size <= 28,
               "interpolate_on_subdomain: bad sizes %u / %u", log_size, domain_log_size);
  CS_CHECK_ARG(log_size <= 2 || (d_itwiddles != nullptr && twiddle_log_size + 1 >= domain_log_size),
               "interpolate_on_subdomain: twiddle tree of log %u does not cover a domain of log %u",
               twiddle_log_size, domain_log_size);
  for (uint32_t i = 0; i < n_cols; i++)
    CS_CHECK_ARG(h_cols[i] != nullptr, "interpolate_on_subdomain: column %u is null", i);
  return run_fft(h_cols, h_cols, n_cols, log_size, log_size, true, d_itwiddles, twiddle_log_size,
                 to_stream(stream), domain_log_size);
}

extern "C" cs_status cs_evaluate_columns(const uint32_t* const* h_coeffs, uint32_t* const* h_evals, uint32_t n_cols,
                                         uint32_t log_coeffs, uint32_t log_size, const uint32_t* d_twiddles,
                                         uint32_t twiddle_log_size, cs_stream stream) {
  CS_CHECK_ARG(n_cols == 0 || (h_coeffs != nullptr && h_evals != nullptr), "evaluate: null column table");
  CS_CHECK_ARG(log_size >= 1 && log_size <= 28, "evaluate: log_size %u out of range [1, 28]", log_size);
  CS_CHECK_ARG(log_coeffs <= log_size, "evaluate: log_coeffs %u > log_size %u", log_coeffs, log_size);
  CS_CHECK_ARG(log_size <= 2 || (d_twiddles != nullptr && twiddle_log_size + 1 >= log_size),
               "evaluate: twiddle tree of log %u does not cover a domain of log %u", twiddle_log_size, log_size);
  for (uint32_t i = 0; i < n_cols; i++) {
    CS_CHECK_ARG(h_coeffs[i] != nullptr && h_evals[i] != nullptr, "evaluate: column %u is null", i);
    CS_CHECK_ARG((const void*)h_coeffs[i] != (const void*)h_evals[i], "evaluate: column %u aliases its output", i);
  }
  return run_fft(h_coeffs, h_evals, n_cols, log_coeffs, log_size, false, d_twiddles, twiddle_log_size,
                 to_stream(stream));
}

extern "C" cs_status cs_interpolate_columns_multi(const uint32_t* const* h_evals, uint32_t* const* h_coeffs,
                                                  const uint32_t* h_log_sizes, uint32_t n_cols,
                                                  const uint32_t* d_itwiddles, uint32_t twiddle_log_size,
                                                  cs_stream stream) {
  CS_CHECK_ARG(n_cols == 0 || (h_evals != nullptr && h_coeffs != nullptr && h_log_sizes != nullptr),
               "interpolate_multi: null table");
  for (uint32_t i = 0; i < n_cols; i++) {
    CS_CHECK_ARG(h_evals[i] != nullptr && h_coeffs[i] != nullptr, "interpolate_multi: column %u is null", i);
    CS_CHECK_ARG(h_log_sizes[i] >= 1 && h_log_sizes[i] <= 28, "interpolate_multi: column %u of log size %u", i,
                 h_log_sizes[i]);
    CS_CHECK_ARG(h_log_sizes[i] <= 2 || (d_itwiddles != nullptr && twiddle_log_size + 1 >= h_log_sizes[i]),
                 "interpolate_multi: twiddle tree of log %u does not cover a domain of log %u", twiddle_log_size,
                 h_log_sizes[i]);
  }
  return run_fft_mixed(h_evals, h_coeffs, h_log_sizes, h_log_sizes, n_cols, true, d_itwiddles, twiddle_log_size,
                       to_stream(stream));
}

extern "C" cs_status cs_evaluate_columns_multi(const uint32_t* const* h_coeffs, uint32_t* const* h_evals,
                                               const uint32_t* h_log_coeffs, uint32_t log_blowup, uint32_t n_cols,
                                               const uint32_t* d_twiddles, uint32_t twiddle_log_size,
                                               cs_stream stream) {
  CS_CHECK_ARG(n_cols == 0 || (h_coeffs != nullptr && h_evals != nullptr && h_log_coeffs != nullptr),
               "evaluate_multi: null table");
  CS_CHECK_ARG(log_blowup <= 8, "evaluate_multi: log_blowup %u", log_blowup);
  std::vector<uint32_t> log_ns(n_cols);
  for (uint32_t i = 0; i < n_cols; i++) {
    CS_CHECK_ARG(h_coeffs[i] != nullptr && h_evals[i] != nullptr, "evaluate_multi: column %u is null", i);
    CS_CHECK_ARG((const void*)h_coeffs[i] != (const void*)h_evals[i], "evaluate_multi: column %u aliases its output",
                 i);
    log_ns[i] = h_log_coeffs[i] + log_blowup;
    CS_CHECK_ARG(log_ns[i] >= 1 && log_ns[i] <= 28, "evaluate_multi: column %u of log size %u", i, log_ns[i]);
    CS_CHECK_ARG(log_ns[i] <= 2 || (d_twiddles != nullptr && twiddle_log_size + 1 >= log_ns[i]),
                 "evaluate_multi: twiddle tree of log %u does not cover a domain of log %u", twiddle_log_size,
                 log_ns[i]);
  }
  return run_fft_mixed(h_coeffs, h_evals, h_log_coeffs, log_ns.data(), n_cols, false, d_twiddles, twiddle_log_size,
                       to_stream(stream));
}

extern "C" cs_status cs_fft_set_plan(uint32_t inverse, uint32_t log_n, uint32_t n_layers, const uint32_t* pass_layers,
                                     uint32_t n_passes) {
  CS_CHECK_ARG(log_n >= 3 && log_n <= 30 && n_layers >= 1 && n_layers <= log_n, "fft_set_plan: bad shape %u/%u",
               log_n, n_layers);
  const PlanKey key{inverse ? 1u : 0u, log_n, n_layers};
  if (n_passes == 0) {
    std::lock_guard<std::mutex> lock(g_plan_mutex);
    g_plans.erase(key);
    return CS_OK;
  }
  CS_CHECK_ARG(pass_layers != nullptr && n_passes <= 32, "fft_set_plan: bad pass list");
  uint32_t total = 0;
  for (uint32_t i = 0; i < n_passes; i++) {
    const uint32_t t = pass_layers[i];
    CS_CHECK_ARG(t >= 1 && t <= (i == 0 ? kMaxContiguousPass : kMaxStridedPass),
                 "fft_set_plan: pass %u has %u layers", i, t);
    total += t;
  }
  CS_CHECK_ARG(total == n_layers, "fft_set_plan: passes cover %u of %u layers", total, n_layers);
  // a strided pass keeps kStridedC low index bits in its tile, so it must start at layer >= kStridedC
  CS_CHECK_ARG(n_passes == 1 || pass_layers[0] >= kStridedC, "fft_set_plan: first pass below %u layers",
               kStridedC);
  std::lock_guard<std::mutex> lock(g_plan_mutex);
  g_plans[key] = std::vector<uint32_t>(pass_layers, pass_layers + n_passes);
  return CS_OK;
}

extern "C" cs_status cs_fft_get_plan(uint32_t inverse, uint32_t log_n, uint32_t n_layers, uint32_t* pass_layers,
                                     uint32_t* n_passes) {
  CS_CHECK_ARG(pass_layers != nullptr && n_passes != nullptr, "fft_get_plan: null output");
  CS_CHECK_ARG(log_n >= 3 && log_n <= 30 && n_layers >= 1 && n_layers <= log_n, "fft_get_plan: bad shape");
  const std::vector<PassPlan> plan = plan_passes(inverse != 0, log_n, n_layers);
  *n_passes = (uint32_t)plan.size();
  for (size_t i = 0; i < plan.size() && i < 32; i++) pass_layers[i] = plan[i].hi - plan[i].lo;
  return CS_OK;
}
