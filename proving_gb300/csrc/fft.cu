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
#include <vector>

#include "common.cuh"
#include "field.cuh"

namespace cs {

namespace {

constexpr int kFftThreads = 256;

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
};

__device__ __forceinline__ uint32_t twiddle_at(const FftPass& p, uint32_t layer, uint32_t h) {
  const uint32_t tw_len = 1u << p.tw_log;
  if (layer == 0) {
    const uint32_t* lt1 = p.tw + (tw_len - (1u << (p.tw_dom - 1)));
    const uint32_t pair = (h >> 2) << 1;
    const uint32_t x = __ldg(lt1 + pair), y = __ldg(lt1 + pair + 1);
    switch (h & 3) {
      case 0: return y;
      case 1: return m31_neg(y);
      case 2: return m31_neg(x);
      default: return x;
    }
  }
  return __ldg(p.tw + (tw_len - (1u << (p.tw_dom - layer))) + h);
}

struct Tile {
  uint32_t o, ib;  // outer group and inner block (inner case) / first outer group (outer case)
};

__device__ __forceinline__ uint32_t tile_gidx(const FftPass& p, const Tile& t, uint32_t m, uint32_t e) {
  if (p.outer) return ((t.o + e) << p.hi) | m;
  return (t.o << p.hi) | (m << p.lo) | (t.ib << p.c) | e;
}

__device__ __forceinline__ uint32_t tile_sidx(const FftPass& p, uint32_t m, uint32_t e) {
  const uint32_t T = p.hi - p.lo;
  return p.outer ? (e << T) | m : (m << p.c) | e;
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

// One register stage: R consecutive local layers [d0, d0 + R) on groups of 2^R elements.
template <int R, bool INV>
__device__ __forceinline__ void run_stage(const FftPass& p, const Tile& t, uint32_t* s, uint32_t d0) {
  const uint32_t T = p.hi - p.lo;
  const uint32_t E = 1u << p.c;
  const uint32_t W = (1u << (T - R)) << p.c;
  for (uint32_t w = threadIdx.x; w < W; w += blockDim.x) {
    uint32_t e, mb;
    if (p.outer) {
      mb = w & ((1u << (T - R)) - 1);
      e = w >> (T - R);
    } else {
      e = w & (E - 1);
      mb = w >> p.c;
    }
    const uint32_t m0 = (mb & ((1u << d0) - 1)) | ((mb >> d0) << (d0 + R));
    uint32_t v[1 << R];
#pragma unroll
    for (int k = 0; k < (1 << R); k++) v[k] = s[tile_sidx(p, m0 + ((uint32_t)k << d0), e)];
    const uint32_t g0 = tile_gidx(p, t, m0, e);
    const uint32_t gstep = d0 + p.lo;
#pragma unroll
    for (int tt = 0; tt < R; tt++) {
      const int lt = INV ? tt : (R - 1 - tt);
      const uint32_t layer = p.lo + d0 + (uint32_t)lt;
#pragma unroll
      for (int k = 0; k < (1 << R); k++) {
        if (k & (1 << lt)) continue;
        const uint32_t g = g0 + ((uint32_t)k << gstep);
        const uint32_t tw = twiddle_at(p, layer, g >> (layer + 1));
        if (INV)
          ibfly(v[k], v[k | (1 << lt)], tw);
        else
          bfly(v[k], v[k | (1 << lt)], tw);
      }
    }
#pragma unroll
    for (int k = 0; k < (1 << R); k++) s[tile_sidx(p, m0 + ((uint32_t)k << d0), e)] = v[k];
  }
}

template <bool INV>
__global__ void __launch_bounds__(kFftThreads) fft_pass_kernel(const FftBatch batch, const FftPass p) {
  extern __shared__ uint32_t s[];
  const uint32_t T = p.hi - p.lo;
  const uint32_t N = 1u << (T + p.c);
  uint32_t* dst = batch.dst[blockIdx.y];
  const uint32_t* src = batch.src[blockIdx.y];
  Tile t;
  if (p.outer) {
    t.o = blockIdx.x << p.c;
    t.ib = 0;
  } else {
    const uint32_t outer_bits = p.log_n - p.hi;
    t.o = blockIdx.x & ((1u << outer_bits) - 1);
    t.ib = blockIdx.x >> outer_bits;
  }
  for (uint32_t L = threadIdx.x; L < N; L += blockDim.x) {
    uint32_t m, e;
    if (p.outer) {
      m = L & ((1u << T) - 1);
      e = L >> T;
    } else {
      e = L & ((1u << p.c) - 1);
      m = L >> p.c;
    }
    s[L] = __ldg(src + (tile_gidx(p, t, m, e) & p.src_mask));
  }
  __syncthreads();
  if (INV) {
    uint32_t d = 0;
    while (d < T) {
      const uint32_t r = min(3u, T - d);
      if (r == 3) run_stage<3, INV>(p, t, s, d);
      else if (r == 2) run_stage<2, INV>(p, t, s, d);
      else run_stage<1, INV>(p, t, s, d);
      d += r;
      __syncthreads();
    }
  } else {
    uint32_t d = T;
    while (d > 0) {
      const uint32_t r = min(3u, d);
      d -= r;
      if (r == 3) run_stage<3, INV>(p, t, s, d);
      else if (r == 2) run_stage<2, INV>(p, t, s, d);
      else run_stage<1, INV>(p, t, s, d);
      __syncthreads();
    }
  }
  for (uint32_t L = threadIdx.x; L < N; L += blockDim.x) {
    uint32_t m, e;
    if (p.outer) {
      m = L & ((1u << T) - 1);
      e = L >> T;
    } else {
      e = L & ((1u << p.c) - 1);
      m = L >> p.c;
    }
    uint32_t v = s[L];
    if (p.scale) v = m31_mul(v, p.scale);
    dst[tile_gidx(p, t, m, e)] = v;
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
  uint32_t lo, hi, c, outer;
};

// Splits layers [0, n_layers) of a column of log size log_n into passes.
std::vector<PassPlan> plan_passes(uint32_t log_n, uint32_t n_layers) {
  std::vector<PassPlan> plan;
  const uint32_t max_first = 12, max_strided = 11;
  uint32_t n_pass = 1;
  while (true) {
    // first pass gets the remainder, strided passes are balanced
    if (n_layers <= max_first + (n_pass - 1) * max_strided) break;
    n_pass++;
  }
  std::vector<uint32_t> sizes(n_pass);
  uint32_t base = n_layers / n_pass, extra = n_layers % n_pass;
  for (uint32_t i = 0; i < n_pass; i++) sizes[i] = base + (i < extra ? 1 : 0);
  uint32_t lo = 0;
  for (uint32_t i = 0; i < n_pass; i++) {
    PassPlan pp;
    pp.lo = lo;
    pp.hi = lo + sizes[i];
    if (lo == 0) {
      // contiguous tile: 2^T elements, widened by outer groups up to 2^11 words
      pp.outer = 1;
      const uint32_t want = sizes[i] >= 11 ? 0 : 11 - sizes[i];
      pp.c = std::min(want, log_n - pp.hi);
    } else {
      pp.outer = 0;
      pp.c = std::min(3u, lo);
    }
    plan.push_back(pp);
    lo = pp.hi;
  }
  return plan;
}

size_t pass_smem(const PassPlan& pp) { return (size_t)4 << (pp.hi - pp.lo + pp.c); }

template <bool INV>
cs_status launch_pass(const FftBatch& b, uint32_t n_cols, const FftPass& p, const PassPlan& pp,
                      cudaStream_t st) {
  const size_t smem = pass_smem(pp);
  static bool configured = false;
  if (!configured) {
    CS_CUDA(cudaFuncSetAttribute(fft_pass_kernel<INV>, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024));
    configured = true;
  }
  const uint32_t T = pp.hi - pp.lo;
  const uint32_t tiles = 1u << (p.log_n - T - pp.c);
  dim3 grid(tiles, n_cols);
  fft_pass_kernel<INV><<<grid, kFftThreads, smem, st>>>(b, p);
  CS_LAUNCHED("fft_pass_kernel");
  return CS_OK;
}

// Runs the FFT over a batch of columns. inverse: interpolate in place
// (src == dst); forward: evaluate from coefficients of log_src into dst of log_n.
cs_status run_fft(const uint32_t* const* srcs, uint32_t* const* dsts, uint32_t n_cols, uint32_t log_src,
                  uint32_t log_n, bool inverse, const uint32_t* tw, uint32_t tw_log, cudaStream_t st,
                  uint32_t tw_dom = 0) {
  if (tw_dom == 0) tw_dom = log_n;
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
    std::vector<PassPlan> plan = plan_passes(log_n, n_layers);
    FftPass p;
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
        cs_status s = launch_pass<true>(batch, nb, p, pp, st);
        if (s != CS_OK) return s;
        // the first pass may read a separate source; later passes work in place
        for (uint32_t i = 0; i < nb; i++) batch.src[i] = batch.dst[i];
      }
    } else {
      if (log_src == 0) {
        // constant polynomial: every evaluation is the constant; a pass over
        // zero layers would be empty, so replicate with a trivial 1-layer-free copy
        PassPlan pp{0, 0, std::min(11u, log_n), 1};
        p.lo = 0; p.hi = 0; p.c = pp.c; p.outer = 1;
        p.src_mask = 0;
        p.scale = 0;
        cs_status s = launch_pass<false>(batch, nb, p, pp, st);
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
          cs_status s = launch_pass<false>(first, nb, p, pp, st);
          if (s != CS_OK) return s;
          for (uint32_t i = 0; i < nb; i++) batch.src[i] = batch.dst[i];
        } else {
          p.src_mask = 0xffffffffu;
          cs_status s = launch_pass<false>(batch, nb, p, pp, st);
          if (s != CS_OK) return s;
        }
      }
    }
  }
  return CS_OK;
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
