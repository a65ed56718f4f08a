// The Poseidon2 AIR of crates/examples/src/poseidon/mod.rs on the device:
// trace generation (gen_trace, mod.rs:195-275), the LogUp interaction trace
// (gen_interaction_trace, mod.rs:277-303, with LogupTraceGenerator,
// crates/constraint-framework/src/prover/logup.rs:55-130) and the constraint
// quotients on an evaluation domain (the device analogue of
// FrameworkComponent::evaluate_constraint_quotients_on_domain,
// crates/constraint-framework/src/prover/component_prover.rs:195-268, for
// eval_poseidon_constraints, mod.rs:137-189).
//
// State width 16, 4 + 4 full rounds and 14 partial rounds, x^5, every round
// constant 1234; 8 instances per row of 158 columns (1264 columns). One
// thread per row in every kernel: a warp reads or writes 32 consecutive rows
// of a column (128 bytes) per access.
#include <algorithm>

#include "common.cuh"
#include "field.cuh"
#include "logup.cuh"
#include "rows.cuh"

namespace cs {

namespace {

constexpr int kState = 16;
constexpr int kPartial = 14;
constexpr int kHalfFull = 4;
constexpr int kInstances = 8;
constexpr int kColsPerRep = kState * (1 + 2 * kHalfFull) + kPartial;  // 158
constexpr int kCols = kInstances * kColsPerRep;                         // 1264
constexpr int kInterCols = 4 * kInstances;                              // 32
constexpr int kRoundConstraints = 2 * kHalfFull * kState + kPartial;    // 142 per instance
constexpr int kConstraints = kInstances * kRoundConstraints + kInstances;  // 1144
constexpr uint32_t kRoundConst = 1234;
constexpr uint32_t kMaxExpand = 5;

// apply_m4 (mod.rs:72-89)
__device__ __forceinline__ void m4(uint32_t* x) {
  const uint32_t t0 = m31_add(x[0], x[1]);
  const uint32_t t02 = m31_add(t0, t0);
  const uint32_t t1 = m31_add(x[2], x[3]);
  const uint32_t t12 = m31_add(t1, t1);
  const uint32_t t2 = m31_add(m31_add(x[1], x[1]), t1);
  const uint32_t t3 = m31_add(m31_add(x[3], x[3]), t0);
  const uint32_t t4 = m31_add(m31_add(t12, t12), t3);
  const uint32_t t5 = m31_add(m31_add(t02, t02), t2);
  x[0] = m31_add(t3, t5);
  x[1] = t5;
  x[2] = m31_add(t2, t4);
  x[3] = t4;
}

// apply_external_round_matrix (mod.rs:91-113): circ(2 M4, M4, M4, M4)
__device__ __forceinline__ void external_matrix(uint32_t* s) {
#pragma unroll
  for (int i = 0; i < 4; i++) m4(s + 4 * i);
#pragma unroll
  for (int j = 0; j < 4; j++) {
    const uint32_t t = m31_add(m31_add(s[j], s[j + 4]), m31_add(s[j + 8], s[j + 12]));
#pragma unroll
    for (int i = 0; i < 4; i++) s[4 * i + j] = m31_add(s[4 * i + j], t);
  }
}

// apply_internal_round_matrix (mod.rs:115-129): s_i <- s_i * 2^(i+1) + sum(s)
__device__ __forceinline__ void internal_matrix(uint32_t* s) {
  uint32_t sum = s[0];
#pragma unroll
  for (int i = 1; i < kState; i++) sum = m31_add(sum, s[i]);
#pragma unroll
  for (int i = 0; i < kState; i++) s[i] = m31_add(m31_mul(s[i], 1u << (i + 1)), sum);
}

__device__ __forceinline__ uint32_t pow5(uint32_t x) {
  const uint32_t x2 = m31_sqr(x);
  return m31_mul(m31_sqr(x2), x);
}

// ---------------------------------------------------------------- trace

struct TraceOut {
  uint32_t* cols[kCols];
};

// One block = 32 rows x the 8 instances: warp k computes instance k of 32 consecutive rows
// (lane = row) and writes its 158 columns, 128 bytes per column per warp.
__global__ void __launch_bounds__(256) poseidon_trace_kernel(uint32_t log_n, const __grid_constant__ TraceOut out) {
  const uint32_t n = 1u << log_n;
  const int k = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint32_t* const* cols = out.cols + k * kColsPerRep;
  for (uint32_t base = blockIdx.x * 32; base < n; base += gridDim.x * 32) {
    const uint32_t r = base + lane;
    if (r >= n) continue;
    uint32_t s[kState];
#pragma unroll
    for (int i = 0; i < kState; i++) {
      s[i] = r + i + k;  // gen_trace's input (mod.rs:215-219)
      cols[i][r] = s[i];
    }
    int c = kState;
#pragma unroll 1
    for (int round = 0; round < 2 * kHalfFull; round++) {
      if (round == kHalfFull) {
#pragma unroll 1
        for (int q = 0; q < kPartial; q++) {
          s[0] = m31_add(s[0], kRoundConst);
          internal_matrix(s);
          s[0] = pow5(s[0]);
          cols[c++][r] = s[0];
        }
      }
#pragma unroll
      for (int i = 0; i < kState; i++) s[i] = m31_add(s[i], kRoundConst);
      external_matrix(s);
#pragma unroll
      for (int i = 0; i < kState; i++) {
        s[i] = pow5(s[i]);
        cols[c + i][r] = s[i];
      }
      c += kState;
    }
  }
}

// ---------------------------------------------------------------- LogUp

// Reduces a sum of fewer than 2^32 canonical words.
__device__ __forceinline__ uint32_t fold64(uint64_t v) {
  const uint64_t t = (v & P) + (v >> 31);
  return m31_reduce_once((uint32_t)((t & P) + (t >> 31)));
}


struct Lookup {
  qm31 z;
  qm31 alpha_pow[kState];
};

// combine (crates/constraint-framework/src/logup.rs:80-93): sum_i alpha^i v_i - z
__device__ __forceinline__ qm31 combine(const Lookup& lk, const uint32_t* v) {
  uint64_t acc[4] = {0, 0, 0, 0};
#pragma unroll
  for (int i = 0; i < kState; i++) {
    acc[0] += m31_mul(lk.alpha_pow[i].a.a, v[i]);
    acc[1] += m31_mul(lk.alpha_pow[i].a.b, v[i]);
    acc[2] += m31_mul(lk.alpha_pow[i].b.a, v[i]);
    acc[3] += m31_mul(lk.alpha_pow[i].b.b, v[i]);
  }
  const qm31 sum = qm31_make(fold64(acc[0]), fold64(acc[1]), fold64(acc[2]), fold64(acc[3]));
  return qm31_sub(sum, lk.z);
}

struct InterParams {
  const uint32_t* trace[kCols];
  uint32_t* out[kInterCols];
  Lookup lk;
  uint32_t log_n;
};

// Row fractions 1/combine(initial) - 1/combine(final) per instance, summed along the row: QM31
// column k < 7 gets the sum over instances 0..k, column 7 the row total (finalized afterwards).
// One block = 32 rows x the 8 instances: warp k computes instance k's fraction, and the prefix
// over instances goes through shared memory.
__global__ void __launch_bounds__(256) poseidon_fractions_kernel(const __grid_constant__ InterParams p) {
  __shared__ uint32_t s_frac[kInstances][4][32];
  const uint32_t n = 1u << p.log_n;
  const int k = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (uint32_t base = blockIdx.x * 32; base < n; base += gridDim.x * 32) {
    const uint32_t r = base + lane;
    qm31 f = qm31_make(0, 0, 0, 0);
    if (r < n) {
      uint32_t v[kState];
#pragma unroll
      for (int i = 0; i < kState; i++) v[i] = __ldg(p.trace[k * kColsPerRep + i] + r);
      const qm31 d0 = combine(p.lk, v);
#pragma unroll
      for (int i = 0; i < kState; i++) v[i] = __ldg(p.trace[k * kColsPerRep + kColsPerRep - kState + i] + r);
      const qm31 d1 = combine(p.lk, v);
      f = qm31_mul(qm31_sub(d1, d0), qm31_inv(qm31_mul(d0, d1)));
    }
    s_frac[k][0][lane] = f.a.a;
    s_frac[k][1][lane] = f.a.b;
    s_frac[k][2][lane] = f.b.a;
    s_frac[k][3][lane] = f.b.b;
    __syncthreads();
    if (r < n) {
      qm31 acc = qm31_make(s_frac[0][0][lane], s_frac[0][1][lane], s_frac[0][2][lane], s_frac[0][3][lane]);
      for (int j = 1; j <= k; j++)
        acc = qm31_add(acc, qm31_make(s_frac[j][0][lane], s_frac[j][1][lane], s_frac[j][2][lane], s_frac[j][3][lane]));
      p.out[4 * k][r] = acc.a.a;
      p.out[4 * k + 1][r] = acc.a.b;
      p.out[4 * k + 2][r] = acc.b.a;
      p.out[4 * k + 3][r] = acc.b.b;
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------- constraint quotients

struct CompParams {
  const uint32_t* trace[kCols];
  const uint32_t* inter[kInterCols];
  Lookup lk;
  qm31 shift;  // claimed_sum / 2^trace_log
  uint32_t den[1u << kMaxExpand];
  uint32_t eval_log, trace_log;
};


__device__ __forceinline__ void add_base(uint64_t* acc, const uint4& w, uint32_t cons) {
  acc[0] += m31_mul(w.x, cons);
  acc[1] += m31_mul(w.y, cons);
  acc[2] += m31_mul(w.z, cons);
  acc[3] += m31_mul(w.w, cons);
}

// Lazy accumulation of weight x constraint products: each product is below 2^62 and is added
// unreduced (one 64-bit multiply-add per coordinate); fold_acc brings the sums back below 2^34,
// so three products may be added between folds without overflow.
__device__ __forceinline__ void add_base_lazy(uint64_t* acc, const uint4& w, uint32_t cons) {
  acc[0] += (uint64_t)w.x * cons;
  acc[1] += (uint64_t)w.y * cons;
  acc[2] += (uint64_t)w.z * cons;
  acc[3] += (uint64_t)w.w * cons;
}
__device__ __forceinline__ void fold_acc(uint64_t* acc) {
#pragma unroll
  for (int c = 0; c < 4; c++) acc[c] = (acc[c] & P) + (acc[c] >> 31);
}

__global__ void __launch_bounds__(128) poseidon_composition_kernel(const __grid_constant__ CompParams p,
                                                                    const uint4* __restrict__ rc, uint32_t* a0,
                                                                    uint32_t* a1, uint32_t* a2, uint32_t* a3) {
  // the 1144 random-coefficient powers (18 KB), read by every thread at the same index
  __shared__ uint4 s_rc[kConstraints];
  for (int i = threadIdx.x; i < kConstraints; i += blockDim.x) s_rc[i] = rc[i];
  __syncthreads();
  const uint32_t n = 1u << p.eval_log;
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    uint64_t acc[4] = {0, 0, 0, 0};
    qm31 lacc = qm31_make(0, 0, 0, 0);  // the LogUp constraints (QM31 values)
    const uint32_t pr = prev_row(r, p.trace_log, p.eval_log);
    qm31 prev_col = qm31_make(0, 0, 0, 0);
    uint32_t idx = 0;
#pragma unroll 1
    for (int k = 0; k < kInstances; k++) {
      const uint32_t* const* col = p.trace + k * kColsPerRep;
      uint32_t s[kState];
#pragma unroll
      for (int i = 0; i < kState; i++) s[i] = __ldg(col[i] + r);
      const qm31 d0 = combine(p.lk, s);
      int c = kState;
#pragma unroll 1
      for (int round = 0; round < 2 * kHalfFull; round++) {
        if (round == kHalfFull) {
#pragma unroll 1
          for (int q = 0; q < kPartial; q++) {
            s[0] = m31_add(s[0], kRoundConst);
            internal_matrix(s);
            const uint32_t m = __ldg(col[c++] + r);
            add_base(acc, s_rc[idx++], m31_sub(pow5(s[0]), m));
            s[0] = m;
          }
        }
#pragma unroll
        for (int i = 0; i < kState; i++) s[i] = m31_add(s[i], kRoundConst);
        external_matrix(s);
#pragma unroll
        for (int i = 0; i < kState; i++) {
          const uint32_t m = __ldg(col[c + i] + r);
          add_base(acc, s_rc[idx + i], m31_sub(pow5(s[i]), m));
          s[i] = m;
        }
        c += kState;
        idx += kState;
      }
      // LogUp batch k (finalize_logup_batched, crates/constraint-framework/src/lib.rs:185-222):
      // fraction (d1 - d0) / (d0 d1); columns k < 7 hold row prefixes, column 7 the running sum
      const qm31 d1 = combine(p.lk, s);
      const uint32_t* const* ic = p.inter + 4 * k;
      const qm31 cur = qm31_make(__ldg(ic[0] + r), __ldg(ic[1] + r), __ldg(ic[2] + r), __ldg(ic[3] + r));
      qm31 diff = qm31_sub(cur, prev_col);
      if (k == kInstances - 1) {
        const qm31 prev = qm31_make(__ldg(ic[0] + pr), __ldg(ic[1] + pr), __ldg(ic[2] + pr), __ldg(ic[3] + pr));
        diff = qm31_add(qm31_sub(diff, prev), p.shift);
      }
      prev_col = cur;
      const qm31 cons = qm31_sub(qm31_mul(diff, qm31_mul(d0, d1)), qm31_sub(d1, d0));
      const uint4 w = s_rc[kInstances * kRoundConstraints + k];
      lacc = qm31_add(lacc, qm31_mul(qm31_make(w.x, w.y, w.z, w.w), cons));
    }
    const uint32_t d = p.den[r >> p.trace_log];
    const qm31 row = qm31_add(qm31_make(fold64(acc[0]), fold64(acc[1]), fold64(acc[2]), fold64(acc[3])), lacc);
    a0[r] = m31_add(a0[r], m31_mul(row.a.a, d));
    a1[r] = m31_add(a1[r], m31_mul(row.a.b, d));
    a2[r] = m31_add(a2[r], m31_mul(row.b.a, d));
    a3[r] = m31_add(a3[r], m31_mul(row.b.b, d));
  }
}


// One block = 32 rows x the 8 instances: warp k evaluates instance k's 142 round constraints and
// its LogUp batch for 32 consecutive rows (lane = row), the eight partial sums meet in shared
// memory, and warp c < 4 adds coordinate c of the row sums times the denominator.
__global__ void __launch_bounds__(256, 3) poseidon_composition_split_kernel(
    const __grid_constant__ CompParams p, const uint4* __restrict__ rc, uint32_t* a0, uint32_t* a1, uint32_t* a2,
    uint32_t* a3) {
  __shared__ uint4 s_rc[kConstraints];
  __shared__ uint32_t s_part[kInstances][4][32];
  for (int i = threadIdx.x; i < kConstraints; i += blockDim.x) s_rc[i] = rc[i];
  __syncthreads();
  const int k = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t n = 1u << p.eval_log;
  uint32_t* const acc_out[4] = {a0, a1, a2, a3};
  for (uint32_t base = blockIdx.x * 32; base < n; base += gridDim.x * 32) {
    const uint32_t r = base + lane;
    uint64_t acc[4] = {0, 0, 0, 0};
    const uint32_t* const* col = p.trace + k * kColsPerRep;
    uint32_t s[kState];
#pragma unroll
    for (int i = 0; i < kState; i++) s[i] = __ldg(col[i] + r);
    const qm31 d0 = combine(p.lk, s);
    int c = kState;
    uint32_t idx = k * kRoundConstraints;
#pragma unroll 1
    for (int round = 0; round < 2 * kHalfFull; round++) {
      if (round == kHalfFull) {
#pragma unroll 1
        for (int q = 0; q < kPartial; q++) {
          s[0] = m31_add(s[0], kRoundConst);
          internal_matrix(s);
          const uint32_t m = __ldg(col[c++] + r);
          add_base_lazy(acc, s_rc[idx++], m31_sub(pow5(s[0]), m));
          fold_acc(acc);
          s[0] = m;
        }
      }
#pragma unroll
      for (int i = 0; i < kState; i++) s[i] = m31_add(s[i], kRoundConst);
      external_matrix(s);
#pragma unroll
      for (int i = 0; i < kState; i++) {
        const uint32_t m = __ldg(col[c + i] + r);
        add_base_lazy(acc, s_rc[idx + i], m31_sub(pow5(s[i]), m));
        if (i % 3 == 2 || i == kState - 1) fold_acc(acc);
        s[i] = m;
      }
      c += kState;
      idx += kState;
    }
    // LogUp batch k (finalize_logup_batched, crates/constraint-framework/src/lib.rs:185-222)
    const qm31 d1 = combine(p.lk, s);
    const uint32_t* const* ic = p.inter + 4 * k;
    const qm31 cur = qm31_make(__ldg(ic[0] + r), __ldg(ic[1] + r), __ldg(ic[2] + r), __ldg(ic[3] + r));
    qm31 diff = cur;
    if (k > 0) {
      const uint32_t* const* pc = ic - 4;
      diff = qm31_sub(diff, qm31_make(__ldg(pc[0] + r), __ldg(pc[1] + r), __ldg(pc[2] + r), __ldg(pc[3] + r)));
    }
    if (k == kInstances - 1) {
      const uint32_t pr = prev_row(r, p.trace_log, p.eval_log);
      const qm31 prev = qm31_make(__ldg(ic[0] + pr), __ldg(ic[1] + pr), __ldg(ic[2] + pr), __ldg(ic[3] + pr));
      diff = qm31_add(qm31_sub(diff, prev), p.shift);
    }
    const qm31 cons = qm31_sub(qm31_mul(diff, qm31_mul(d0, d1)), qm31_sub(d1, d0));
    const uint4 w = s_rc[kInstances * kRoundConstraints + k];
    const qm31 part = qm31_add(qm31_make(fold64(acc[0]), fold64(acc[1]), fold64(acc[2]), fold64(acc[3])),
                               qm31_mul(qm31_make(w.x, w.y, w.z, w.w), cons));
    s_part[k][0][lane] = part.a.a;
    s_part[k][1][lane] = part.a.b;
    s_part[k][2][lane] = part.b.a;
    s_part[k][3][lane] = part.b.b;
    __syncthreads();
    if (k < 4) {
      uint32_t v = s_part[0][k][lane];
#pragma unroll
      for (int j = 1; j < kInstances; j++) v = m31_add(v, s_part[j][k][lane]);
      acc_out[k][r] = m31_add(acc_out[k][r], m31_mul(v, p.den[r >> p.trace_log]));
    }
    __syncthreads();
  }
}

cpoint point_at_index(uint32_t idx) {
  cpoint r{1, 0}, cur{2u, 1268011823u};
  while (idx) {
    if (idx & 1) r = cpoint_add(r, cur);
    cur = cpoint_add(cur, cur);
    idx >>= 1;
  }
  return r;
}

void set_lookup(Lookup& lk, const uint32_t* w) {
  lk.z = qm31_make(w[0], w[1], w[2], w[3]);
  const qm31 alpha = qm31_make(w[4], w[5], w[6], w[7]);
  qm31 cur = qm31_make(1, 0, 0, 0);
  for (int i = 0; i < kState; i++) {
    lk.alpha_pow[i] = cur;
    cur = qm31_mul(cur, alpha);
  }
}

// Blocks of 32 rows x 8 instances for 2^log_n rows, at most 16 per SM (grid-stride beyond).
uint32_t row_group_blocks(uint32_t n) { return std::max(1u, std::min((n + 31) / 32, 152u * 16)); }

}  // namespace
}  // namespace cs

using namespace cs;

extern "C" cs_status cs_poseidon_trace(uint32_t log_n, uint32_t* const* h_cols, cs_stream stream) {
  CS_CHECK_ARG(h_cols != nullptr, "poseidon_trace: null column table");
  CS_CHECK_ARG(log_n >= 1 && log_n <= 26, "poseidon_trace: log size %u outside [1, 26]", log_n);
  static thread_local TraceOut out;
  for (int k = 0; k < kCols; k++) {
    CS_CHECK_ARG(h_cols[k] != nullptr, "poseidon_trace: column %d is null", k);
    out.cols[k] = h_cols[k];
  }
  const uint32_t n = 1u << log_n;
  poseidon_trace_kernel<<<row_group_blocks(n), 256, 0, to_stream(stream)>>>(log_n, out);
  CS_LAUNCHED("poseidon_trace_kernel");
  return CS_OK;
}

extern "C" cs_status cs_poseidon_interaction(const uint32_t* const* h_trace, uint32_t log_n, const uint32_t lookup[8],
                                             uint32_t* const* h_out, uint32_t claimed_sum_out[4], cs_stream stream) {
  CS_CHECK_ARG(h_trace != nullptr && lookup != nullptr && h_out != nullptr && claimed_sum_out != nullptr,
               "poseidon_interaction: null pointer");
  CS_CHECK_ARG(log_n >= 1 && log_n <= 26, "poseidon_interaction: log size %u outside [1, 26]", log_n);
  static thread_local InterParams p;
  for (int k = 0; k < kCols; k++) {
    CS_CHECK_ARG(h_trace[k] != nullptr, "poseidon_interaction: trace column %d is null", k);
    p.trace[k] = h_trace[k];
  }
  for (int k = 0; k < kInterCols; k++) {
    CS_CHECK_ARG(h_out[k] != nullptr, "poseidon_interaction: output column %d is null", k);
    p.out[k] = h_out[k];
  }
  set_lookup(p.lk, lookup);
  p.log_n = log_n;
  cudaStream_t st = to_stream(stream);
  const uint32_t n = 1u << log_n;
  poseidon_fractions_kernel<<<row_group_blocks(n), 256, 0, st>>>(p);
  CS_LAUNCHED("poseidon_fractions_kernel");
  Q4 last;
  for (int c = 0; c < 4; c++) last.c[c] = h_out[4 * (kInstances - 1) + c];
  return logup_finalize_last(last, log_n, claimed_sum_out, st);
}

extern "C" cs_status cs_poseidon_composition(const uint32_t* const* h_trace, const uint32_t* const* h_inter,
                                             uint32_t eval_log, uint32_t trace_log, const uint32_t lookup[8],
                                             const uint32_t claimed_sum[4], const uint32_t* h_rc,
                                             uint32_t* const h_accum[4], cs_stream stream) {
  CS_CHECK_ARG(h_trace != nullptr && h_inter != nullptr && lookup != nullptr && claimed_sum != nullptr &&
                   h_rc != nullptr && h_accum != nullptr,
               "poseidon_composition: null pointer");
  CS_CHECK_ARG(trace_log >= 1 && eval_log >= trace_log && eval_log - trace_log <= kMaxExpand && eval_log <= 28,
               "poseidon_composition: bad sizes eval %u trace %u", eval_log, trace_log);
  static thread_local CompParams p;
  for (int k = 0; k < kCols; k++) {
    CS_CHECK_ARG(h_trace[k] != nullptr, "poseidon_composition: trace column %d is null", k);
    p.trace[k] = h_trace[k];
  }
  for (int k = 0; k < kInterCols; k++) {
    CS_CHECK_ARG(h_inter[k] != nullptr, "poseidon_composition: interaction column %d is null", k);
    p.inter[k] = h_inter[k];
  }
  for (int c = 0; c < 4; c++) CS_CHECK_ARG(h_accum[c] != nullptr, "poseidon_composition: null accumulator");
  set_lookup(p.lk, lookup);
  // cumsum_shift = claimed_sum / 2^trace_log (LogupAtRow::new, crates/constraint-framework/src/logup.rs:32-40)
  p.shift = qm31_mul_m31(qm31_make(claimed_sum[0], claimed_sum[1], claimed_sum[2], claimed_sum[3]),
                         1u << (31 - trace_log));
  p.eval_log = eval_log;
  p.trace_log = trace_log;
  // denom_inv[i] = 1 / V_trace(eval_domain.at(i)), bit-reversed (component_prover.rs:101-108); on
  // the trace domain itself no denominator applies
  const uint32_t log_expand = eval_log - trace_log, n_den = 1u << log_expand;
  if (log_expand == 0) {
    p.den[0] = 1;
  } else {
    for (uint32_t i = 0; i < n_den; i++) {
      const uint32_t idx = (subgroup_gen(eval_log + 1) + i * subgroup_gen(eval_log - 1)) & 0x7fffffffu;
      uint32_t x = point_at_index(idx).x;
      for (uint32_t k = 1; k < trace_log; k++) x = m31_sub(m31_add(m31_sqr(x), m31_sqr(x)), 1);
      uint32_t j = 0;
      for (uint32_t b = 0; b < log_expand; b++) j |= ((i >> b) & 1u) << (log_expand - 1 - b);
      p.den[j] = m31_inv(x);
    }
  }
  cudaStream_t st = to_stream(stream);
  uint4* d_rc = nullptr;
  CS_CUDA(stream_alloc(reinterpret_cast<void**>(&d_rc), sizeof(uint4) * kConstraints, st));
  cudaError_t e = cudaMemcpyAsync(d_rc, h_rc, sizeof(uint4) * kConstraints, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    const uint32_t n = 1u << eval_log;
    if (n >= 32)
      poseidon_composition_split_kernel<<<std::min<uint32_t>(n / 32, 152u * 16), 256, 0, st>>>(
          p, d_rc, h_accum[0], h_accum[1], h_accum[2], h_accum[3]);
    else
      poseidon_composition_kernel<<<1, 128, 0, st>>>(p, d_rc, h_accum[0], h_accum[1], h_accum[2], h_accum[3]);
    note_launch();
    e = cudaGetLastError();
  }
  const cudaError_t ef = cudaFreeAsync(d_rc, st);
  if (e == cudaSuccess) e = ef;
  if (e != cudaSuccess) return from_cuda(e, "poseidon_composition");
  return CS_OK;
}
