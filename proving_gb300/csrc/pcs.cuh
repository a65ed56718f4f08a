// Parameter blocks of the accumulation / quotient / sampling kernels (pcs.cu).
#pragma once
#include <cstdint>

#include "common.cuh"
#include "field.cuh"

namespace cs {

constexpr uint32_t kMaxTerms = 512;   // numerator terms per launch (larger batches are split)
constexpr uint32_t kMaxPoints = 16;   // sample points per quotient launch

struct GenPowersTable {
  cpoint p[31];  // 2^b * M31_CIRCLE_GEN
};
GenPowersTable gen_powers();

struct BaryColumns {
  const uint32_t* ptr[kMaxBatch];
};

struct NumeratorTerms {
  const uint32_t* col[kMaxTerms];
  qm31 c[kMaxTerms];
  qm31 b_sum;
  uint32_t n;
};

struct QuotientAcc {
  const uint32_t* c[4];
};

// The first half of a circle domain: point j = init + j step = T[0][j0] + T[1][j1] + T[2][j2] with
// j = j0 + 2^9 j1 + 2^18 j2 (T[0] holding init + j0 step); the second half is its conjugate.
struct DomainTables {
  cpoint t[3][512];
};
void fill_domain_tables(DomainTables& d, uint32_t half_init, uint32_t half_step);

struct QuotientParams {
  DomainTables tables;
  uint32_t half_init, half_step, sub_log, n_points;
  qm31 px[kMaxPoints], py[kMaxPoints], first_linear[kMaxPoints];
  uint32_t acc_log[kMaxPoints];
  QuotientAcc acc[kMaxPoints];
};

cs_status quotients_on_subdomain(const QuotientParams& q, uint32_t* const out[4], cudaStream_t st);

}  // namespace cs
