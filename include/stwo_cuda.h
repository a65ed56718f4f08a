/*
 * stwo_cuda.h — C ABI of the GB300 (sm_103a) backend for the Stwo
 * Circle-STARK prover hot path.
 *
 * Each entry point is what a Rust `CudaBackend` binds through `extern "C"` to
 * implement one method of the reference's backend trait family
 * (crates/stwo/src/prover/backend/mod.rs:17-35). The reference line each
 * function replaces is cited beside it.
 *
 * Conventions
 *  - Plain pointers and sizes only. Pointers named d_* are device pointers;
 *    h_* are host pointers. Columns of M31 are arrays of uint32_t words in
 *    [0, P), P = 2^31 - 1 (the reference's BaseColumn,
 *    crates/stwo/src/prover/backend/simd/column.rs:26-30). A QM31 column is
 *    four such coordinate arrays (SecureColumnByCoords,
 *    crates/stwo/src/prover/secure_column.rs:13-15). Evaluations are in
 *    bit-reversed order, as in the reference.
 *  - Blake2s digests are 32 bytes, stored as 8 little-endian uint32_t words.
 *  - `cs_stream` is a cudaStream_t (NULL = the legacy default stream). All
 *    device work is enqueued on it and is asynchronous unless stated.
 *  - Every function returns a cs_status. On failure, cs_last_error() gives a
 *    message for the calling thread. The reference's trait methods panic on
 *    misuse; its Rust binding panics on a non-OK status to keep that contract.
 *  - All entry points are thread-safe: they keep no mutable global state
 *    beyond the per-thread error message.
 */
#ifndef STWO_CUDA_H
#define STWO_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  CS_OK = 0,
  CS_ERR_INVALID_ARG = 1,
  CS_ERR_OOM = 2,
  CS_ERR_DEVICE = 3,
  CS_ERR_TIMEOUT = 4,
  CS_ERR_NOT_FOUND = 5
} cs_status;

typedef void *cs_stream;

/* ------------------------------------------------------------ runtime */

/* Message for the last failing call on this thread ("" if none). */
const char *cs_last_error(void);
/* Library version and the compiled architecture, e.g. "stwo-cuda 0.1 sm_103a". */
const char *cs_version(void);

/* Number of kernels this library has launched since it was loaded (all
   threads). Instrumentation only; it has no counterpart in the reference. */
uint64_t cs_kernel_launch_count(void);

/* Device memory for columns: Column::zeros / Column::uninitialized
   (crates/stwo/src/prover/backend/mod.rs:45-66). */
cs_status cs_malloc(void **d_ptr, size_t bytes);
cs_status cs_free(void *d_ptr);
cs_status cs_memset_zero(void *d_ptr, size_t bytes, cs_stream stream);
/* Column::to_cpu / FromIterator (backend/mod.rs:45-66): host <-> device copies. */
cs_status cs_memcpy_h2d(void *d_dst, const void *h_src, size_t bytes, cs_stream stream);
cs_status cs_memcpy_d2h(void *h_dst, const void *d_src, size_t bytes, cs_stream stream);
cs_status cs_memcpy_d2d(void *d_dst, const void *d_src, size_t bytes, cs_stream stream);
cs_status cs_stream_synchronize(cs_stream stream);

/* ------------------------------------------------------------ columns */

/* ColumnOps<BaseField>::bit_reverse_column (crates/stwo/src/prover/backend/mod.rs:37-40;
   SIMD crates/stwo/src/prover/backend/simd/bit_reverse.rs:22-110). In place. */
cs_status cs_bit_reverse_m31(uint32_t *d_col, uint32_t log_size, cs_stream stream);

/* ---------------------------------------------------------- polynomials */

/* PolyOps::precompute_twiddles (crates/stwo/src/prover/poly/circle/ops.rs:160;
   SIMD crates/stwo/src/prover/backend/simd/circle.rs:431-462). Fills the
   TwiddleTree buffers (crates/stwo/src/prover/poly/twiddles.rs:10-15) for the
   coset (root_initial_index + <G_{root_log_size}>): per doubling, the
   x-coordinates of the first half of the coset in bit-reversed order,
   concatenated, plus one pad word = 1. d_twiddles and d_itwiddles (the
   inverses) hold 2^root_log_size words each. */
cs_status cs_precompute_twiddles(uint32_t root_initial_index, uint32_t root_log_size, uint32_t *d_twiddles,
                                 uint32_t *d_itwiddles, cs_stream stream);

/* PolyOps::interpolate / interpolate_columns (crates/stwo/src/prover/poly/circle/ops.rs:25-40;
   SIMD crates/stwo/src/prover/backend/simd/circle.rs:135-163). In place: each
   column holds bit-reversed evaluations on CanonicCoset(log_size) and becomes
   the coefficients in the circle FFT basis. The itwiddle tree must cover the
   domain (root log size >= log_size - 1). */
cs_status cs_interpolate_columns(uint32_t *const *h_cols, uint32_t n_cols, uint32_t log_size,
                                 const uint32_t *d_itwiddles, uint32_t twiddle_log_size, cs_stream stream);

/* Same as cs_interpolate_columns but out of place: h_evals[i] is read and
   left intact, h_coeffs[i] receives the coefficients (the reference's
   interpolate consumes its evaluation and returns new coefficients,
   crates/stwo/src/prover/poly/circle/ops.rs:25-29). Each output may equal its
   input (then it is in place). */
cs_status cs_interpolate_columns_into(const uint32_t *const *h_evals, uint32_t *const *h_coeffs, uint32_t n_cols,
                                      uint32_t log_size, const uint32_t *d_itwiddles, uint32_t twiddle_log_size,
                                      cs_stream stream);

/* PolyOps::evaluate_polynomials / evaluate_into
   (crates/stwo/src/prover/poly/circle/ops.rs:102-140; SIMD
   crates/stwo/src/prover/backend/simd/circle.rs:389-425): coefficients of log
   size log_coeffs, zero-padded, evaluated on CanonicCoset(log_size) in
   bit-reversed order. Each coefficient column is read once for all
   2^(log_size - log_coeffs) blown-up replicas. h_coeffs[i] may not alias h_evals[i]. */
cs_status cs_evaluate_columns(const uint32_t *const *h_coeffs, uint32_t *const *h_evals, uint32_t n_cols,
                              uint32_t log_coeffs, uint32_t log_size, const uint32_t *d_twiddles,
                              uint32_t twiddle_log_size, cs_stream stream);

/* ------------------------------------------------------- lifted Merkle */

/* MerkleOpsLifted::build_leaves (crates/stwo/src/prover/vcs_lifted/ops.rs:14-15;
   CPU crates/stwo/src/prover/backend/cpu/merkle_lifted.rs:46-90; SIMD
   crates/stwo/src/prover/backend/simd/blake2s_lifted.rs:46-229). Columns must
   be sorted by non-decreasing log size (as MerkleProverLifted::commit does,
   crates/stwo/src/prover/vcs_lifted/prover.rs:68). Leaf i = Blake2s-256 of the
   LE words col[(i >> (L - l + 1) << 1) + (i & 1)] of every column in order,
   L = lifting_log_size, l = the column's log size. d_leaves receives 2^L
   digests (8 words each); with n_cols == 0 it receives the one digest of the
   empty input. Up to 2048 columns per call. */
cs_status cs_merkle_build_leaves(const uint32_t *const *h_cols, const uint32_t *h_log_sizes, uint32_t n_cols,
                                 uint32_t lifting_log_size, uint32_t *d_leaves, cs_stream stream);

/* MerkleOpsLifted::build_next_layer (crates/stwo/src/prover/vcs_lifted/ops.rs:19;
   SIMD crates/stwo/src/prover/backend/simd/blake2s_lifted.rs:232-263):
   node i = Blake2s(prev[2i] || prev[2i+1]); d_out gets 2^out_log_size digests. */
cs_status cs_merkle_build_next_layer(const uint32_t *d_prev, uint32_t out_log_size, uint32_t *d_out,
                                     cs_stream stream);

/* MerkleProverLifted::commit without leaf packing
   (crates/stwo/src/prover/vcs_lifted/prover.rs:35-80): leaves, then every
   node layer, in one call. Columns are sorted here (stable, by log size).
   d_layers holds 2^(L+1) - 1 digests: leaves first (2^L), then each parent
   layer, the root last. */
cs_status cs_merkle_commit(const uint32_t *const *h_cols, const uint32_t *h_log_sizes, uint32_t n_cols,
                           uint32_t lifting_log_size, uint32_t *d_layers, cs_stream stream);

/* PackLeavesOps::pack_leaves_input (crates/stwo/src/prover/vcs_lifted/ops.rs:22-30;
   CPU crates/stwo/src/prover/backend/cpu/merkle_lifted.rs:100-124): 4 QM31
   coordinate columns of 2^log_size -> 16 columns of 2^(log_size-2), output
   column coord + 4*offset holds input[coord][4*r + offset]. */
cs_status cs_pack_leaves_input(const uint32_t *const h_in[4], uint32_t log_size, uint32_t *const h_out[16],
                               cs_stream stream);

/* ------------------------------------------------------------------ FRI */

/* FriOps::fold_line (crates/stwo/src/prover/fri.rs:41-45; CPU
   crates/stwo/src/prover/backend/cpu/fri.rs:66-91; SIMD
   crates/stwo/src/prover/backend/simd/fri.rs:32-109) for one step: the QM31
   evaluation (4 coordinate columns of 2^log_size) on the line domain
   x(half_odds(log_size)) folds to 2^(log_size-1) values
   f0 + alpha * f1 with (f0, f1) = ibutterfly(f(x), f(-x), 1/x). The inverse
   x-coordinates come from the itwiddle tree. fold_step > 1 calls it with
   alpha, alpha^2, ... in turn. */
cs_status cs_fold_line(const uint32_t *const h_src[4], uint32_t log_size, const uint32_t alpha[4],
                       uint32_t *const h_dst[4], const uint32_t *d_itwiddles, uint32_t twiddle_log_size,
                       cs_stream stream);

/* FriOps::fold_circle_into_line (crates/stwo/src/prover/fri.rs:62-66; CPU
   crates/stwo/src/prover/backend/cpu/fri.rs:94-116; SIMD
   crates/stwo/src/prover/backend/simd/fri.rs:111-166): from CanonicCoset(log_size)
   to 2^(log_size-1) values alpha * f1 + f0 with (f0, f1) = ibutterfly(f(p), f(-p), 1/p.y). */
cs_status cs_fold_circle_into_line(const uint32_t *const h_src[4], uint32_t log_size, const uint32_t alpha[4],
                                   uint32_t *const h_dst[4], const uint32_t *d_itwiddles,
                                   uint32_t twiddle_log_size, cs_stream stream);

/* -------------------------------------------------------- proof of work */

/* GrindOps<Blake2sChannel>::grind (crates/stwo/src/core/proof_of_work.rs:10-14;
   SIMD crates/stwo/src/prover/backend/simd/grind.rs:36-62): the smallest nonce
   with trailing_zeros(Blake2s(Blake2s(0x12345678_le || digest || bits_le) ||
   nonce_le64)) >= pow_bits, pow_bits <= 32. Synchronous on `stream`: *nonce_out
   is valid on return. Allocates an 8-byte device slot per call (stream-ordered).
   Gives CS_ERR_TIMEOUT when no nonce below max_nonce qualifies. */
cs_status cs_grind_blake2s(const uint8_t digest[32], uint32_t pow_bits, uint64_t max_nonce, uint64_t *nonce_out,
                           cs_stream stream);

#ifdef __cplusplus
}
#endif

#endif /* STWO_CUDA_H */
