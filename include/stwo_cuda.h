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
 *  - All entry points are thread-safe. Process-wide state is limited to:
 *    the per-thread error message; the FFT pass-plan table (cs_fft_set_plan,
 *    guarded by a lock); the fold plan (cs_fold_set_plan, one atomic word);
 *    per-device set-up flags (kernel shared-memory
 *    limits, the memory pool's release threshold; set once under a lock);
 *    the kernel launch counter; and the static slot array of
 *    cs_grind_blake2s_noalloc (shared by its calls, see there).
 *  - Digest and layer buffers of the Merkle entry points must be 16-byte
 *    aligned (digests move as 16-byte words); a misaligned pointer gives
 *    CS_ERR_INVALID_ARG.
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

/* PolyOps::interpolate_columns over a batch of columns of different sizes
   (crates/stwo/src/prover/poly/circle/ops.rs:30-40; SIMD
   crates/stwo/src/prover/backend/simd/circle.rs:135-163): column i holds
   2^h_log_sizes[i] bit-reversed evaluations on CanonicCoset(h_log_sizes[i]);
   h_coeffs[i] receives the coefficients (it may equal h_evals[i]). The
   columns of each size take one batched launch sequence, and the size groups
   run on side streams forked from and joined back into `stream` (events;
   stream capture follows them), so small sizes run beside large ones. */
cs_status cs_interpolate_columns_multi(const uint32_t *const *h_evals, uint32_t *const *h_coeffs,
                                       const uint32_t *h_log_sizes, uint32_t n_cols, const uint32_t *d_itwiddles,
                                       uint32_t twiddle_log_size, cs_stream stream);

/* PolyOps::evaluate_polynomials over polynomials of different sizes
   (crates/stwo/src/prover/poly/circle/ops.rs:109-140): coefficients of log
   size h_log_coeffs[i] evaluated on CanonicCoset(h_log_coeffs[i] + log_blowup)
   into h_evals[i] (no aliasing), size groups concurrent as in
   cs_interpolate_columns_multi. */
cs_status cs_evaluate_columns_multi(const uint32_t *const *h_coeffs, uint32_t *const *h_evals,
                                    const uint32_t *h_log_coeffs, uint32_t log_blowup, uint32_t n_cols,
                                    const uint32_t *d_twiddles, uint32_t twiddle_log_size, cs_stream stream);

/* FFT pass plans (no counterpart in the reference; the reference's SIMD FFT
   fixes its radix split in code). A column of 2^log_n words whose FFT runs
   n_layers layers (interpolate: n_layers = log_n; evaluate: the coefficient
   log size) is processed in passes of consecutive layers, each staged once
   through shared memory. cs_fft_set_plan installs the pass sizes for one
   (direction, log_n, n_layers) shape, process-wide (first pass 1..12 layers and
   at least 3 when more follow, later passes 1..11, summing to n_layers);
   n_passes = 0 removes it. Results do not depend on the plan, only speed does.
   cs_fft_get_plan returns the plan in use (up to 32 passes). Thread-safe. */
cs_status cs_fft_set_plan(uint32_t inverse, uint32_t log_n, uint32_t n_layers, const uint32_t *pass_layers,
                          uint32_t n_passes);
cs_status cs_fft_get_plan(uint32_t inverse, uint32_t log_n, uint32_t n_layers, uint32_t *pass_layers,
                          uint32_t *n_passes);

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

/* The layer loop of MerkleProverLifted::commit (crates/stwo/src/prover/vcs_lifted/prover.rs:35-80)
   above given leaves: d_layers holds the 2^lifting_log_size leaf digests followed by room for
   every node layer (2^(L+1) - 1 digests in all, root last, the layout of cs_merkle_commit).
   Layers of more than 2^10 nodes take one launch each, the rest of the tree one launch. */
cs_status cs_merkle_build_layers(uint32_t *d_layers, uint32_t lifting_log_size, cs_stream stream);

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
   x-coordinates come from the itwiddle tree. */
cs_status cs_fold_line(const uint32_t *const h_src[4], uint32_t log_size, const uint32_t alpha[4],
                       uint32_t *const h_dst[4], const uint32_t *d_itwiddles, uint32_t twiddle_log_size,
                       cs_stream stream);

/* FriOps::fold_line with n_alphas challenges (crates/stwo/src/prover/fri.rs:27-45):
   the evaluation folded n_alphas times (1 <= n_alphas <= log_size), fold j
   with h_alphas[4 j .. 4 j + 3] (host words), into 2^(log_size - n_alphas)
   values in h_dst; only the last layer is written. Up to 12 folds per launch
   in registers, warp shuffles and shared memory (16-byte aligned source and
   twiddles), else up to 10 on tiles staged in shared memory; uses
   stream-ordered device scratch between launches. cs_fold_set_plan sets how
   many values (2^3 or 2^4, the default) a thread of the register launches
   folds before the shuffles; it changes the launch shapes, not the results.
   Process-wide, thread-safe. */
cs_status cs_fold_set_plan(uint32_t log_values_per_thread);
cs_status cs_fold_get_plan(uint32_t *log_values_per_thread);
cs_status cs_fold_line_steps(const uint32_t *const h_src[4], uint32_t log_size, uint32_t n_alphas,
                             const uint32_t *h_alphas, uint32_t *const h_dst[4], const uint32_t *d_itwiddles,
                             uint32_t twiddle_log_size, cs_stream stream);

/* FriOps::fold_circle_into_line (crates/stwo/src/prover/fri.rs:62-66; CPU
   crates/stwo/src/prover/backend/cpu/fri.rs:94-116; SIMD
   crates/stwo/src/prover/backend/simd/fri.rs:111-166): from CanonicCoset(log_size)
   to 2^(log_size-1) values alpha * f1 + f0 with (f0, f1) = ibutterfly(f(p), f(-p), 1/p.y). */
cs_status cs_fold_circle_into_line(const uint32_t *const h_src[4], uint32_t log_size, const uint32_t alpha[4],
                                   uint32_t *const h_dst[4], const uint32_t *d_itwiddles,
                                   uint32_t twiddle_log_size, cs_stream stream);

/* Same as cs_interpolate_columns on the subdomain of log size log_size of
   CanonicCoset(domain_log_size): its first 2^log_size points in bit-reversed
   order, a non-canonic circle domain. Its twiddles are the prefixes of the
   domain's layers (TwiddleBuffer::extract_subdomain_twiddles,
   crates/stwo/src/prover/poly/twiddles.rs:40-76); used by the quotient
   combination (crates/stwo/src/prover/backend/cpu/quotients.rs:82-99) and
   DomainEvaluationAccumulator::finalize
   (crates/stwo/src/prover/air/accumulation.rs:153-167). In place. */
cs_status cs_interpolate_columns_on_subdomain(uint32_t *const *h_cols, uint32_t n_cols, uint32_t log_size,
                                              uint32_t domain_log_size, const uint32_t *d_itwiddles,
                                              uint32_t twiddle_log_size, cs_stream stream);

/* ------------------------------------------------------- accumulation */

/* AccumulationOps::accumulate (crates/stwo/src/prover/air/accumulation.rs:186;
   CPU crates/stwo/src/prover/backend/cpu/accumulation.rs:9-14): col += other
   for QM31 columns of 2^log_size. */
cs_status cs_accumulate(uint32_t *const h_col[4], const uint32_t *const h_other[4], uint32_t log_size,
                        cs_stream stream);

/* AccumulationOps::generate_secure_powers (accumulation.rs:189; CPU
   cpu/accumulation.rs:16-24): felt^0 .. felt^(n-1) into h_out (4 words each).
   Host computation, synchronous. */
cs_status cs_generate_secure_powers(const uint32_t felt[4], uint32_t n_powers, uint32_t *h_out);

/* AccumulationOps::lift_and_accumulate (accumulation.rs:198-200; CPU
   cpu/accumulation.rs:26-47): h_cols holds n_cols x 4 coordinate pointers of
   QM31 columns with strictly increasing log sizes; each column is updated in
   place with the lift of the running sum, so the last holds the result. */
cs_status cs_lift_and_accumulate(uint32_t *const *h_cols, const uint32_t *h_log_sizes, uint32_t n_cols,
                                 cs_stream stream);

/* ------------------------------------------------- out-of-domain samples */

/* PolyOps::barycentric_weights_into (crates/stwo/src/prover/poly/circle/ops.rs:54-58;
   CPU crates/stwo/src/prover/backend/cpu/circle.rs:100-132) for
   CanonicCoset(log_size) and the QM31 point (px, py): 2^log_size QM31 weights
   in bit-reversed order. The point must lie outside the domain. */
cs_status cs_barycentric_weights(uint32_t log_size, const uint32_t px[4], const uint32_t py[4],
                                 uint32_t *const h_out[4], cs_stream stream);

/* PolyOps::barycentric_eval_at_point (ops.rs:70-78; CPU cpu/circle.rs:134-140)
   for n_cols columns of 2^log_size sharing one weight column: d_out[4 i .. 4 i + 3]
   receives column i's value (QM31). */
cs_status cs_barycentric_eval(const uint32_t *const *h_cols, uint32_t n_cols, uint32_t log_size,
                              const uint32_t *const h_weights[4], uint32_t *d_out, cs_stream stream);

/* PolyOps::eval_at_point on coefficients (ops.rs:44-47; CPU cpu/circle.rs:81-98)
   for n_cols coefficient columns of 2^log_size at the QM31 point (px, py):
   d_out[4 i ..] receives column i's value. */
cs_status cs_eval_at_point(const uint32_t *const *h_coeffs, uint32_t n_cols, uint32_t log_size, const uint32_t px[4],
                           const uint32_t py[4], uint32_t *d_out, cs_stream stream);

/* ------------------------------------------------------ DEEP quotients */

/* QuotientOps::accumulate_numerators for one ColumnSampleBatch
   (crates/stwo/src/prover/pcs/quotient_ops.rs:29-34; CPU
   crates/stwo/src/prover/backend/cpu/quotients.rs:23-49): the batch's n_terms
   columns (all of 2^log_size), and per term the line coefficients (a, b, c)
   already scaled by the term's random power (12 words per term, from
   complex_conjugate_line_coeffs, crates/stwo/src/core/constraints.rs:119-135).
   Row r < 2^(log_size - log_blowup) of h_out gets sum_t (c_t col_t[r] - b_t);
   first_linear_out = sum_t a_t. */
cs_status cs_accumulate_numerators(const uint32_t *const *h_cols, uint32_t n_terms, uint32_t log_size,
                                   uint32_t log_blowup, const uint32_t *h_coeffs, uint32_t *const h_out[4],
                                   uint32_t first_linear_out[4], cs_stream stream);

/* First half of QuotientOps::compute_quotients_and_combine
   (quotient_ops.rs:47-52; CPU cpu/quotients.rs:51-81): for each of n_points
   sample points (h_points: x then y, 8 words each) with its lifted partial
   numerator column (h_accs: 4 coordinate pointers per point, log size
   h_acc_log_sizes[k] <= L - b) and first linear term (4 words), the quotient
   sum_k (acc_k[lifted r] - a_k * y) / den_k(x, y) on the subdomain of log
   L - b of CanonicCoset(L), bit-reversed. The caller then interpolates it on
   that subdomain and evaluates it on CanonicCoset(L). Up to 16 points. */
cs_status cs_quotients_on_subdomain(const uint32_t *const *h_accs, const uint32_t *h_acc_log_sizes, uint32_t n_points,
                                    const uint32_t *h_points, const uint32_t *h_first_linear, uint32_t lifting_log_size,
                                    uint32_t log_blowup, uint32_t *const h_out[4], cs_stream stream);

/* FriOps::decompose (crates/stwo/src/prover/fri.rs:73-75; CPU
   crates/stwo/src/prover/backend/cpu/fri.rs:39-61,134-145): lambda = (sum of
   the first half - sum of the second half) / 2^log_size; dst = src - lambda
   on the first half, src + lambda on the second. Synchronous: lambda_out is
   valid on return. Uses an 8-word stream-ordered device scratch buffer. */
cs_status cs_decompose(const uint32_t *const h_src[4], uint32_t log_size, uint32_t *const h_dst[4],
                       uint32_t lambda_out[4], cs_stream stream);

/* ------------------------------------------------ AIR: Wide-Fibonacci */

/* Constraint quotients of the Wide-Fibonacci component on its evaluation
   domain: the device analogue of FrameworkComponent::
   evaluate_constraint_quotients_on_domain
   (crates/constraint-framework/src/prover/component_prover.rs:195-268) for
   WideFibonacciEval (crates/examples/src/wide_fibonacci/mod.rs:87-97), in
   the SubDomain mode with log_expansion 0. h_cols: the n_cols trace
   evaluations on CanonicCoset(eval_log) (bit-reversed); h_rc: the component's
   n_cols - 2 random-coefficient powers in constraint order (4 words each).
   Row r adds sum_k rc[k] (c_{k+2} - c_k^2 - c_{k+1}^2) / V_trace(x_r) to the
   QM31 accumulator h_accum (2^eval_log values). */
cs_status cs_wide_fib_composition(const uint32_t *const *h_cols, uint32_t n_cols, uint32_t eval_log, uint32_t trace_log,
                                  const uint32_t *h_rc, uint32_t *const h_accum[4], cs_stream stream);

/* Wide-Fibonacci trace generation (crates/examples/src/wide_fibonacci/mod.rs:27-48)
   on the device: column 0 = a, column 1 = b, then (a, b) <- (b, a^2 + b^2). */
cs_status cs_wide_fib_trace(const uint32_t *d_a, const uint32_t *d_b, uint32_t log_n, uint32_t n_cols,
                            uint32_t *const *h_cols, cs_stream stream);

/* LogUp interaction column on the device: the last column of
   LogupTraceGenerator (crates/constraint-framework/src/prover/logup.rs:50-130)
   with numerator 1 and denominator z - v_i for the M31 column d_values
   (2^log_size values, bit-reversed circle-domain order, log_size >= 1):
   claimed_sum = sum_i 1/(z - v_i) (returned on the host, synchronous), then
   the shifted fractions' inclusive prefix sum in coset order
   (inclusive_prefix_sum, crates/stwo/src/prover/backend/simd/prefix_sum.rs:20)
   into the QM31 column h_out. Uses stream-ordered device scratch. */
cs_status cs_logup_running_sum(const uint32_t *d_values, uint32_t log_size, const uint32_t z[4], uint32_t *const h_out[4],
                               uint32_t claimed_sum_out[4], cs_stream stream);

/* LogupTraceGenerator (crates/constraint-framework/src/prover/logup.rs:22-196) on the
   device, for relations of any number of values and multiplicities; columns of
   2^log_size rows in bit-reversed circle-domain order, QM31 columns as 4
   coordinate arrays.
   cs_logup_combine: LookupElements::combine (crates/constraint-framework/src/
   logup.rs:80-94) per row, den = sum_i alpha^i values_i - z over n_values M31
   columns h_values[i], alpha_powers holding alpha^i as 4 words each.
   cs_logup_gen_col: LogupColGenerator::write_frac for every row then
   finalize_col: out = num / den + prev, with num either the QM31 column h_num
   (4 coordinates) or the M31 column d_num_m31 (exactly one of them non-null)
   and prev the generator's previous column (h_prev, 4 coordinates) or null for
   the first. A zero denominator gives a zero fraction.
   cs_logup_finalize_last: LogupTraceGenerator::finalize_last in place on the
   last column: claimed_sum = its sum (returned on the host, synchronous), every
   value minus claimed_sum / 2^log_size, then the inclusive prefix sum in coset
   order (1 <= log_size <= 28). */
cs_status cs_logup_combine(const uint32_t *const *h_values, uint32_t n_values, uint32_t log_size,
                           const uint32_t *alpha_powers, const uint32_t z[4], uint32_t *const h_den[4],
                           cs_stream stream);
cs_status cs_logup_gen_col(const uint32_t *const *h_num, const uint32_t *d_num_m31, const uint32_t *const h_den[4],
                           const uint32_t *const *h_prev, uint32_t log_size, uint32_t *const h_out[4],
                           cs_stream stream);
cs_status cs_logup_finalize_last(uint32_t *const h_col[4], uint32_t log_size, uint32_t claimed_sum_out[4],
                                 cs_stream stream);

/* cs_logup_running_sum for n_cols columns of any log sizes in [1, 28] in one
   batch of launches (three per 48 columns), with no host synchronization:
   column i reads h_values[i] (2^h_log_sizes[i] device words) and writes its
   running sum into the coordinates h_out[4 i .. 4 i + 3]; its claimed sum
   goes to d_claimed[4 i .. 4 i + 3] in device memory. Uses stream-ordered
   device scratch. */
cs_status cs_logup_running_sums(uint32_t n_cols, const uint32_t *const *h_values, const uint32_t *h_log_sizes,
                                const uint32_t z[4], uint32_t *const *h_out, uint32_t *d_claimed, cs_stream stream);

/* Constraint quotients of a single-column LogUp component (no counterpart
   AIR in the reference; built from its constraint framework): the relation
   entry (multiplicity -1, values [v]) finalized with finalize_logup
   (crates/constraint-framework/src/lib.rs:185-227), whose interaction column is
   cs_logup_running_sum's. Row r of CanonicCoset(eval_log) adds
   rc (cur - prev + claimed_sum / 2^trace_log) (v - z) + 1 over V_trace(x_r)
   to h_accum, with cur / prev the interaction column (h_inter, 4 coordinates)
   at the row and one trace step before, v = d_values[r]. */
cs_status cs_logup_composition(const uint32_t *d_values, const uint32_t *const h_inter[4], uint32_t eval_log,
                               uint32_t trace_log, const uint32_t z[4], const uint32_t claimed_sum[4],
                               const uint32_t rc[4], uint32_t *const h_accum[4], cs_stream stream);

/* cs_logup_composition for n_comp components of the same trace size, their
   quotients summed per row and added to h_accum once: component k reads
   h_values[k] and the coordinates h_inter[4 k .. 4 k + 3], with its claimed
   sum claimed_sums[4 k .. 4 k + 3] and weight rcs[4 k .. 4 k + 3] (host
   words). One launch per 24 components. */
cs_status cs_logup_compositions(uint32_t n_comp, const uint32_t *const *h_values, const uint32_t *const *h_inter,
                                uint32_t eval_log, uint32_t trace_log, const uint32_t z[4],
                                const uint32_t *claimed_sums, const uint32_t *rcs, uint32_t *const h_accum[4],
                                cs_stream stream);

/* ------------------------------------------------- GKR lookups (GkrOps, MleOps) */

/* The backend's GkrOps and MleOps (crates/stwo/src/prover/lookups/gkr_prover.rs:22-42,
   crates/stwo/src/prover/lookups/mle.rs:9-14). A multilinear extension of n
   variables is its 2^n values on the boolean hypercube (variable j = index bit
   n-1-j): a secure MLE is 4 coordinate columns, a base MLE one column. Layer
   kinds follow gkr_prover.rs Layer: a grand-product layer is one secure column,
   passed as the denominators; LogUp layers have numerators (secure, base for
   multiplicities, none for singles, whose numerators are all 1) and secure
   denominators. Input columns of next_layer and sum_as_poly are 8-byte aligned. */
enum {
  CS_GKR_GRAND_PRODUCT = 0,
  CS_GKR_LOGUP_GENERIC = 1,
  CS_GKR_LOGUP_MULTIPLICITIES = 2,
  CS_GKR_LOGUP_SINGLES = 3
};

/* GkrOps::gen_eq_evals: h_out[k][i] = coordinate k of v * eq(x, y) for the
   2^n_y points x of the hypercube (n_y <= 28; y is n_y QM31 values of 4 host
   words each, v 4 host words). */
cs_status cs_gkr_gen_eq_evals(const uint32_t *h_y, uint32_t n_y, const uint32_t h_v[4], uint32_t *const h_out[4],
                              cs_stream stream);

/* MleOps::fix_first_variable for a base (src_is_base != 0: h_src[0] only) or
   secure MLE of 2^log_n values: the 2^(log_n - 1) secure values
   a * (rhs - lhs) + lhs of the two halves. h_dst may alias h_src. */
cs_status cs_mle_fix_first_variable(const uint32_t *const h_src[4], uint32_t src_is_base, uint32_t log_n,
                                    const uint32_t h_assignment[4], uint32_t *const h_dst[4], cs_stream stream);

/* GkrOps::next_layer for an input layer of 2^log_n values per column
   (log_n >= 1): a grand-product layer gives the pairwise products in
   h_out_den; a LogUp layer gives the pairwise fraction sums as a generic
   LogUp layer (h_out_num, h_out_den). */
cs_status cs_gkr_next_layer(uint32_t kind, const uint32_t *const h_num[4], const uint32_t *const h_den[4],
                            uint32_t log_n, uint32_t *const h_out_num[4], uint32_t *const h_out_den[4],
                            cs_stream stream);

/* The device sums of GkrOps::sum_as_poly_in_first_variable for the oracle
   whose input layer has 2^log_n values per column (log_n >= 2): with
   n_terms = 2^(log_n - 2), sum over i < n_terms of eq[i] times the gate's
   output on the input layer at t = 0 and t = 2 (LogUp gates combined as
   numerator + lambda * denominator), written as 8 words (f(0), f(2)) to
   device memory d_out. The eq column holds at least n_terms values. The host
   applies eq_fixed_var_correction and correct_sum_as_poly_in_first_variable.
   Uses stream-ordered device scratch. */
cs_status cs_gkr_sum_as_poly(uint32_t kind, const uint32_t *const h_eq[4], const uint32_t *const h_num[4],
                             const uint32_t *const h_den[4], uint32_t log_n, const uint32_t h_lambda[4], uint32_t *d_out,
                             cs_stream stream);

/* GKR batch proof (prove_batch, crates/stwo/src/prover/lookups/gkr_prover.rs,
   with sumcheck::prove_batch, crates/stwo/src/prover/lookups/sumcheck.rs) with
   the protocol in native code over the kernels above. Instance i has layer
   kind h_kinds[i], h_n_variables[i] variables (1..29) and columns
   h_columns[8 i .. 8 i + 7]: the numerators' 4 coordinates (generic LogUp; the
   first only for multiplicities; unused otherwise), then the 4 coordinates of
   the denominators or of the grand-product column. The input columns are read,
   not changed. h_channel is the Blake2s channel state (8 digest words, then the
   draw counter), updated on return. The words written (one u64 each):
     proof:    n_layers, per layer: n_rounds, per round: n_coeffs, coeffs;
               n_instances, per instance: n_masks, per mask: n_columns, per
               column: v0, v1; per instance: n_output_claims, claims;
     artifact: n_ood, ood point; per instance: n_claims, claims to verify;
               per instance: n_variables,
   each QM31 as its 4 coordinates. With h_words null only *n_words is set.
   Uses stream-ordered device scratch; synchronises the stream once per
   sum-check round. */
cs_status cs_gkr_prove_batch(uint32_t n_instances, const uint32_t *h_kinds, const uint32_t *h_n_variables,
                             const uint32_t *const *h_columns, uint32_t h_channel[9], uint64_t *h_words,
                             size_t capacity, size_t *n_words, cs_stream stream);

/* ------------------------------------------------- native Wide-Fibonacci prover */

/* The whole proof of Wide-Fibonacci components (the generic prover's loop,
   prove_ex, crates/stwo/src/prover/mod.rs:39-138, over this library's
   kernels, with the host work in native code): the empty preprocessed tree,
   the components' traces in one lifted tree, the constraint quotients, the
   OODS samples, FRI (fold_step folds per layer) and the decommitments, returned as the
   CairoSerialize felt stream of the StarkProof (one u64 per felt). The
   channel starts from the zero digest. d_trace holds the components'
   columns one after another (2^log_sizes[k] words each, bit-reversed
   evaluations on CanonicCoset(log_sizes[k]); interpolated in place).
   lifting_log_size must be the largest log size + 1 (log_blowup_factor 1).
   The twiddle trees cover CanonicCoset(lifting_log_size). With h_words null
   only *n_words is set. */
typedef struct {
  uint32_t n_components;
  const uint32_t *n_cols;    /* per component, >= 3 */
  const uint32_t *log_sizes; /* per component */
  uint32_t lifting_log_size;
  uint32_t pow_bits, log_blowup_factor, log_last_layer_degree_bound, n_queries;
  const uint32_t *d_twiddles, *d_itwiddles;
  uint32_t twiddle_log_size;
  uint32_t flags; /* 0, or CS_PROVE_PLAIN */
  uint32_t fold_step; /* FRI folds per layer, 1..8 (0 reads as 1); above 1 the layer
                         trees commit packed leaves of 4 values per coordinate and the
                         channel stays on the host for the layer loop */
} cs_wide_fib_proof_params;
/* flags: the plain form, one launch per column for every per-column stage (interpolate, evaluate,
   running sums, out-of-domain sampling, LogUp quotients), as the trait's default per-column loops
   run on a backend without batched overrides. Same proof bytes; for comparison. */
#define CS_PROVE_PLAIN 1u
cs_status cs_prove_wide_fib(const cs_wide_fib_proof_params *params, uint32_t *const *d_trace, uint64_t *h_words,
                            size_t capacity, size_t *n_words, cs_stream stream);
/* cs_prove_wide_fib with n_lookups single-column LogUp components beside the
   Wide-Fibonacci components (relation entry of multiplicity -1 and values [v]):
   component k's looked-up values are d_values[k] (2^h_lookup_log_sizes[k] words,
   trace domain, kept); their value columns follow the Wide-Fibonacci columns in
   the trace tree, their QM31 running sums form the interaction tree (mixed into
   the channel after the claimed sums, which go to h_claimed, 4 words each).
   The lifting log size is the largest of all log sizes + 1. */
cs_status cs_prove_fib_and_lookups(const cs_wide_fib_proof_params *params, uint32_t *const *d_trace,
                                   uint32_t n_lookups, const uint32_t *const *d_values,
                                   const uint32_t *h_lookup_log_sizes, uint32_t *h_claimed, uint64_t *h_words,
                                   size_t capacity, size_t *n_words, cs_stream stream);

/* The whole proof of the Poseidon2 AIR at 2^log_n_rows rows (8 instances per
   row, prove_poseidon, crates/examples/src/poseidon/mod.rs:320-379), trace and
   interaction generated on the device, constraint quotients on
   CanonicCoset(log_n_rows + 2). params: the FRI parameters and twiddles
   (n_components, n_cols and log_sizes unused); lifting_log_size =
   log_n_rows + 2. Without the sanity check, which the reference's own prove of
   this AIR fails (lifted protocol, constraint degree 5): the words are the
   proof it computes before it. */
cs_status cs_prove_poseidon(uint32_t log_n_rows, const cs_wide_fib_proof_params *params, uint64_t *h_words,
                            size_t capacity, size_t *n_words, cs_stream stream);

/* Blake2s-256 of a message on the host (RFC 7693), the native prover's channel hash. */
cs_status cs_host_blake2s(const uint8_t *msg, size_t n, uint8_t out[32]);

/* ------------------------------------------- run-time compiled constraints */

/* The generic constraint path: the source of one kernel, made by
   proving_gb300/framework.py from an AIR's constraints (the reference's
   ExprEvaluator form, crates/constraint-framework/src/expr/evaluator.rs:58-123),
   compiled with NVRTC for sm_103a (libnvrtc opened at run time) and loaded with
   the runtime's library API. The kernel is
     extern "C" __global__ void cs_air_composition(const uint32_t* const* cols,
         const uint32_t* rc, const uint32_t* params, const uint32_t* den,
         uint32_t eval_log, uint32_t trace_log,
         uint32_t* a0, uint32_t* a1, uint32_t* a2, uint32_t* a3)
   and adds, at every row of CanonicCoset(eval_log), the sum over the
   constraints of rc[k] C_k(row) over V_trace(row) to the accumulator.
   cs_rtc_available reports whether NVRTC can be opened. cs_rtc_compile_air
   compiles `source` with the given in-memory headers and returns a handle (and
   the compiler log, truncated to log_capacity). cs_rtc_air_composition runs it:
   h_cols holds the n_cols mask columns (device, evaluation domain), h_rc 4
   words per constraint and h_params 4 words per QM31 parameter (host). */
cs_status cs_rtc_available(void);
cs_status cs_rtc_compile_air(const char *source, uint32_t n_headers, const char *const *header_sources,
                             const char *const *header_names, uint32_t n_cols, uint32_t n_constraints,
                             uint32_t n_params, void **handle_out, char *log_out, size_t log_capacity);
cs_status cs_rtc_air_composition(void *handle, const uint32_t *const *h_cols, const uint32_t *h_rc,
                                 const uint32_t *h_params, uint32_t eval_log, uint32_t trace_log,
                                 uint32_t *const h_accum[4], cs_stream stream);
/* The same on the subdomain of a committed evaluation (EvaluationMode::SubDomain
   { log_expansion }, crates/stwo/src/prover/air/accumulation.rs:20-62, with
   subdomain_eval_domain, crates/constraint-framework/src/prover/component_prover.rs:234-238):
   the rows are the first 2^eval_log of columns committed on
   CanonicCoset(eval_log + log_expansion) in bit-reversed order, and the
   denominators are V_trace at those points. log_expansion 0 is
   cs_rtc_air_composition. */
cs_status cs_rtc_air_composition_subdomain(void *handle, const uint32_t *const *h_cols, const uint32_t *h_rc,
                                           const uint32_t *h_params, uint32_t eval_log, uint32_t trace_log,
                                           uint32_t log_expansion, uint32_t *const h_accum[4], cs_stream stream);
cs_status cs_rtc_release(void *handle);
/* cs_rtc_compile_air for an AIR with LogUp batches (finalize_logup_batched): the
   source also holds cs_air_fractions(cols, params, log_n, out), which writes at
   every row of the trace domain each batch's combined numerator and denominator
   (QM31, out[8 j .. 8 j + 3] and out[8 j + 4 .. 8 j + 7]) from the n_frac_cols
   trace columns its masks read; cs_rtc_air_fractions launches it (h_cols: those
   columns on the trace domain, h_out: 8 n_batches device columns of 2^log_n
   words). The values LogupTraceGenerator's columns are written from
   (crates/constraint-framework/src/prover/logup.rs:22-130). */
cs_status cs_rtc_compile_air_logup(const char *source, uint32_t n_headers, const char *const *header_sources,
                                   const char *const *header_names, uint32_t n_cols, uint32_t n_constraints,
                                   uint32_t n_params, uint32_t n_frac_cols, uint32_t n_batches, void **handle_out,
                                   char *log_out, size_t log_capacity);
cs_status cs_rtc_air_fractions(void *handle, const uint32_t *const *h_cols, const uint32_t *h_params, uint32_t log_n,
                               uint32_t *const *h_out, cs_stream stream);
/* The column-table size, constraint count and parameter count a kernel was compiled for. */
cs_status cs_rtc_kernel_shape(void *handle, uint32_t *n_cols, uint32_t *n_constraints, uint32_t *n_params);

/* prove_ex for components written against the constraint evaluator
   (proving_gb300/air_prover.py's FrameworkComponent), their constraints through
   kernels compiled with cs_rtc_compile_air(_logup): the empty preprocessed tree,
   one trace tree of every component's columns in component order (d_trace,
   2^log_size words each on the trace domain, bit-reversed; interpolated in place
   unless the component has relations, so consumed), then, when a component has
   LogUp relations, the lookup elements (z, alpha: two channel draws) and one
   interaction tree of every such component's 4 n_batches coordinate columns,
   generated from its fraction kernel (cs_rtc_air_fractions) as the
   LogupTraceGenerator writes them; with flags & CS_PROVE_MIX_CLAIMED the claimed
   sums are mixed into the channel before that tree's root. log_blowup_factor
   1..16, any fold_step. The evaluation mode is EvaluationMode::infer's
   (crates/stwo/src/prover/air/accumulation.rs:42-62): when every component's
   constraint log degree d is at most the blowup b, by the same b - d, the
   constraints run on the first 2^(log_size + d) committed evaluations (SubDomain)
   and the composition is interpolated on that subdomain; else on
   CanonicCoset(log_size + d), the committed evaluations when that is their
   domain, else the coefficients evaluated there (ExtendToEvalDomain). Constraints
   of log degree 2 are proved without the sanity check, which the reference's
   lifted protocol fails for them (the words are the proof it computes before it).
   A trace column is sampled at the OODS point plus each of its mask offsets in
   steps of CanonicCoset(lifting_log_size - 1) (component.rs:202-214), an
   interaction column at the point, or at the previous row and the point when
   inter_two says so. The constraints at the point come from `program`: n_nodes
   nodes of 5 words (op, a0..a3) in topological order, op 0 = the sampled value
   of column a0 of tree a2 (1: trace, 2: interaction; local to the component) at
   its a1-th offset, 1 = the M31 constant a0, 2 = parameter a0, 3 =
   from_partial_evals of nodes a0..a3, 4 = -a0, 5 = a0 + a1, 6 = a0 - a1, 7 =
   a0 * a1; constraint k is node constraints[k]. Kernel mask i reads local
   column mask_cols[i] of tree mask_trees[i]. param_kinds: per parameter, 0 =
   its value in params, 1 = z, 2 = the shift claimed sum / 2^log_size, 3 + i =
   alpha^i. params: the FRI parameters and twiddles (n_components, n_cols and
   log_sizes unused); lifting_log_size = the largest log_size + degree - 1 +
   log_blowup_factor. */
typedef struct {
  void *kernel;                  /* cs_rtc_compile_air(_logup) handle */
  uint32_t log_size;             /* 2^log_size trace rows */
  uint32_t constraint_log_degree;/* 1 or 2 */
  uint32_t n_cols;               /* trace columns the component takes */
  const int32_t *offsets;        /* every trace column's mask offsets, concatenated */
  const uint32_t *offsets_start; /* n_cols + 1 starts into offsets */
  uint32_t n_masks;              /* the kernel's column table */
  const uint32_t *mask_cols;
  const uint32_t *mask_trees;
  const uint32_t *program;       /* 5 words per node */
  uint32_t n_nodes;
  const uint32_t *constraints;
  uint32_t n_constraints;
  const uint32_t *params;        /* 4 words per parameter */
  const uint32_t *param_kinds;   /* one per parameter */
  uint32_t n_params;
  uint32_t n_batches;            /* LogUp interaction columns (0: none) */
  uint32_t n_frac_cols;          /* the trace columns the fraction kernel reads */
  const uint32_t *frac_cols;
  const uint32_t *inter_two;     /* 4 n_batches flags */
} cs_air_component;
#define CS_PROVE_MIX_CLAIMED 2u
cs_status cs_prove_air(const cs_wide_fib_proof_params *params, const cs_air_component *components,
                       uint32_t n_components, uint32_t *const *d_trace, uint64_t *h_words, size_t capacity,
                       size_t *n_words, cs_stream stream);

/* ------------------------------------------------------- AIR: Poseidon2 */

/* The Poseidon2 AIR of crates/examples/src/poseidon/mod.rs (state width 16,
   4 + 4 full rounds, 14 partial rounds, x^5, round constants 1234, 8
   instances of 158 columns per row: 1264 trace columns, 32 interaction
   columns, 1144 constraints). Columns are 2^log_n words in bit-reversed
   circle-domain order; tables hold device pointers. */

/* gen_trace (mod.rs:195-275) on the device: instance k of row r starts from
   state word i = r + i + k. h_cols: 1264 columns of 2^log_n words. */
cs_status cs_poseidon_trace(uint32_t log_n, uint32_t *const *h_cols, cs_stream stream);

/* gen_interaction_trace (mod.rs:277-303) with LogupTraceGenerator
   (crates/constraint-framework/src/prover/logup.rs:55-130): for instance k the
   fraction 1/combine(initial) - 1/combine(final), combine(v) = sum_i alpha^i v_i - z
   (crates/constraint-framework/src/logup.rs:80-93); QM31 column k < 7 (h_out[4k .. 4k+4])
   holds the row sum over instances 0..k, column 7 the row totals minus
   claimed_sum / 2^log_n, inclusive-prefix-summed in coset order. lookup = z || alpha
   (8 words). Synchronous: claimed_sum_out is valid on return. */
cs_status cs_poseidon_interaction(const uint32_t *const *h_trace, uint32_t log_n, const uint32_t lookup[8],
                                  uint32_t *const *h_out, uint32_t claimed_sum_out[4], cs_stream stream);

/* Constraint quotients of the Poseidon component on CanonicCoset(eval_log):
   the device analogue of FrameworkComponent::evaluate_constraint_quotients_on_domain
   (crates/constraint-framework/src/prover/component_prover.rs:111-193) for
   eval_poseidon_constraints (mod.rs:137-189). h_trace / h_inter: the 1264
   trace and 32 interaction columns evaluated on that domain; h_rc: the 1144
   random-coefficient powers in constraint order (host, 4 words each); row r
   adds sum_k rc[k] C_k(r) / V_trace(x_r) to the QM31 accumulator h_accum.
   With eval_log == trace_log the rows are the trace domain and no denominator
   is applied (a valid trace gives all-zero rows). */
cs_status cs_poseidon_composition(const uint32_t *const *h_trace, const uint32_t *const *h_inter, uint32_t eval_log,
                                  uint32_t trace_log, const uint32_t lookup[8], const uint32_t claimed_sum[4],
                                  const uint32_t *h_rc, uint32_t *const h_accum[4], cs_stream stream);

/* FriOps::fold_line / fold_circle_into_line with the folding challenge read
   from device memory (4 words at d_alpha, where cs_channel_draw_secure_felt
   left it) instead of the host. Same results as the host-alpha forms. */
cs_status cs_fold_line_device_alpha(const uint32_t *const h_src[4], uint32_t log_size, const uint32_t *d_alpha,
                                    uint32_t *const h_dst[4], const uint32_t *d_itwiddles, uint32_t twiddle_log_size,
                                    cs_stream stream);
cs_status cs_fold_circle_into_line_device_alpha(const uint32_t *const h_src[4], uint32_t log_size,
                                                const uint32_t *d_alpha, uint32_t *const h_dst[4],
                                                const uint32_t *d_itwiddles, uint32_t twiddle_log_size,
                                                cs_stream stream);

/* ------------------------------------------------------- channel */

/* The Blake2s channel (crates/stwo/src/core/channel/blake2s.rs:16-118) with
   its state in device memory: d_state holds 9 words, the 32-byte digest as 8
   LE words then the draw counter. Lets the FRI commit loop (commit a layer, mix
   its root, draw the challenge, fold) run without a host round trip per layer;
   the caller copies the state back once.
   cs_channel_mix_root: Blake2sMerkleChannel::mix_hash
   (crates/stwo/src/core/vcs_lifted/blake2_merkle.rs:56-58) of the 8-word digest
   at d_root (e.g. the last digest of a cs_merkle_commit layer buffer).
   cs_channel_draw_secure_felt: Channel::draw_secure_felt (blake2s.rs:69-74)
   into d_felt (4 words). Both enqueue one single-thread kernel on `stream`. */
cs_status cs_channel_mix_root(uint32_t *d_state, const uint32_t *d_root, cs_stream stream);
cs_status cs_channel_draw_secure_felt(uint32_t *d_state, uint32_t *d_felt, cs_stream stream);

/* The small layers of FriProver::commit (crates/stwo/src/prover/fri.rs:113-207, fold_step 1) in one
   launch: for j = 0 .. n_layers - 1, the line layer j of log (log_size - j) at h_evals[4j .. 4j+3]
   (four coordinate columns) is committed into h_trees[j] (the cs_merkle_commit layout of a tree of
   that height: ((2 << m) - 1) x 8 words, leaves first, root last; 16-byte aligned), its root is
   mixed into the channel at d_state (cs_channel_mix_root), the folding challenge drawn into
   d_alphas[4j .. 4j+3] (cs_channel_draw_secure_felt), and the layer folded
   (cs_fold_line_device_alpha) into h_evals[4(j+1) .. 4(j+1)+3]. The same words as those calls made
   layer by layer; one block, the layer and the tree level in shared memory. 1 <= n_layers <=
   log_size <= 10. */
cs_status cs_fri_commit_fold_tail(uint32_t *d_state, uint32_t *d_alphas, uint32_t *const *h_evals,
                                  uint32_t *const *h_trees, uint32_t log_size, uint32_t n_layers,
                                  const uint32_t *d_itwiddles, uint32_t twiddle_log_size, cs_stream stream);

/* ------------------------------------------------------- measurement */

/* Integer-pipe throughput probe (no counterpart in the reference): `blocks` x
   256 threads each run 8 independent chains of `iters` operations of one kind
   (0: 3-input add, 1: 3-input logic, 2: funnel shift, 3: multiply-add) and
   write one word per thread to d_out (blocks x 256 words). The caller times
   the launch; ops = blocks x 256 x 8 x iters. The measured denominator for
   the integer-bound kernels (FFT butterflies, Blake2s). */
cs_status cs_int_peak_probe(uint32_t kind, uint32_t blocks, uint32_t iters, uint32_t *d_out, cs_stream stream);

/* ------------------------------------------------------- decommitment */

/* Batched reads for decommitment. Replaces the element-wise Column::at reads
   of MerkleProverLifted::decommit (crates/stwo/src/prover/vcs_lifted/prover.rs:97-162)
   and compute_decommitment_positions_and_witness_evals
   (crates/stwo/src/prover/fri.rs:408-438): h_out[k] = h_table[h_slot[k]][h_index[k]]
   for k < n, where h_table holds n_table device pointers to u32 words (column
   data, or Merkle layers as 8 words per digest) of h_lengths[t] words each.
   Every slot and index is checked on the host (CS_ERR_INVALID_ARG, nothing
   read). One upload, one launch, one copy back; synchronous on `stream`. */
cs_status cs_gather_u32(const uint32_t *const *h_table, const uint64_t *h_lengths, uint32_t n_table,
                        const uint32_t *h_slot, const uint32_t *h_index, uint32_t n, uint32_t *h_out,
                        cs_stream stream);

/* -------------------------------------------------------- proof of work */

/* GrindOps<Blake2sChannel>::grind (crates/stwo/src/core/proof_of_work.rs:10-14;
   SIMD crates/stwo/src/prover/backend/simd/grind.rs:36-62): the smallest nonce
   with trailing_zeros(Blake2s(Blake2s(0x12345678_le || digest || bits_le) ||
   nonce_le64)) >= pow_bits, pow_bits <= 32. Synchronous on `stream`: *nonce_out
   is valid on return. Allocates an 8-byte device slot per call (stream-ordered).
   Gives CS_ERR_TIMEOUT when no nonce below max_nonce qualifies. */
cs_status cs_grind_blake2s(const uint8_t digest[32], uint32_t pow_bits, uint64_t max_nonce, uint64_t *nonce_out,
                           cs_stream stream);

/* Allocation-free proof-of-work search. It has no counterpart in the
   reference. It is for callers that cannot allocate device memory: a prover
   embedded in a service that carves all device memory into a fixed arena up
   front, or code that must not add allocation calls to a stream it does not
   own. It gives the same nonces as cs_grind_blake2s, one per digest
   (digests: n_digests x 32 bytes, nonces_out: n_digests values), but keeps
   its best-nonce slots in a static device array of 64 slots (512 bytes,
   resident on every GPU that loads this library until the process exits)
   instead of allocating, so n_digests above 64 is rejected with
   CS_ERR_INVALID_ARG. The first call on a device, with that device current,
   looks up the array's device address; make that call before any stream
   capture. That address stays cached for the life of the process; a
   cudaDeviceReset unloads the module and leaves it stale, so a process
   that resets a device must not call this entry point on it afterwards.
   Calls share the array: calls that overlap on the GPU race.
   Synchronous on `stream`. */
cs_status cs_grind_blake2s_noalloc(const uint8_t *digests, uint32_t n_digests, uint32_t pow_bits, uint64_t max_nonce,
                                   uint64_t *nonces_out, cs_stream stream);

#ifdef __cplusplus
}
#endif

#endif /* STWO_CUDA_H */
