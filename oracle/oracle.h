/*
 * ORACLE — test infrastructure only: the CPU restatement of the reference
 * prover used as the parity checker by tests/, the smoke check and the CPU
 * baseline in bench.py. The product (proving_gb300, include/) never links it.
 *
 * Arrays of M31 values are uint32_t words in [0, P). QM31 values are 4 words
 * (a, b, c, d) for (a + b i) + (c + d i) u. Hashes are 32 raw bytes.
 */
#ifndef STWO_ORACLE_H
#define STWO_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    uint8_t digest[32];
    uint32_t n_draws;
} orc_channel;

int orc_num_threads(void);
void orc_set_num_threads(int n);
void orc_bit_reverse(uint32_t *v, uint32_t log_n);
void orc_circle_index_to_point(uint32_t idx, uint32_t out[2]);
void orc_m31_mul_batch(const uint32_t *a, const uint32_t *b, uint32_t *out, uint64_t n);
void orc_qm31_mul(const uint32_t a[4], const uint32_t b[4], uint32_t out[4]);
void orc_qm31_inv(const uint32_t a[4], uint32_t out[4]);

void orc_precompute_twiddles(uint32_t initial_index, uint32_t log_size, uint32_t *tw, uint32_t *itw);
void orc_interpolate(uint32_t *v, uint32_t log_n, const uint32_t *itw, uint32_t tw_log);
void orc_interpolate_on(uint32_t *v, uint32_t log_n, const uint32_t *itw, uint32_t tw_log,
                        uint32_t half_initial_index);
void orc_evaluate(const uint32_t *coeffs, uint32_t log_coeffs, uint32_t *out, uint32_t log_n,
                  const uint32_t *tw, uint32_t tw_log);
void orc_interpolate_batch(uint32_t **cols, const uint32_t *log_sizes, uint32_t n_cols,
                           const uint32_t *itw, uint32_t tw_log);
void orc_evaluate_batch(const uint32_t **coeffs, const uint32_t *log_coeffs, uint32_t **outs,
                        const uint32_t *log_ns, uint32_t n_cols, const uint32_t *tw, uint32_t tw_log);
void orc_eval_at_point(const uint32_t *coeffs, uint32_t log_n, const uint32_t px[4], const uint32_t py[4],
                       uint32_t out[4]);

void orc_merkle_build_leaves(const uint32_t **cols, const uint32_t *log_sizes, uint32_t n_cols,
                             uint32_t lifting_log_size, uint8_t *out);
void orc_merkle_build_next_layer(const uint8_t *prev, uint32_t out_log_size, uint8_t *out);
void orc_merkle_commit(const uint32_t **cols, const uint32_t *log_sizes, uint32_t n_cols,
                       uint32_t lifting_log_size, uint8_t root[32], uint8_t *layers_out);

void orc_fold_line(const uint32_t *const in[4], uint32_t initial_index, uint32_t log_n,
                   const uint32_t alpha[4], uint32_t *const out[4]);
void orc_fold_circle_into_line(const uint32_t *const in[4], uint32_t log_n, const uint32_t alpha[4],
                               uint32_t *const out[4]);

void orc_blake2s(const uint8_t *data, uint64_t len, uint8_t out[32]);
void orc_channel_mix_u32s(orc_channel *ch, const uint32_t *data, uint32_t n);
void orc_channel_mix_u64(orc_channel *ch, uint64_t v);
void orc_channel_mix_felts(orc_channel *ch, const uint32_t *felts, uint32_t n_felts);
void orc_channel_mix_root(orc_channel *ch, const uint8_t root[32]);
void orc_channel_draw_u32s(orc_channel *ch, uint32_t out[8]);
void orc_channel_draw_secure_felt(orc_channel *ch, uint32_t out[4]);
void orc_channel_draw_queries(orc_channel *ch, uint32_t log_domain_size, uint32_t n_queries, uint32_t *out);
void orc_pow_prefixed_digest(const uint8_t digest[32], uint32_t n_bits, uint8_t out[32]);
int orc_verify_pow_nonce(const uint8_t digest[32], uint32_t n_bits, uint64_t nonce);
uint64_t orc_grind(const uint8_t digest[32], uint32_t n_bits);

/* accumulation, quotients, out-of-domain sampling (oracle_pcs.c) */
void orc_accumulate(uint32_t *const col[4], const uint32_t *const other[4], uint64_t n);
void orc_generate_secure_powers(const uint32_t felt[4], uint32_t n, uint32_t *out);
void orc_lift_and_accumulate(uint32_t *const *cols, const uint32_t *log_sizes, uint32_t n_cols);
void orc_barycentric_weights(uint32_t log_n, const uint32_t px[4], const uint32_t py[4], uint32_t *const out[4]);
void orc_barycentric_eval(const uint32_t *evals, uint32_t log_n, const uint32_t *const weights[4], uint32_t out[4]);
void orc_line_coeffs(const uint32_t py[4], const uint32_t value[4], const uint32_t alpha[4], uint32_t out[12]);
void orc_accumulate_numerators(const uint32_t **cols, uint32_t n_terms, uint32_t log_size, uint32_t log_blowup,
                               const uint32_t *coeffs, uint32_t *const out[4], uint32_t first_linear_out[4]);
void orc_quotients_on_subdomain(const uint32_t *const *accs, const uint32_t *acc_logs, uint32_t n_points,
                                const uint32_t *points, const uint32_t *first_linear, uint32_t lifting_log_size,
                                uint32_t log_blowup, uint32_t *const out[4]);
void orc_decompose(const uint32_t *const in[4], uint32_t log_n, uint32_t *const out[4], uint32_t lambda_out[4]);
void orc_random_point_from_t(const uint32_t t[4], uint32_t px[4], uint32_t py[4]);
void orc_wide_fib_composition(const uint32_t **cols, uint32_t n_cols, uint32_t eval_log, uint32_t trace_log,
                              const uint32_t *rc, uint32_t *const out[4]);
void orc_wide_fib_trace(const uint32_t *a0, const uint32_t *b0, uint32_t log_n, uint32_t n_cols, uint32_t **cols);
void orc_logup_running_sum(const uint32_t *values, uint32_t log_n, const uint32_t z[4], uint32_t *const out[4],
                           uint32_t claimed_out[4]);
void orc_logup_combine(const uint32_t *const *values, uint32_t n_values, uint32_t log_n,
                       const uint32_t *alpha_powers, const uint32_t z[4], uint32_t *const out[4]);
void orc_logup_gen_col(const uint32_t *const num[4], const uint32_t *num_m31, const uint32_t *const den[4],
                       const uint32_t *const prev[4], uint32_t log_n, uint32_t *const out[4]);
void orc_logup_finalize_last(uint32_t *const col[4], uint32_t log_n, uint32_t claimed_out[4]);
uint64_t orc_offset_row(uint64_t r, int64_t offset, uint32_t trace_log, uint32_t eval_log);
uint64_t orc_prev_row(uint64_t r, uint32_t trace_log, uint32_t eval_log);
void orc_offset_rows(int64_t offset, uint32_t trace_log, uint32_t eval_log, uint64_t *out);
void orc_prev_rows(uint32_t trace_log, uint32_t eval_log, uint64_t *out);
void orc_logup_composition(const uint32_t *values, const uint32_t *const inter[4], uint32_t eval_log,
                           uint32_t trace_log, const uint32_t z[4], const uint32_t claimed[4], const uint32_t rc[4],
                           uint32_t *const out[4]);
void orc_poseidon_m4(uint32_t x[4]);
void orc_poseidon_external(uint32_t s[16]);
void orc_poseidon_internal(uint32_t s[16]);
void orc_poseidon_trace(uint32_t log_n, uint32_t **cols);
void orc_poseidon_interaction(const uint32_t **trace, uint32_t log_n, const uint32_t z[4], const uint32_t alpha[4],
                              uint32_t **out, uint32_t claimed_out[4]);
void orc_poseidon_composition(const uint32_t **trace, const uint32_t **inter, uint32_t eval_log, uint32_t trace_log,
                              const uint32_t lookup[8], const uint32_t claimed[4], const uint32_t *rc,
                              uint32_t *const out[4]);

/* whole proofs (oracle_prover.c): the reference's prove_ex flow restated over the ops above.
   fri = {pow_bits, log_blowup_factor, log_last_layer_degree_bound, n_queries, fold_step}.
   Return 0 on success, 1 when the sanity check fails (ConstraintsNotSatisfied), 2 when the last
   FRI layer is not of low degree, -1 for unsupported arguments, -2 when the words do not fit
   (*n_words is still set). */
int orc_prove_fib_and_lookups(const uint32_t fri[5], uint32_t n_fib, const uint32_t *fib_n_cols,
                              const uint32_t *fib_log_sizes, const uint32_t *const *fib_trace,
                              uint32_t n_lookups, const uint32_t *lookup_log_sizes,
                              const uint32_t *const *lookup_values, int check, uint32_t *claimed_out,
                              uint64_t *words, size_t capacity, size_t *n_words);
int orc_prove_poseidon(const uint32_t fri[5], uint32_t log_n_rows, uint64_t *words, size_t capacity,
                       size_t *n_words);

#ifdef __cplusplus
}
#endif

#endif
