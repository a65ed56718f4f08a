/*
 * ORACLE — test infrastructure only. CPU restatement of the reference's
 * CpuBackend for the prover hot path: twiddle trees, circle FFT, lifted
 * Blake2s Merkle, FRI folds, the Blake2s channel and proof-of-work.
 * Only tests/, the smoke check and bench.py's CPU baseline call it, as the
 * checker; the product never does.
 *
 * Parity is pinned by the reference's known-answer tests (tests/golden/) and
 * by its structural tests restated in tests/test_oracle_*.py.
 */
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "fields.h"
#include "circle.h"
#include "blake2s.h"
#include "oracle.h"

/* The OpenMP thread count of the calling process's parallel regions (a launcher such as
   torch.distributed.run sets OMP_NUM_THREADS=1 per rank; a rank that times the CPU baseline alone
   raises it back to the host's cores). */
void orc_set_num_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------ misc */

void orc_bit_reverse(uint32_t *v, uint32_t log_n) {
    /* crates/stwo/src/core/utils.rs:118-128 */
    uint64_t n = 1ull << log_n;
    for (uint64_t i = 0; i < n; i++) {
        uint64_t j = bit_reverse_index((uint32_t)i, log_n);
        if (j > i) { uint32_t t = v[i]; v[i] = v[j]; v[j] = t; }
    }
}

void orc_circle_index_to_point(uint32_t idx, uint32_t out[2]) {
    cpoint p = cidx_to_point(idx & CIRCLE_INDEX_MASK);
    out[0] = p.x; out[1] = p.y;
}

void orc_m31_mul_batch(const uint32_t *a, const uint32_t *b, uint32_t *out, uint64_t n) {
    for (uint64_t i = 0; i < n; i++) out[i] = m31_mul(a[i], b[i]);
}

void orc_qm31_mul(const uint32_t a[4], const uint32_t b[4], uint32_t out[4]) {
    qm31_to_words(qm31_mul(qm31_from_words(a), qm31_from_words(b)), out);
}

void orc_qm31_inv(const uint32_t a[4], uint32_t out[4]) {
    qm31_to_words(qm31_inv(qm31_from_words(a)), out);
}

/* -------------------------------------------------------------- twiddles */

/*
 * slow_precompute_twiddles (crates/stwo/src/prover/backend/cpu/circle.rs:274-285):
 * per doubling of the coset, the x-coordinates of its first half, bit-reversed,
 * concatenated, then one pad element = 1. Length 2^log_size.
 * itwiddles are the field inverses (circle.rs:240-264).
 */
void orc_precompute_twiddles(uint32_t initial_index, uint32_t log_size, uint32_t *tw, uint32_t *itw) {
    coset_t c = coset_new(initial_index, log_size);
    uint64_t off = 0;
    for (uint32_t layer = 0; layer < log_size; layer++) {
        uint64_t half = (1ull << c.log_size) / 2;
        cpoint p = c.initial;
        for (uint64_t i = 0; i < half; i++) {
            tw[off + i] = p.x;
            p = cpoint_add(p, c.step);
        }
        orc_bit_reverse(tw + off, c.log_size - 1);
        off += half;
        c = coset_double(c);
    }
    tw[off] = 1;
    if (itw) {
        uint64_t n = 1ull << log_size;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < (int64_t)n; i++) itw[i] = m31_inv(tw[i]);
    }
}

/* -------------------------------------------------------------- circle FFT */

static inline void butterfly(m31 *v0, m31 *v1, m31 t) {
    /* crates/stwo/src/core/fft.rs:5-12 */
    m31 tmp = m31_mul(*v1, t);
    *v1 = m31_sub(*v0, tmp);
    *v0 = m31_add(*v0, tmp);
}
static inline void ibutterfly(m31 *v0, m31 *v1, m31 t) {
    /* crates/stwo/src/core/fft.rs:14-21 */
    m31 tmp = *v0;
    *v0 = m31_add(tmp, *v1);
    *v1 = m31_mul(m31_sub(tmp, *v1), t);
}

/*
 * domain_line_twiddles_from_tree (crates/stwo/src/core/poly/utils.rs:98-111):
 * for a domain whose half coset has log size D, line layer j (FFT layer j+1)
 * uses buf[len - 2^(D-j) .. len - 2^(D-1-j)).
 */
static const uint32_t *line_layer(const uint32_t *buf, uint64_t buf_len, uint32_t domain_log, uint32_t fft_layer) {
    uint32_t D = domain_log - 1;
    uint32_t j = fft_layer - 1;
    return buf + (buf_len - (1ull << (D - j)));
}

/* circle_twiddles_from_line_twiddles (cpu/circle.rs:306-323): [x, y] -> [y, -y, -x, x]. */
static inline m31 circle_twiddle(const uint32_t *lt1, uint64_t h) {
    m31 x = lt1[(h >> 2) * 2], y = lt1[(h >> 2) * 2 + 1];
    switch (h & 3) {
        case 0: return y;
        case 1: return m31_neg(y);
        case 2: return m31_neg(x);
        default: return x;
    }
}

/* fft_layer_loop (cpu/circle.rs:287-301). */
static void layer_loop(uint32_t *v, uint32_t i, uint64_t h, m31 t, int inverse) {
    uint64_t base = h << (i + 1), stride = 1ull << i;
    for (uint64_t l = 0; l < stride; l++) {
        if (inverse) ibutterfly(&v[base + l], &v[base + l + stride], t);
        else butterfly(&v[base + l], &v[base + l + stride], t);
    }
}

/*
 * PolyOps::interpolate for CpuBackend (cpu/circle.rs:26-79) on the canonic
 * circle domain of log size log_n; values are bit-reversed evaluations and
 * become coefficients in place. itw is the itwiddle buffer of a tree whose
 * root coset is a canonic half coset of log >= log_n - 1.
 */
void orc_interpolate(uint32_t *v, uint32_t log_n, const uint32_t *itw, uint32_t tw_log) {
    orc_interpolate_on(v, log_n, itw, tw_log, canonic_half_coset(log_n).initial_index);
}

/* interpolate on a circle domain whose half coset starts at half_initial_index: a canonic domain,
   or a subdomain (bit-reversed prefix) of one, e.g. CanonicCoset(L).split(b).0 in
   compute_quotients_and_combine. Domains of log size 1 and 2 use that first point directly, as
   the CPU backend does with eval.domain.half_coset.initial (cpu/circle.rs:34-58); larger ones read
   the twiddle tree, which carries the domain. */
void orc_interpolate_on(uint32_t *v, uint32_t log_n, const uint32_t *itw, uint32_t tw_log,
                        uint32_t half_initial_index) {
    coset_t half = coset_new(half_initial_index, log_n - 1);
    uint64_t n = 1ull << log_n;
    if (log_n == 1) {
        m31 y = half.initial.y, nn = 2;
        m31 yn_inv = m31_inv(m31_mul(y, nn));
        m31 y_inv = m31_mul(yn_inv, nn), n_inv = m31_mul(yn_inv, y);
        ibutterfly(&v[0], &v[1], y_inv);
        v[0] = m31_mul(v[0], n_inv); v[1] = m31_mul(v[1], n_inv);
        return;
    }
    if (log_n == 2) {
        m31 x = half.initial.x, y = half.initial.y, nn = 4;
        m31 xyn_inv = m31_inv(m31_mul(m31_mul(x, y), nn));
        m31 x_inv = m31_mul(m31_mul(xyn_inv, y), nn);
        m31 y_inv = m31_mul(m31_mul(xyn_inv, x), nn);
        m31 n_inv = m31_mul(m31_mul(xyn_inv, x), y);
        ibutterfly(&v[0], &v[1], y_inv);
        ibutterfly(&v[2], &v[3], m31_neg(y_inv));
        ibutterfly(&v[0], &v[2], x_inv);
        ibutterfly(&v[1], &v[3], x_inv);
        for (int k = 0; k < 4; k++) v[k] = m31_mul(v[k], n_inv);
        return;
    }
    uint64_t buf_len = 1ull << tw_log;
    const uint32_t *lt1 = line_layer(itw, buf_len, log_n, 1);
    for (uint64_t h = 0; h < n / 2; h++) layer_loop(v, 0, h, circle_twiddle(lt1, h), 1);
    for (uint32_t i = 1; i < log_n; i++) {
        const uint32_t *lt = line_layer(itw, buf_len, log_n, i);
        for (uint64_t h = 0; h < (n >> (i + 1)); h++) layer_loop(v, i, h, lt[h], 1);
    }
    m31 inv = m31_inv((m31)(n % M31_P));
    for (uint64_t k = 0; k < n; k++) v[k] = m31_mul(v[k], inv);
}

/*
 * PolyOps::evaluate_into for CpuBackend (cpu/circle.rs:187-238): zero-pad the
 * coefficients to the canonic domain of log size log_n and run the FFT.
 */
void orc_evaluate(const uint32_t *coeffs, uint32_t log_coeffs, uint32_t *out, uint32_t log_n,
                  const uint32_t *tw, uint32_t tw_log) {
    uint64_t n = 1ull << log_n, nc = 1ull << log_coeffs;
    memcpy(out, coeffs, nc * 4);
    memset(out + nc, 0, (n - nc) * 4);
    coset_t half = canonic_half_coset(log_n);
    if (log_n == 1) {
        butterfly(&out[0], &out[1], half.initial.y);
        return;
    }
    if (log_n == 2) {
        m31 x = half.initial.x, y = half.initial.y;
        butterfly(&out[0], &out[2], x);
        butterfly(&out[1], &out[3], x);
        butterfly(&out[0], &out[1], y);
        butterfly(&out[2], &out[3], m31_neg(y));
        return;
    }
    uint64_t buf_len = 1ull << tw_log;
    for (uint32_t i = log_n - 1; i >= 1; i--) {
        const uint32_t *lt = line_layer(tw, buf_len, log_n, i);
        for (uint64_t h = 0; h < (n >> (i + 1)); h++) layer_loop(out, i, h, lt[h], 0);
    }
    const uint32_t *lt1 = line_layer(tw, buf_len, log_n, 1);
    for (uint64_t h = 0; h < n / 2; h++) layer_loop(out, 0, h, circle_twiddle(lt1, h), 0);
}

void orc_interpolate_batch(uint32_t **cols, const uint32_t *log_sizes, uint32_t n_cols,
                           const uint32_t *itw, uint32_t tw_log) {
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t c = 0; c < (int64_t)n_cols; c++) orc_interpolate(cols[c], log_sizes[c], itw, tw_log);
}

void orc_evaluate_batch(const uint32_t **coeffs, const uint32_t *log_coeffs, uint32_t **outs,
                        const uint32_t *log_ns, uint32_t n_cols, const uint32_t *tw, uint32_t tw_log) {
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t c = 0; c < (int64_t)n_cols; c++)
        orc_evaluate(coeffs[c], log_coeffs[c], outs[c], log_ns[c], tw, tw_log);
}

/*
 * CircleCoefficients::eval_at_point (cpu/circle.rs:81-98) using
 * fold (crates/stwo/src/core/poly/utils.rs:27-38): mappings [.., pi(x), x, y]
 * reversed. Evaluated iteratively from the leaves of the fold tree.
 */
void orc_eval_at_point(const uint32_t *coeffs, uint32_t log_n, const uint32_t px[4], const uint32_t py[4],
                       uint32_t out[4]) {
    if (log_n == 0) { out[0] = coeffs[0]; out[1] = out[2] = out[3] = 0; return; }
    /* folding factors in order: factors[0] = top-level (last mapping). */
    qm31 *mapping = (qm31 *)malloc(sizeof(qm31) * log_n);
    qm31 x = qm31_from_words(px);
    mapping[0] = qm31_from_words(py);
    for (uint32_t k = 1; k < log_n; k++) { mapping[k] = x; x = qcircle_double_x(x); }
    /* fold(values, factors) with factors = reverse(mapping): factor for tree level
       d (d=0 top) is mapping[log_n-1-d]. Bottom level (pairs) uses mapping[0]. */
    uint64_t n = 1ull << log_n;
    qm31 *acc = (qm31 *)malloc(sizeof(qm31) * (n / 2));
    for (uint64_t i = 0; i < n / 2; i++)
        acc[i] = qm31_add(qm31_from_m31(coeffs[2 * i]), qm31_mul_m31(mapping[0], coeffs[2 * i + 1]));
    uint64_t m = n / 2;
    for (uint32_t lvl = 1; lvl < log_n; lvl++) {
        for (uint64_t i = 0; i < m / 2; i++) acc[i] = qm31_add(acc[2 * i], qm31_mul(acc[2 * i + 1], mapping[lvl]));
        m /= 2;
    }
    qm31_to_words(acc[0], out);
    free(acc);
    free(mapping);
}

/* ------------------------------------------------------------ lifted Merkle */

/*
 * MerkleOpsLifted::build_leaves (crates/stwo/src/prover/backend/cpu/merkle_lifted.rs:46-90).
 * Columns are sorted by increasing length. Leaf i of a tree of height
 * lifting_log_size absorbs, column by column, the LE bytes of
 * col[(i >> (L - l + 1) << 1) + (i & 1)] for a column of log size l; the
 * reference builds the same byte stream by cloning hasher states from the
 * previous size group (merkle_lifted.rs:57-59,83-88), and its decommit reads
 * the same index (crates/stwo/src/prover/vcs_lifted/prover.rs:114).
 */
void orc_merkle_build_leaves(const uint32_t **cols, const uint32_t *log_sizes, uint32_t n_cols,
                             uint32_t lifting_log_size, uint8_t *out) {
    if (n_cols == 0) { b2s_hash(NULL, 0, out); return; }
    uint64_t n_leaves = 1ull << lifting_log_size;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n_leaves; i++) {
        b2s_state s;
        b2s_init(&s);
        for (uint32_t c = 0; c < n_cols; c++) {
            uint32_t l = log_sizes[c];
            uint64_t idx = (((uint64_t)i >> (lifting_log_size - l + 1)) << 1) + ((uint64_t)i & 1);
            b2s_update_u32(&s, cols[c][idx]);
        }
        b2s_final(&s, out + 32 * i);
    }
}

/* build_next_layer (merkle_lifted.rs:92-97) with hash_children
   (crates/stwo/src/core/vcs_lifted/blake2_merkle.rs:29-36). */
void orc_merkle_build_next_layer(const uint8_t *prev, uint32_t out_log_size, uint8_t *out) {
    uint64_t n = 1ull << out_log_size;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; i++) b2s_hash(prev + 64 * i, 64, out + 32 * i);
}

/*
 * MerkleProverLifted::commit (crates/stwo/src/prover/vcs_lifted/prover.rs:35-80)
 * without leaf packing: stable sort by length, leaves, then lifting_log_size
 * node layers. layers_out (optional) receives all layers, leaves first, each
 * 32 * 2^k bytes, total 32 * (2^(L+1) - 1) bytes.
 */
void orc_merkle_commit(const uint32_t **cols, const uint32_t *log_sizes, uint32_t n_cols,
                       uint32_t lifting_log_size, uint8_t root[32], uint8_t *layers_out) {
    if (n_cols == 0) { b2s_hash(NULL, 0, root); if (layers_out) memcpy(layers_out, root, 32); return; }
    uint32_t *order = (uint32_t *)malloc(sizeof(uint32_t) * n_cols);
    for (uint32_t i = 0; i < n_cols; i++) order[i] = i;
    /* stable insertion sort by log size */
    for (uint32_t i = 1; i < n_cols; i++) {
        uint32_t k = order[i]; int64_t j = (int64_t)i - 1;
        while (j >= 0 && log_sizes[order[j]] > log_sizes[k]) { order[j + 1] = order[j]; j--; }
        order[j + 1] = k;
    }
    const uint32_t **sc = (const uint32_t **)malloc(sizeof(void *) * n_cols);
    uint32_t *sl = (uint32_t *)malloc(sizeof(uint32_t) * n_cols);
    for (uint32_t i = 0; i < n_cols; i++) { sc[i] = cols[order[i]]; sl[i] = log_sizes[order[i]]; }
    uint64_t total = 0;
    for (uint32_t k = 0; k <= lifting_log_size; k++) total += 1ull << k;
    uint8_t *layers = layers_out ? layers_out : (uint8_t *)malloc(32 * total);
    orc_merkle_build_leaves(sc, sl, n_cols, lifting_log_size, layers);
    uint8_t *cur = layers;
    for (uint32_t k = lifting_log_size; k >= 1; k--) {
        uint8_t *next = cur + 32 * (1ull << k);
        orc_merkle_build_next_layer(cur, k - 1, next);
        cur = next;
    }
    memcpy(root, cur, 32);
    if (!layers_out) free(layers);
    free(sc); free(sl); free(order);
}

/* --------------------------------------------------------------- FRI folds */

static inline void qm31_ibutterfly(qm31 *v0, qm31 *v1, m31 t) {
    qm31 tmp = *v0;
    *v0 = qm31_add(tmp, *v1);
    *v1 = qm31_mul_m31(qm31_sub(tmp, *v1), t);
}

/*
 * fold_line_cpu (crates/stwo/src/prover/backend/cpu/fri.rs:66-91) on the line
 * domain x(coset(initial_index, log_n)); inputs and outputs are SoA QM31
 * columns (4 coordinate arrays). Output length 2^(log_n - 1).
 */
void orc_fold_line(const uint32_t *const in[4], uint32_t initial_index, uint32_t log_n,
                   const uint32_t alpha_w[4], uint32_t *const out[4]) {
    coset_t dom = coset_new(initial_index, log_n);
    qm31 alpha = qm31_from_words(alpha_w);
    uint64_t half = (1ull << log_n) / 2;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)half; i++) {
        m31 x = coset_at(dom, bit_reverse_index((uint32_t)(i << 1), log_n)).x;
        qm31 f0 = qm31_make(in[0][2 * i], in[1][2 * i], in[2][2 * i], in[3][2 * i]);
        qm31 f1 = qm31_make(in[0][2 * i + 1], in[1][2 * i + 1], in[2][2 * i + 1], in[3][2 * i + 1]);
        qm31_ibutterfly(&f0, &f1, m31_inv(x));
        qm31 r = qm31_add(f0, qm31_mul(alpha, f1));
        uint32_t w[4];
        qm31_to_words(r, w);
        for (int k = 0; k < 4; k++) out[k][i] = w[k];
    }
}

/*
 * fold_circle_into_line_cpu (crates/stwo/src/prover/backend/cpu/fri.rs:94-116)
 * from the canonic circle domain of log size log_n.
 */
void orc_fold_circle_into_line(const uint32_t *const in[4], uint32_t log_n, const uint32_t alpha_w[4],
                               uint32_t *const out[4]) {
    coset_t half_c = canonic_half_coset(log_n);
    qm31 alpha = qm31_from_words(alpha_w);
    uint64_t half = (1ull << log_n) / 2;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)half; i++) {
        cpoint p = domain_at(half_c, bit_reverse_index((uint32_t)(i << 1), log_n));
        qm31 f0 = qm31_make(in[0][2 * i], in[1][2 * i], in[2][2 * i], in[3][2 * i]);
        qm31 f1 = qm31_make(in[0][2 * i + 1], in[1][2 * i + 1], in[2][2 * i + 1], in[3][2 * i + 1]);
        qm31_ibutterfly(&f0, &f1, m31_inv(p.y));
        qm31 r = qm31_add(qm31_mul(alpha, f1), f0);
        uint32_t w[4];
        qm31_to_words(r, w);
        for (int k = 0; k < 4; k++) out[k][i] = w[k];
    }
}

/* -------------------------------------------------------- Blake2s channel */

void orc_blake2s(const uint8_t *data, uint64_t len, uint8_t out[32]) { b2s_hash(data, len, out); }

/* Blake2sChannel (crates/stwo/src/core/channel/blake2s.rs:16-118). */
void orc_channel_mix_u32s(orc_channel *ch, const uint32_t *data, uint32_t n) {
    b2s_state s;
    b2s_init(&s);
    b2s_update(&s, ch->digest, 32);
    for (uint32_t i = 0; i < n; i++) b2s_update_u32(&s, data[i]);
    b2s_final(&s, ch->digest);
    ch->n_draws = 0;
}

void orc_channel_mix_u64(orc_channel *ch, uint64_t v) {
    uint32_t w[2] = {(uint32_t)v, (uint32_t)(v >> 32)};
    orc_channel_mix_u32s(ch, w, 2);
}

void orc_channel_mix_felts(orc_channel *ch, const uint32_t *felts, uint32_t n_felts) {
    /* QM31 felts as 4 LE u32 words each (blake2s.rs:42-53) */
    orc_channel_mix_u32s(ch, felts, 4 * n_felts);
}

void orc_channel_mix_root(orc_channel *ch, const uint8_t root[32]) {
    /* Blake2sMerkleChannel::mix_hash (crates/stwo/src/core/vcs_lifted/blake2_merkle.rs:56-58) */
    b2s_state s;
    b2s_init(&s);
    b2s_update(&s, ch->digest, 32);
    b2s_update(&s, root, 32);
    b2s_final(&s, ch->digest);
    ch->n_draws = 0;
}

void orc_channel_draw_u32s(orc_channel *ch, uint32_t out[8]) {
    uint8_t in[37], h[32];
    memcpy(in, ch->digest, 32);
    in[32] = (uint8_t)ch->n_draws; in[33] = (uint8_t)(ch->n_draws >> 8);
    in[34] = (uint8_t)(ch->n_draws >> 16); in[35] = (uint8_t)(ch->n_draws >> 24);
    in[36] = 0;
    ch->n_draws++;
    b2s_hash(in, 37, h);
    for (int i = 0; i < 8; i++)
        out[i] = (uint32_t)h[4 * i] | ((uint32_t)h[4 * i + 1] << 8) | ((uint32_t)h[4 * i + 2] << 16) |
                 ((uint32_t)h[4 * i + 3] << 24);
}

void orc_channel_draw_secure_felt(orc_channel *ch, uint32_t out[4]) {
    uint32_t w[8];
    orc_channel_draw_u32s(ch, w);
    m31 f[8];
    for (int i = 0; i < 8; i++) f[i] = m31_reduce64(w[i]);
    for (int i = 0; i < 4; i++) out[i] = m31_add(m31_add(f[2 * i], f[2 * i + 1]), f[2 * i + 1]);
}

/* draw_queries (crates/stwo/src/core/queries.rs:11-28). */
void orc_channel_draw_queries(orc_channel *ch, uint32_t log_domain_size, uint32_t n_queries, uint32_t *out) {
    uint32_t mask = (uint32_t)((1ull << log_domain_size) - 1), k = 0;
    while (k < n_queries) {
        uint32_t w[8];
        orc_channel_draw_u32s(ch, w);
        for (int i = 0; i < 8 && k < n_queries; i++) out[k++] = w[i] & mask;
    }
}

void orc_pow_prefixed_digest(const uint8_t digest[32], uint32_t n_bits, uint8_t out[32]) {
    /* H(POW_PREFIX_le || digest || n_bits_le), blake2s.rs:102-109 */
    b2s_state s;
    b2s_init(&s);
    b2s_update_u32(&s, 0x12345678u);
    b2s_update(&s, digest, 32);
    b2s_update_u32(&s, n_bits);
    b2s_final(&s, out);
}

static uint32_t pow_trailing_zeros(const uint8_t prefixed[32], uint64_t nonce) {
    uint8_t in[40], h[32];
    memcpy(in, prefixed, 32);
    for (int i = 0; i < 8; i++) in[32 + i] = (uint8_t)(nonce >> (8 * i));
    b2s_hash(in, 40, h);
    /* trailing zeros of the low 128 bits, little-endian (blake2s.rs:115) */
    uint32_t tz = 0;
    for (int i = 0; i < 16; i++) {
        if (h[i] == 0) { tz += 8; continue; }
        uint8_t b = h[i];
        while (!(b & 1)) { tz++; b >>= 1; }
        return tz;
    }
    return tz;
}

int orc_verify_pow_nonce(const uint8_t digest[32], uint32_t n_bits, uint64_t nonce) {
    uint8_t pre[32];
    orc_pow_prefixed_digest(digest, n_bits, pre);
    return pow_trailing_zeros(pre, nonce) >= n_bits;
}

/* GrindOps for CpuBackend (crates/stwo/src/prover/backend/cpu/grind.rs:5-15): smallest nonce. */
uint64_t orc_grind(const uint8_t digest[32], uint32_t n_bits) {
    uint8_t pre[32];
    orc_pow_prefixed_digest(digest, n_bits, pre);
    for (uint64_t nonce = 0;; nonce++)
        if (pow_trailing_zeros(pre, nonce) >= n_bits) return nonce;
}
