// The host side of the Wide-Fibonacci prover in native code: the generic
// prover's loop (prove_ex, crates/stwo/src/prover/mod.rs:39-138), the
// commitment scheme (crates/stwo/src/prover/pcs/mod.rs:83-398), the FRI prover
// (crates/stwo/src/prover/fri.rs:113-438) and the proof's felt stream
// (CairoSerialize, crates/cairo-serialize/src/serialize.rs:99-210), driving
// this library's kernels through its own C ABI. It produces the bytes of
// proving_gb300.prover.prove_wide_fib_components without a Python interpreter
// between the launches: the host work between synchronisation points is a few
// microseconds instead of milliseconds.
#include <algorithm>
#include <cstring>
#include <map>
#include <vector>

#include "common.cuh"
#include "field.cuh"

namespace cs {
namespace hp {
namespace {

// ---------------------------------------------------------------- Blake2s-256 (RFC 7693), host

const uint32_t kIV[8] = {0x6a09e667u, 0xbb67ae85u, 0x3c6ef372u, 0xa54ff53au,
                         0x510e527fu, 0x9b05688cu, 0x1f83d9abu, 0x5be0cd19u};
const uint8_t kSigma[10][16] = {
    {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15}, {14, 10, 4, 8, 9, 15, 13, 6, 1, 12, 0, 2, 11, 7, 5, 3},
    {11, 8, 12, 0, 5, 2, 15, 13, 10, 14, 3, 6, 7, 1, 9, 4}, {7, 9, 3, 1, 13, 12, 11, 14, 2, 6, 5, 10, 4, 0, 15, 8},
    {9, 0, 5, 7, 2, 4, 10, 15, 14, 1, 11, 12, 6, 8, 3, 13}, {2, 12, 6, 10, 0, 11, 8, 3, 4, 13, 7, 5, 15, 14, 1, 9},
    {12, 5, 1, 15, 14, 13, 4, 10, 0, 7, 6, 3, 9, 2, 8, 11}, {13, 11, 7, 14, 12, 1, 3, 9, 5, 0, 15, 4, 8, 6, 2, 10},
    {6, 15, 14, 9, 11, 3, 0, 8, 12, 2, 13, 7, 1, 4, 10, 5}, {10, 2, 8, 4, 7, 6, 1, 5, 15, 11, 9, 14, 3, 12, 13, 0}};

inline uint32_t rotr(uint32_t x, int n) { return (x >> n) | (x << (32 - n)); }

void compress(uint32_t h[8], const uint8_t block[64], uint64_t t, bool last) {
  uint32_t m[16], v[16];
  for (int i = 0; i < 16; i++)
    m[i] = (uint32_t)block[4 * i] | ((uint32_t)block[4 * i + 1] << 8) | ((uint32_t)block[4 * i + 2] << 16) |
           ((uint32_t)block[4 * i + 3] << 24);
  for (int i = 0; i < 8; i++) {
    v[i] = h[i];
    v[i + 8] = kIV[i];
  }
  v[12] ^= (uint32_t)t;
  v[13] ^= (uint32_t)(t >> 32);
  if (last) v[14] = ~v[14];
  const auto g = [&](int a, int b, int c, int d, uint32_t x, uint32_t y) {
    v[a] = v[a] + v[b] + x;
    v[d] = rotr(v[d] ^ v[a], 16);
    v[c] = v[c] + v[d];
    v[b] = rotr(v[b] ^ v[c], 12);
    v[a] = v[a] + v[b] + y;
    v[d] = rotr(v[d] ^ v[a], 8);
    v[c] = v[c] + v[d];
    v[b] = rotr(v[b] ^ v[c], 7);
  };
  for (int r = 0; r < 10; r++) {
    const uint8_t* s = kSigma[r];
    g(0, 4, 8, 12, m[s[0]], m[s[1]]);
    g(1, 5, 9, 13, m[s[2]], m[s[3]]);
    g(2, 6, 10, 14, m[s[4]], m[s[5]]);
    g(3, 7, 11, 15, m[s[6]], m[s[7]]);
    g(0, 5, 10, 15, m[s[8]], m[s[9]]);
    g(1, 6, 11, 12, m[s[10]], m[s[11]]);
    g(2, 7, 8, 13, m[s[12]], m[s[13]]);
    g(3, 4, 9, 14, m[s[14]], m[s[15]]);
  }
  for (int i = 0; i < 8; i++) h[i] ^= v[i] ^ v[i + 8];
}

// Blake2s-256 of a message (no key).
void blake2s(const uint8_t* msg, size_t n, uint8_t out[32]) {
  uint32_t h[8];
  for (int i = 0; i < 8; i++) h[i] = kIV[i];
  h[0] ^= 0x01010000u ^ 32u;
  uint8_t block[64];
  size_t off = 0;
  while (n - off > 64) {
    compress(h, msg + off, off + 64, false);
    off += 64;
  }
  std::memset(block, 0, 64);
  if (n > off) std::memcpy(block, msg + off, n - off);
  compress(h, block, n, true);
  for (int i = 0; i < 8; i++)
    for (int b = 0; b < 4; b++) out[4 * i + b] = (uint8_t)(h[i] >> (8 * b));
}

// ---------------------------------------------------------------- channel

// Blake2sChannel (crates/stwo/src/core/channel/blake2s.rs:16-118).
struct Channel {
  uint8_t digest[32] = {0};
  uint32_t n_draws = 0;

  void set(const uint8_t d[32]) {
    std::memcpy(digest, d, 32);
    n_draws = 0;
  }
  void mix_bytes(const std::vector<uint8_t>& data) {
    std::vector<uint8_t> msg(digest, digest + 32);
    msg.insert(msg.end(), data.begin(), data.end());
    uint8_t d[32];
    blake2s(msg.data(), msg.size(), d);
    set(d);
  }
  void mix_u32s(const std::vector<uint32_t>& w) {
    std::vector<uint8_t> b(4 * w.size());
    for (size_t i = 0; i < w.size(); i++)
      for (int k = 0; k < 4; k++) b[4 * i + k] = (uint8_t)(w[i] >> (8 * k));
    mix_bytes(b);
  }
  void mix_u64(uint64_t v) { mix_u32s({(uint32_t)v, (uint32_t)(v >> 32)}); }
  void mix_felts(const std::vector<qm31>& f) {
    std::vector<uint32_t> w;
    for (const qm31& x : f) {
      w.push_back(x.a.a);
      w.push_back(x.a.b);
      w.push_back(x.b.a);
      w.push_back(x.b.b);
    }
    mix_u32s(w);
  }
  // Blake2sMerkleChannel::mix_hash (crates/stwo/src/core/vcs_lifted/blake2_merkle.rs:56-58)
  void mix_root(const uint8_t root[32]) { mix_bytes(std::vector<uint8_t>(root, root + 32)); }
  void draw_u32s(uint32_t out[8]) {
    uint8_t msg[37];
    std::memcpy(msg, digest, 32);
    for (int k = 0; k < 4; k++) msg[32 + k] = (uint8_t)(n_draws >> (8 * k));
    msg[36] = 0;
    uint8_t h[32];
    blake2s(msg, 37, h);
    n_draws++;
    for (int i = 0; i < 8; i++)
      out[i] = (uint32_t)h[4 * i] | ((uint32_t)h[4 * i + 1] << 8) | ((uint32_t)h[4 * i + 2] << 16) |
               ((uint32_t)h[4 * i + 3] << 24);
  }
  qm31 draw_secure_felt() {
    uint32_t w[8];
    draw_u32s(w);
    uint32_t c[4];
    for (int i = 0; i < 4; i++) c[i] = (uint32_t)(((uint64_t)(w[2 * i] % P) + 2ull * (w[2 * i + 1] % P)) % P);
    return qm31_make(c[0], c[1], c[2], c[3]);
  }
  // draw_queries (crates/stwo/src/core/queries.rs:11-28)
  std::vector<uint32_t> draw_queries(uint32_t log_size, uint32_t n) {
    std::vector<uint32_t> out;
    const uint32_t mask = (1u << log_size) - 1;
    while (out.size() < n) {
      uint32_t w[8];
      draw_u32s(w);
      for (int i = 0; i < 8 && out.size() < n; i++) out.push_back(w[i] & mask);
    }
    return out;
  }
};

// ---------------------------------------------------------------- points

struct qpoint {
  qm31 x, y;
};

qm31 q1() { return qm31_make(1, 0, 0, 0); }
qm31 qm(uint32_t a) { return qm31_make(a, 0, 0, 0); }

qm31 q_double_x(const qm31& x) {
  const qm31 s = qm31_mul(x, x);
  return qm31_sub(qm31_add(s, s), q1());
}
qpoint q_double(const qpoint& p) { return {q_double_x(p.x), qm31_mul(qm(2), qm31_mul(p.x, p.y))}; }

// CirclePoint::get_random_point (crates/stwo/src/core/circle.rs:150-160)
qpoint random_point(const qm31& t) {
  const qm31 t2 = qm31_mul(t, t);
  const qm31 inv = qm31_inv(qm31_add(t2, q1()));
  return {qm31_mul(qm31_sub(q1(), t2), inv), qm31_mul(qm31_add(t, t), inv)};
}

cpoint index_to_point(uint32_t idx) {
  cpoint r{1, 0}, cur{2u, 1268011823u};
  idx &= 0x7fffffffu;
  while (idx) {
    if (idx & 1) r = cpoint_add(r, cur);
    cur = cpoint_add(cur, cur);
    idx >>= 1;
  }
  return r;
}

uint32_t bitrev(uint32_t i, uint32_t log) {
  uint32_t r = 0;
  for (uint32_t b = 0; b < log; b++) r |= ((i >> b) & 1u) << (log - 1 - b);
  return r;
}

// ---------------------------------------------------------------- device memory of one proof

struct Arena {
  cudaStream_t st;
  std::vector<void*> ptrs;
  cs_status status = CS_OK;
  explicit Arena(cudaStream_t s) : st(s) {}
  uint32_t* alloc(size_t words) {
    void* p = nullptr;
    if (cudaMallocAsync(&p, std::max<size_t>(4, 4 * words), st) != cudaSuccess) {
      status = CS_ERR_OOM;
      return nullptr;
    }
    ptrs.push_back(p);
    return static_cast<uint32_t*>(p);
  }
  ~Arena() {
    for (void* p : ptrs) cudaFreeAsync(p, st);
  }
};

// A lifted Merkle tree: its layer buffer (leaves first, 8 words per digest) and height.
struct Tree {
  uint32_t* layers;
  uint32_t height;
  uint8_t root[32];
  // node i of layer k (2^k nodes): word offset (2^(L+1) - 2^(k+1) + i) * 8
  size_t node_word(uint32_t k, uint64_t i) const { return (((2ull << height) - (2ull << k)) + i) * 8; }
  size_t words() const { return ((2ull << height) - 1) * 8; }
};

#define HP_TRY(call)                  \
  do {                                \
    const cs_status s_ = (call);      \
    if (s_ != CS_OK) return s_;       \
  } while (0)

cs_status commit(Arena& A, const std::vector<uint32_t*>& cols, const std::vector<uint32_t>& logs, uint32_t L,
                 Tree& t) {
  t.height = L;
  t.layers = A.alloc(((2ull << L) - 1) * 8);
  if (t.layers == nullptr) return A.status;
  std::vector<const uint32_t*> c(cols.begin(), cols.end());
  return cs_merkle_commit(c.data(), logs.data(), (uint32_t)cols.size(), L, t.layers, A.st);
}

cs_status read_root(Arena& A, Tree& t) {
  uint32_t w[8];
  CS_CUDA(cudaMemcpyAsync(w, t.layers + t.words() - 8, 32, cudaMemcpyDeviceToHost, A.st));
  CS_CUDA(cudaStreamSynchronize(A.st));
  for (int i = 0; i < 8; i++)
    for (int b = 0; b < 4; b++) t.root[4 * i + b] = (uint8_t)(w[i] >> (8 * b));
  return CS_OK;
}

// The witness of MerkleProverLifted::decommit (crates/stwo/src/prover/vcs_lifted/prover.rs:119-150):
// per layer from the leaves, the sibling of every queried node whose sibling is not queried.
std::vector<std::pair<uint32_t, std::vector<uint64_t>>> witness_nodes(uint32_t height, std::vector<uint64_t> q) {
  std::sort(q.begin(), q.end());
  q.erase(std::unique(q.begin(), q.end()), q.end());
  std::vector<std::pair<uint32_t, std::vector<uint64_t>>> out;
  for (int layer = (int)height - 1; layer >= 0; layer--) {
    std::vector<uint64_t> need;
    for (size_t i = 0; i < q.size(); i++) {
      const uint64_t sib = q[i] ^ 1;
      const bool present = (i + 1 < q.size() && q[i + 1] == sib) || (i > 0 && q[i - 1] == sib);
      if (!present) need.push_back(sib);
    }
    if (!need.empty()) out.push_back({(uint32_t)layer + 1, need});
    std::vector<uint64_t> up;
    for (uint64_t x : q)
      if (up.empty() || up.back() != (x >> 1)) up.push_back(x >> 1);
    q = up;
  }
  return out;
}

// Every device read of a proof's decommitment, collected and made in one cs_gather_u32 call.
struct Reads {
  std::vector<const uint32_t*> table;
  std::vector<uint64_t> lengths;
  std::map<const uint32_t*, uint32_t> slot_of;
  std::vector<uint32_t> slots, index;
  std::vector<uint32_t> out;
  uint32_t slot(const uint32_t* p, uint64_t len) {
    auto it = slot_of.find(p);
    if (it != slot_of.end()) return it->second;
    const uint32_t s = (uint32_t)table.size();
    table.push_back(p);
    lengths.push_back(len);
    slot_of[p] = s;
    return s;
  }
  size_t add(const uint32_t* p, uint64_t len, uint64_t i) {
    slots.push_back(slot(p, len));
    index.push_back((uint32_t)i);
    return slots.size() - 1;
  }
  cs_status run(cudaStream_t st) {
    out.assign(slots.size(), 0);
    if (slots.empty()) return CS_OK;
    return cs_gather_u32(table.data(), lengths.data(), (uint32_t)table.size(), slots.data(), index.data(),
                         (uint32_t)slots.size(), out.data(), st);
  }
};

// A tree's witness digests registered with a Reads: (first read, count of digests).
std::pair<size_t, size_t> read_witness(Reads& R, const Tree& t, const std::vector<uint64_t>& q) {
  size_t first = R.slots.size(), n = 0;
  for (auto& [k, nodes] : witness_nodes(t.height, q))
    for (uint64_t node : nodes) {
      for (int w = 0; w < 8; w++) R.add(t.layers, t.words(), t.node_word(k, node) + w);
      n++;
    }
  return {first, n};
}

// LineEvaluation::interpolate + into_ordered_coefficients (crates/stwo/src/prover/line.rs:54-99) of an
// evaluation on LineDomain(half_odds(log_size)) in bit-reversed order; natural-order coefficients.
std::vector<qm31> line_interpolate(const std::vector<qm31>& values, uint32_t log_size) {
  const uint32_t n = 1u << log_size;
  std::vector<qm31> v(n);
  for (uint32_t i = 0; i < n; i++) v[i] = values[bitrev(i, log_size)];
  uint32_t init = 1u << (31 - (log_size + 2)), step = 1u << (31 - log_size);
  for (uint32_t dom = log_size; dom > 0; dom--) {
    const uint32_t size = 1u << dom;
    for (uint32_t start = 0; start < n; start += size)
      for (uint32_t i = 0; i < size / 2; i++) {
        const uint32_t xinv = m31_inv(index_to_point((init + i * step) & 0x7fffffffu).x);
        const qm31 a = v[start + i], c = v[start + size / 2 + i];
        v[start + i] = qm31_add(a, c);
        v[start + size / 2 + i] = qm31_mul_m31(qm31_sub(a, c), xinv);
      }
    init = (init * 2) & 0x7fffffffu;
    step = (step * 2) & 0x7fffffffu;
  }
  const uint32_t ninv = m31_inv(n % P);
  std::vector<qm31> out(n);
  for (uint32_t i = 0; i < n; i++) out[i] = qm31_mul_m31(v[bitrev(i, log_size)], ninv);
  return out;
}

// complex_conjugate_line_coeffs (crates/stwo/src/core/constraints.rs:119-135) times alpha.
void line_coeffs(const qm31& py, const qm31& v, const qm31& alpha, uint32_t out[12]) {
  const auto conj = [](const qm31& x) { return qm31{x.a, cm31_neg(x.b)}; };
  const qm31 a = qm31_sub(conj(v), v), c = qm31_sub(conj(py), py);
  const qm31 b = qm31_sub(qm31_mul(v, c), qm31_mul(a, py));
  const qm31 r[3] = {qm31_mul(alpha, a), qm31_mul(alpha, b), qm31_mul(alpha, c)};
  for (int k = 0; k < 3; k++) {
    out[4 * k] = r[k].a.a;
    out[4 * k + 1] = r[k].a.b;
    out[4 * k + 2] = r[k].b.a;
    out[4 * k + 3] = r[k].b.b;
  }
}

std::vector<qm31> powers(const qm31& f, uint32_t n) {
  std::vector<qm31> p(n);
  qm31 x = q1();
  for (uint32_t i = 0; i < n; i++) {
    p[i] = x;
    x = qm31_mul(x, f);
  }
  return p;
}

struct Words {
  std::vector<uint64_t> w;
  void u(uint64_t x) { w.push_back(x); }
  void q(const qm31& x) {
    w.push_back(x.a.a);
    w.push_back(x.a.b);
    w.push_back(x.b.a);
    w.push_back(x.b.b);
  }
  void h(const uint8_t d[32]) {
    for (int i = 0; i < 8; i++)
      w.push_back((uint32_t)d[4 * i] | ((uint32_t)d[4 * i + 1] << 8) | ((uint32_t)d[4 * i + 2] << 16) |
                  ((uint32_t)d[4 * i + 3] << 24));
  }
  void hw(const std::vector<uint32_t>& words, size_t first, size_t n) {  // n digests of 8 words
    u(n);
    for (size_t i = 0; i < 8 * n; i++) w.push_back(words[first + i]);
  }
};

struct FriLayer {
  Tree tree;
  std::vector<uint32_t*> eval;  // 4 coordinates
  uint32_t log_size;
};

}  // namespace

void blake2s_public(const uint8_t* msg, size_t n, uint8_t out[32]) { blake2s(msg, n, out); }

cs_status prove_wide_fib(const cs_wide_fib_proof_params& pp, uint32_t* const* d_trace, std::vector<uint64_t>& words,
                         cudaStream_t st) {
  Arena A(st);
  const uint32_t b = pp.log_blowup_factor, L = pp.lifting_log_size;
  const uint32_t n_comp = pp.n_components;
  Channel ch;
  // --- preprocessed tree: empty (a single hash of no data at height 0, pcs/mod.rs:83-96)
  uint8_t pre_root[32];
  blake2s(nullptr, 0, pre_root);
  ch.mix_root(pre_root);
  // --- trace tree: every component's columns (interpolated in place, evaluated on log + b)
  std::vector<uint32_t*> trace_evals;
  std::vector<uint32_t> trace_logs;
  std::vector<std::vector<uint32_t*>> comp_evals(n_comp);
  size_t c0 = 0;
  for (uint32_t k = 0; k < n_comp; k++) {
    const uint32_t n = pp.n_cols[k], lg = pp.log_sizes[k];
    std::vector<uint32_t*> cols(d_trace + c0, d_trace + c0 + n);
    HP_TRY(cs_interpolate_columns(cols.data(), n, lg, pp.d_itwiddles, pp.twiddle_log_size, st));
    uint32_t* block = A.alloc((size_t)n << (lg + b));
    if (!block) return A.status;
    for (uint32_t j = 0; j < n; j++) comp_evals[k].push_back(block + ((size_t)j << (lg + b)));
    std::vector<const uint32_t*> src(cols.begin(), cols.end());
    HP_TRY(cs_evaluate_columns(src.data(), comp_evals[k].data(), n, lg, lg + b, pp.d_twiddles, pp.twiddle_log_size,
                               st));
    for (uint32_t* e : comp_evals[k]) {
      trace_evals.push_back(e);
      trace_logs.push_back(lg + b);
    }
    c0 += n;
  }
  Tree trace_tree;
  HP_TRY(commit(A, trace_evals, trace_logs, L, trace_tree));
  HP_TRY(read_root(A, trace_tree));
  ch.mix_root(trace_tree.root);

  // --- composition (component_prover.rs:95-116): components take the last powers, reversed
  const qm31 random_coeff = ch.draw_secure_felt();
  uint32_t total = 0;
  for (uint32_t k = 0; k < n_comp; k++) total += pp.n_cols[k] - 2;
  const std::vector<qm31> pw = powers(random_coeff, total);
  std::map<uint32_t, std::vector<uint32_t*>> sub_acc;  // eval log -> 4 coordinates
  uint32_t start = 0;
  for (uint32_t k = 0; k < n_comp; k++) {
    const uint32_t n = pp.n_cols[k] - 2, lg = pp.log_sizes[k], el = lg + 1;
    if (!sub_acc.count(el)) {
      uint32_t* blk = A.alloc(4ull << el);
      if (!blk) return A.status;
      CS_CUDA(cudaMemsetAsync(blk, 0, 16ull << el, st));
      sub_acc[el] = {blk, blk + (1ull << el), blk + (2ull << el), blk + (3ull << el)};
    }
    std::vector<uint32_t> rc(4 * n);
    for (uint32_t j = 0; j < n; j++) {  // rc[j] = powers[total - start - 1 - j]
      const qm31 x = pw[total - start - 1 - j];
      rc[4 * j] = x.a.a;
      rc[4 * j + 1] = x.a.b;
      rc[4 * j + 2] = x.b.a;
      rc[4 * j + 3] = x.b.b;
    }
    std::vector<const uint32_t*> ev(comp_evals[k].begin(), comp_evals[k].end());
    HP_TRY(cs_wide_fib_composition(ev.data(), n + 2, el, lg, rc.data(), sub_acc[el].data(), st));
    start += n;
  }
  std::vector<uint32_t*> acc_cols;
  std::vector<uint32_t> acc_logs;
  for (auto& [el, coords] : sub_acc) {
    acc_cols.insert(acc_cols.end(), coords.begin(), coords.end());
    acc_logs.push_back(el);
  }
  if (sub_acc.size() > 1) HP_TRY(cs_lift_and_accumulate(acc_cols.data(), acc_logs.data(), (uint32_t)acc_logs.size(), st));
  const uint32_t comp_log = acc_logs.back();
  std::vector<uint32_t*> accum(acc_cols.end() - 4, acc_cols.end());
  HP_TRY(cs_interpolate_columns(accum.data(), 4, comp_log, pp.d_itwiddles, pp.twiddle_log_size, st));
  const size_t half = 1ull << (comp_log - 1);
  std::vector<const uint32_t*> split;
  for (int c = 0; c < 4; c++) split.push_back(accum[c]);
  for (int c = 0; c < 4; c++) split.push_back(accum[c] + half);
  const uint32_t comp_eval_log = (comp_log - 1) + b;
  uint32_t* cblk = A.alloc(8ull << comp_eval_log);
  if (!cblk) return A.status;
  std::vector<uint32_t*> comp_cols;
  for (int c = 0; c < 8; c++) comp_cols.push_back(cblk + ((size_t)c << comp_eval_log));
  HP_TRY(cs_evaluate_columns(split.data(), comp_cols.data(), 8, comp_log - 1, comp_eval_log, pp.d_twiddles,
                             pp.twiddle_log_size, st));
  Tree comp_tree;
  HP_TRY(commit(A, comp_cols, std::vector<uint32_t>(8, comp_eval_log), L, comp_tree));
  HP_TRY(read_root(A, comp_tree));
  ch.mix_root(comp_tree.root);

  // --- OODS proof of work and point (mod.rs:75-83)
  uint64_t oods_pow = 0;
  HP_TRY(cs_grind_blake2s(ch.digest, 16, 1ull << 48, &oods_pow, st));
  ch.mix_u64(oods_pow);
  const qpoint oods = random_point(ch.draw_secure_felt());

  // --- sampled values (pcs/mod.rs:175-214): every column at the point doubled L - size times; one
  // weight column per size; every value read back once
  std::vector<uint32_t*> all_cols(trace_evals);
  std::vector<uint32_t> all_logs(trace_logs);
  all_cols.insert(all_cols.end(), comp_cols.begin(), comp_cols.end());
  all_logs.insert(all_logs.end(), 8, comp_eval_log);
  const size_t n_all = all_cols.size();
  uint32_t* d_samples = A.alloc(4 * n_all);
  if (!d_samples) return A.status;
  std::map<uint32_t, std::vector<size_t>> by_log;
  for (size_t i = 0; i < n_all; i++) by_log[all_logs[i]].push_back(i);
  std::vector<size_t> order;  // column index of each row of d_samples
  for (auto& [ls, idx] : by_log) {
    qpoint pt = oods;
    for (uint32_t d = ls; d < L; d++) pt = q_double(pt);
    uint32_t* w = A.alloc(4ull << ls);
    if (!w) return A.status;
    uint32_t* wc[4] = {w, w + (1ull << ls), w + (2ull << ls), w + (3ull << ls)};
    const uint32_t px[4] = {pt.x.a.a, pt.x.a.b, pt.x.b.a, pt.x.b.b}, py[4] = {pt.y.a.a, pt.y.a.b, pt.y.b.a, pt.y.b.b};
    HP_TRY(cs_barycentric_weights(ls, px, py, wc, st));
    std::vector<const uint32_t*> cols;
    for (size_t i : idx) cols.push_back(all_cols[i]);
    const uint32_t* wcc[4] = {wc[0], wc[1], wc[2], wc[3]};
    HP_TRY(cs_barycentric_eval(cols.data(), (uint32_t)cols.size(), ls, wcc, d_samples + 4 * order.size(), st));
    order.insert(order.end(), idx.begin(), idx.end());
  }
  std::vector<uint32_t> samples(4 * n_all);
  CS_CUDA(cudaMemcpyAsync(samples.data(), d_samples, 16 * n_all, cudaMemcpyDeviceToHost, st));
  CS_CUDA(cudaStreamSynchronize(st));
  std::vector<qm31> sampled(n_all);
  for (size_t j = 0; j < n_all; j++)
    sampled[order[j]] = qm31_make(samples[4 * j], samples[4 * j + 1], samples[4 * j + 2], samples[4 * j + 3]);
  ch.mix_felts(sampled);

  // --- FRI quotients (quotient_ops.rs:86-160): one sample point; batches by size, ascending
  const qm31 quotient_coeff = ch.draw_secure_felt();
  const std::vector<qm31> qp = powers(quotient_coeff, (uint32_t)n_all);
  std::vector<uint32_t*> parts;
  std::vector<uint32_t> part_logs;
  qm31 first_linear = qm31_make(0, 0, 0, 0);
  for (auto& [ls, idx] : by_log) {
    std::vector<uint32_t> coeffs(12 * idx.size());
    std::vector<const uint32_t*> cols;
    for (size_t j = 0; j < idx.size(); j++) {
      line_coeffs(oods.y, sampled[idx[j]], qp[idx[j]], &coeffs[12 * j]);
      cols.push_back(all_cols[idx[j]]);
    }
    const uint32_t pl = ls - b;
    uint32_t* blk = A.alloc(4ull << pl);
    if (!blk) return A.status;
    uint32_t* out[4] = {blk, blk + (1ull << pl), blk + (2ull << pl), blk + (3ull << pl)};
    uint32_t fl[4];
    HP_TRY(cs_accumulate_numerators(cols.data(), (uint32_t)cols.size(), ls, b, coeffs.data(), out, fl, st));
    first_linear = qm31_add(first_linear, qm31_make(fl[0], fl[1], fl[2], fl[3]));
    parts.insert(parts.end(), out, out + 4);
    part_logs.push_back(pl);
  }
  if (part_logs.size() > 1) HP_TRY(cs_lift_and_accumulate(parts.data(), part_logs.data(), (uint32_t)part_logs.size(), st));
  const uint32_t sub_log = L - b;
  uint32_t* qblk = A.alloc(4ull << sub_log);
  if (!qblk) return A.status;
  uint32_t* qcols[4] = {qblk, qblk + (1ull << sub_log), qblk + (2ull << sub_log), qblk + (3ull << sub_log)};
  const uint32_t* accs[4] = {parts[parts.size() - 4], parts[parts.size() - 3], parts[parts.size() - 2],
                             parts[parts.size() - 1]};
  const uint32_t acc_log = part_logs.back();
  const uint32_t pts[8] = {oods.x.a.a, oods.x.a.b, oods.x.b.a, oods.x.b.b,
                           oods.y.a.a, oods.y.a.b, oods.y.b.a, oods.y.b.b};
  const uint32_t flw[4] = {first_linear.a.a, first_linear.a.b, first_linear.b.a, first_linear.b.b};
  HP_TRY(cs_quotients_on_subdomain(accs, &acc_log, 1, pts, flw, L, b, qcols, st));
  HP_TRY(cs_interpolate_columns_on_subdomain(qcols, 4, sub_log, L, pp.d_itwiddles, pp.twiddle_log_size, st));
  uint32_t* fblk = A.alloc(4ull << L);
  if (!fblk) return A.status;
  std::vector<uint32_t*> quotients = {fblk, fblk + (1ull << L), fblk + (2ull << L), fblk + (3ull << L)};
  const uint32_t* qsrc[4] = {qcols[0], qcols[1], qcols[2], qcols[3]};
  HP_TRY(cs_evaluate_columns(qsrc, quotients.data(), 4, sub_log, L, pp.d_twiddles, pp.twiddle_log_size, st));

  // --- FRI commit (fri.rs:113-226), fold_step 1, the channel kept on the device for the layer loop
  const uint32_t last_log = pp.log_last_layer_degree_bound + b;
  // 9 state words, then (from word 12, 16-byte aligned) room for the 64 challenges of up to 64 layers
  uint32_t* d_state = A.alloc(12 + 4 * 64);
  if (!d_state) return A.status;
  uint32_t state[9];
  std::memcpy(state, ch.digest, 32);
  state[8] = ch.n_draws;
  CS_CUDA(cudaMemcpyAsync(d_state, state, sizeof(state), cudaMemcpyHostToDevice, st));
  uint32_t* d_felts = d_state + 12;  // 16-byte aligned
  uint32_t n_felts = 0;
  std::vector<FriLayer> layers;
  Tree first_tree;
  HP_TRY(commit(A, quotients, std::vector<uint32_t>(4, L), L, first_tree));
  HP_TRY(cs_channel_mix_root(d_state, first_tree.layers + first_tree.words() - 8, st));
  HP_TRY(cs_channel_draw_secure_felt(d_state, d_felts + 4 * n_felts, st));
  std::vector<uint32_t*> cur = quotients;
  uint32_t line_log = L - 1;
  {
    uint32_t* blk = A.alloc(4ull << line_log);
    if (!blk) return A.status;
    std::vector<uint32_t*> nxt = {blk, blk + (1ull << line_log), blk + (2ull << line_log), blk + (3ull << line_log)};
    const uint32_t* src[4] = {cur[0], cur[1], cur[2], cur[3]};
    HP_TRY(cs_fold_circle_into_line_device_alpha(src, L, d_felts + 4 * n_felts, nxt.data(), pp.d_itwiddles,
                                                 pp.twiddle_log_size, st));
    n_felts++;
    cur = nxt;
  }
  while (line_log >= last_log + 1 && n_felts < 64) {  // every layer above the last folds once
    FriLayer lay;
    lay.log_size = line_log;
    lay.eval = cur;
    HP_TRY(commit(A, cur, std::vector<uint32_t>(4, line_log), line_log, lay.tree));
    HP_TRY(cs_channel_mix_root(d_state, lay.tree.layers + lay.tree.words() - 8, st));
    HP_TRY(cs_channel_draw_secure_felt(d_state, d_felts + 4 * n_felts, st));
    const uint32_t nl = line_log - 1;
    uint32_t* blk = A.alloc(4ull << nl);
    if (!blk) return A.status;
    std::vector<uint32_t*> nxt = {blk, blk + (1ull << nl), blk + (2ull << nl), blk + (3ull << nl)};
    const uint32_t* src[4] = {cur[0], cur[1], cur[2], cur[3]};
    HP_TRY(cs_fold_line_device_alpha(src, line_log, d_felts + 4 * n_felts, nxt.data(), pp.d_itwiddles,
                                     pp.twiddle_log_size, st));
    n_felts++;
    layers.push_back(lay);
    cur = nxt;
    line_log = nl;
  }
  // the state, every layer root and the last layer's evaluation back in one read
  std::vector<qm31> last_poly;
  {
    Reads R;
    for (int i = 0; i < 9; i++) R.add(d_state, 9, i);
    std::vector<Tree*> trees = {&first_tree};
    for (FriLayer& l : layers) trees.push_back(&l.tree);
    for (Tree* t : trees)
      for (int i = 0; i < 8; i++) R.add(t->layers, t->words(), t->words() - 8 + i);
    const uint32_t last_n = 1u << last_log;
    for (int c = 0; c < 4; c++)
      for (uint32_t i = 0; i < last_n; i++) R.add(cur[c], last_n, i);
    HP_TRY(R.run(st));
    for (int i = 0; i < 8; i++)
      for (int k = 0; k < 4; k++) ch.digest[4 * i + k] = (uint8_t)(R.out[i] >> (8 * k));
    ch.n_draws = R.out[8];
    size_t o = 9;
    for (Tree* t : trees) {
      for (int i = 0; i < 8; i++)
        for (int k = 0; k < 4; k++) t->root[4 * i + k] = (uint8_t)(R.out[o + i] >> (8 * k));
      o += 8;
    }
    std::vector<qm31> last_values(last_n);
    for (uint32_t i = 0; i < last_n; i++)
      last_values[i] = qm31_make(R.out[o + i], R.out[o + last_n + i], R.out[o + 2 * last_n + i],
                                 R.out[o + 3 * last_n + i]);
    // commit_last_layer (fri.rs:208-226)
    const std::vector<qm31> coeffs = line_interpolate(last_values, last_log);
    const uint32_t bound = 1u << pp.log_last_layer_degree_bound;
    for (uint32_t i = bound; i < last_n; i++)
      CS_CHECK_ARG(coeffs[i].a.a == 0 && coeffs[i].a.b == 0 && coeffs[i].b.a == 0 && coeffs[i].b.b == 0,
                   "prove_wide_fib: invalid degree in the last FRI layer");
    last_poly.resize(bound);
    for (uint32_t i = 0; i < bound; i++) last_poly[i] = coeffs[bitrev(i, pp.log_last_layer_degree_bound)];
    ch.mix_felts(last_poly);
  }

  // --- FRI proof of work and queries (fri.rs:229-283)
  uint64_t fri_pow = 0;
  HP_TRY(cs_grind_blake2s(ch.digest, pp.pow_bits, 1ull << 48, &fri_pow, st));
  ch.mix_u64(fri_pow);
  std::vector<uint32_t> qraw = ch.draw_queries(L, pp.n_queries);
  std::vector<uint64_t> queries(qraw.begin(), qraw.end());
  std::sort(queries.begin(), queries.end());
  queries.erase(std::unique(queries.begin(), queries.end()), queries.end());

  // --- decommitments: every read registered, one gather
  Reads R;
  struct LayerDec {
    std::vector<uint64_t> positions;
    std::vector<bool> is_witness;
    size_t coord_first;
    std::pair<size_t, size_t> wit;
  };
  const auto fri_layer = [&](const std::vector<uint32_t*>& eval, uint32_t log_size, const Tree& t,
                             const std::vector<uint64_t>& q) {
    LayerDec d;
    std::vector<uint64_t> starts;
    for (uint64_t x : q)
      if (starts.empty() || starts.back() != ((x >> 1) << 1)) starts.push_back((x >> 1) << 1);
    for (uint64_t s : starts)
      for (uint64_t j = 0; j < 2; j++) {
        d.positions.push_back(s + j);
        d.is_witness.push_back(!std::binary_search(q.begin(), q.end(), s + j));
      }
    d.coord_first = R.slots.size();
    for (int c = 0; c < 4; c++)
      for (uint64_t p : d.positions) R.add(eval[c], 1ull << log_size, p);
    d.wit = read_witness(R, t, d.positions);
    return d;
  };
  LayerDec first_dec = fri_layer(quotients, L, first_tree, queries);
  std::vector<LayerDec> inner_dec;
  std::vector<uint64_t> lq;
  for (uint64_t x : queries)
    if (lq.empty() || lq.back() != (x >> 1)) lq.push_back(x >> 1);
  for (FriLayer& l : layers) {
    inner_dec.push_back(fri_layer(l.eval, l.log_size, l.tree, lq));
    std::vector<uint64_t> nq;
    for (uint64_t x : lq)
      if (nq.empty() || nq.back() != (x >> 1)) nq.push_back(x >> 1);
    lq = nq;
  }
  // tree decommitments (MerkleProverLifted::decommit): queried values per column, then the witness
  struct TreeDec {
    size_t values_first;
    std::pair<size_t, size_t> wit;
  };
  const auto tree_dec = [&](const Tree& t, const std::vector<uint32_t*>& cols, const std::vector<uint32_t>& logs) {
    TreeDec d;
    d.values_first = R.slots.size();
    for (size_t c = 0; c < cols.size(); c++) {
      const uint32_t shift = t.height - logs[c];
      for (uint64_t q : queries) R.add(cols[c], 1ull << logs[c], ((q >> (shift + 1)) << 1) + (q & 1));
    }
    d.wit = read_witness(R, t, queries);
    return d;
  };
  TreeDec trace_dec = tree_dec(trace_tree, trace_evals, trace_logs);
  TreeDec comp_dec = tree_dec(comp_tree, comp_cols, std::vector<uint32_t>(8, comp_eval_log));
  HP_TRY(R.run(st));

  // --- sanity check (mod.rs:121-132): the composition at the OODS point against the AIR
  {
    const uint32_t mldb = L - b;
    const qm31* cs = sampled.data() + trace_evals.size();
    const auto from_partial_evals = [](const qm31* e) {
      qm31 r = e[0];
      r = qm31_add(r, qm31_mul(e[1], qm31_make(0, 1, 0, 0)));
      r = qm31_add(r, qm31_mul(e[2], qm31_make(0, 0, 1, 0)));
      r = qm31_add(r, qm31_mul(e[3], qm31_make(0, 0, 0, 1)));
      return r;
    };
    const qm31 left = from_partial_evals(cs), right = from_partial_evals(cs + 4);
    qm31 x = oods.x;
    for (uint32_t i = 0; i + 1 < mldb; i++) x = q_double_x(x);
    const qm31 comp = qm31_add(left, qm31_mul(x, right));
    qm31 acc = qm31_make(0, 0, 0, 0);
    size_t s = 0;
    for (uint32_t k = 0; k < n_comp; k++) {
      const qm31* m = sampled.data() + s;
      for (uint32_t j = 0; j + 2 < pp.n_cols[k]; j++) {
        const qm31 cons = qm31_sub(m[j + 2], qm31_add(qm31_mul(m[j], m[j]), qm31_mul(m[j + 1], m[j + 1])));
        acc = qm31_add(qm31_mul(acc, random_coeff), cons);
      }
      s += pp.n_cols[k];
    }
    const qm31 expected = qm31_mul(acc, qm31_inv(x));
    CS_CHECK_ARG(std::memcmp(&comp, &expected, sizeof(qm31)) == 0,
                 "prove_wide_fib: constraints not satisfied (ProvingError::ConstraintsNotSatisfied)");
  }

  // --- the felt stream (CairoSerialize for StarkProof)
  Words W;
  W.u(pp.pow_bits);
  W.u(b);
  W.u(pp.log_last_layer_degree_bound);
  W.u(pp.n_queries);
  W.u(1);
  W.u(3);  // commitments
  W.h(pre_root);
  W.h(trace_tree.root);
  W.h(comp_tree.root);
  W.u(oods_pow);
  W.u(3);  // sampled values: trees
  W.u(0);
  W.u(trace_evals.size());
  for (size_t i = 0; i < trace_evals.size(); i++) {
    W.u(1);
    W.q(sampled[i]);
  }
  W.u(8);
  for (size_t i = 0; i < 8; i++) {
    W.u(1);
    W.q(sampled[trace_evals.size() + i]);
  }
  W.u(3);  // decommitments
  W.u(0);
  W.hw(R.out, trace_dec.wit.first, trace_dec.wit.second);
  W.hw(R.out, comp_dec.wit.first, comp_dec.wit.second);
  W.u(3);  // queried values
  W.u(0);
  const size_t nq = queries.size();
  W.u(trace_evals.size());
  for (size_t c = 0; c < trace_evals.size(); c++) {
    W.u(nq);
    for (size_t i = 0; i < nq; i++) W.u(R.out[trace_dec.values_first + c * nq + i]);
  }
  W.u(8);
  for (size_t c = 0; c < 8; c++) {
    W.u(nq);
    for (size_t i = 0; i < nq; i++) W.u(R.out[comp_dec.values_first + c * nq + i]);
  }
  const auto layer_words = [&](const LayerDec& d, const Tree& t) {
    const size_t np = d.positions.size();
    size_t n_w = 0;
    for (bool wsel : d.is_witness) n_w += wsel;
    W.u(n_w);
    for (size_t i = 0; i < np; i++)
      if (d.is_witness[i])
        W.q(qm31_make(R.out[d.coord_first + i], R.out[d.coord_first + np + i], R.out[d.coord_first + 2 * np + i],
                      R.out[d.coord_first + 3 * np + i]));
    W.hw(R.out, d.wit.first, d.wit.second);
    W.h(t.root);
  };
  layer_words(first_dec, first_tree);
  W.u(layers.size());
  for (size_t i = 0; i < layers.size(); i++) layer_words(inner_dec[i], layers[i].tree);
  W.u(last_poly.size());
  for (const qm31& c : last_poly) W.q(c);
  W.u(pp.log_last_layer_degree_bound);
  W.u(fri_pow);
  words.swap(W.w);
  return CS_OK;
}

}  // namespace hp
}  // namespace cs

using namespace cs;

extern "C" cs_status cs_host_blake2s(const uint8_t* msg, size_t n, uint8_t out[32]) {
  CS_CHECK_ARG((msg != nullptr || n == 0) && out != nullptr, "host_blake2s: null pointer");
  hp::blake2s_public(msg, n, out);
  return CS_OK;
}

extern "C" cs_status cs_prove_wide_fib(const cs_wide_fib_proof_params* params, uint32_t* const* d_trace,
                                       uint64_t* h_words, size_t capacity, size_t* n_words, cs_stream stream) {
  CS_CHECK_ARG(params != nullptr && d_trace != nullptr && n_words != nullptr, "prove_wide_fib: null pointer");
  const cs_wide_fib_proof_params& pp = *params;
  CS_CHECK_ARG(pp.n_components >= 1 && pp.n_cols != nullptr && pp.log_sizes != nullptr,
               "prove_wide_fib: no components");
  CS_CHECK_ARG(pp.log_blowup_factor == 1, "prove_wide_fib: log_blowup_factor 1 (SubDomain evaluation)");
  CS_CHECK_ARG(pp.d_twiddles != nullptr && pp.d_itwiddles != nullptr, "prove_wide_fib: null twiddles");
  CS_CHECK_ARG(pp.pow_bits <= 32 && pp.n_queries >= 1, "prove_wide_fib: bad FRI parameters");
  uint32_t max_log = 0, n_total = 0;
  for (uint32_t k = 0; k < pp.n_components; k++) {
    CS_CHECK_ARG(pp.n_cols[k] >= 3 && pp.log_sizes[k] >= 1, "prove_wide_fib: component %u: %u columns of 2^%u", k,
                 pp.n_cols[k], pp.log_sizes[k]);
    max_log = std::max(max_log, pp.log_sizes[k]);
    n_total += pp.n_cols[k];
  }
  for (uint32_t c = 0; c < n_total; c++) CS_CHECK_ARG(d_trace[c] != nullptr, "prove_wide_fib: column %u is null", c);
  CS_CHECK_ARG(pp.lifting_log_size == max_log + pp.log_blowup_factor,
               "prove_wide_fib: lifting_log_size must be the largest evaluation size (%u)", max_log + 1);
  CS_CHECK_ARG(pp.lifting_log_size > pp.log_last_layer_degree_bound + pp.log_blowup_factor + 1,
               "prove_wide_fib: the trace is too small for the FRI parameters");
  CS_CHECK_ARG(pp.twiddle_log_size >= pp.lifting_log_size, "prove_wide_fib: twiddle tree too small");
  std::vector<uint64_t> words;
  cs_status s = hp::prove_wide_fib(pp, d_trace, words, to_stream(stream));
  if (s != CS_OK) return s;
  *n_words = words.size();
  CS_CHECK_ARG(h_words == nullptr || capacity >= words.size(), "prove_wide_fib: %zu words do not fit in %zu",
               words.size(), capacity);
  if (h_words != nullptr) std::copy(words.begin(), words.end(), h_words);
  return CS_OK;
}
