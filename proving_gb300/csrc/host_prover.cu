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
    if (stream_alloc(&p, std::max<size_t>(4, 4 * words), st) != cudaSuccess) {
      status = CS_ERR_OOM;
      return nullptr;
    }
    ptrs.push_back(p);
    return static_cast<uint32_t*>(p);
  }
  // frees one allocation early (stream-ordered)
  void release(void* p) {
    auto it = std::find(ptrs.begin(), ptrs.end(), p);
    if (it == ptrs.end()) return;
    cudaFreeAsync(p, st);
    ptrs.erase(it);
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
// emit(k, node) is called for each witness node of layer k (2^k nodes), leaves' layer first, in
// increasing node order; q is this thread's scratch copy of the queried leaves.
template <class Emit>
void for_each_witness_node(uint32_t height, const std::vector<uint64_t>& queried, Emit emit) {
  thread_local std::vector<uint64_t> q, up;
  q.assign(queried.begin(), queried.end());
  if (!std::is_sorted(q.begin(), q.end())) std::sort(q.begin(), q.end());  // the callers' are sorted
  q.erase(std::unique(q.begin(), q.end()), q.end());
  for (int layer = (int)height - 1; layer >= 0; layer--) {
    for (size_t i = 0; i < q.size(); i++) {
      const uint64_t sib = q[i] ^ 1;
      const bool present = (i + 1 < q.size() && q[i + 1] == sib) || (i > 0 && q[i - 1] == sib);
      if (!present) emit((uint32_t)layer + 1, sib);
    }
    up.clear();
    for (uint64_t x : q)
      if (up.empty() || up.back() != (x >> 1)) up.push_back(x >> 1);
    q.swap(up);
  }
}

// Every device read of a proof's decommitment, collected and made in one gather_runs call (a digest is
// one request of 8 words).
// The vectors keep their capacity from one proof to the next (see reads_for), so a proof's tens of
// thousands of requests do not fault in fresh pages each time.
struct Reads {
  std::vector<const uint32_t*> table;
  std::vector<uint64_t> lengths;
  std::map<const uint32_t*, uint32_t> slot_of;
  std::vector<uint32_t> slots, index, offset{0};  // offset[k]: request k's first word in out
  std::vector<uint32_t> out;
  size_t n_words = 0;
  const uint32_t* last_p = nullptr;  // the most recent slot lookup (requests come in runs per buffer)
  uint32_t last_slot = 0;
  void clear() {
    table.clear();
    lengths.clear();
    slot_of.clear();
    slots.clear();
    index.clear();
    offset.assign(1, 0);
    out.clear();
    n_words = 0;
    last_p = nullptr;
  }
  uint32_t slot(const uint32_t* p, uint64_t len) {
    if (p == last_p) return last_slot;
    auto it = slot_of.find(p);
    uint32_t s;
    if (it != slot_of.end()) {
      s = it->second;
    } else {
      s = (uint32_t)table.size();
      table.push_back(p);
      lengths.push_back(len);
      slot_of[p] = s;
    }
    last_p = p;
    last_slot = s;
    return s;
  }
  // words [i, i + count) of p (len words): out[returned offset ..]
  size_t add(const uint32_t* p, uint64_t len, uint64_t i, uint32_t count = 1) {
    slots.push_back(slot(p, len));
    index.push_back((uint32_t)i);
    const size_t first = n_words;
    n_words += count;
    offset.push_back((uint32_t)n_words);
    return first;
  }
  cs_status run(cudaStream_t st) {
    out.assign(n_words, 0);
    if (slots.empty()) return CS_OK;
    return gather_runs(table.data(), lengths.data(), (uint32_t)table.size(), slots.data(), index.data(),
                       offset.data(), (uint32_t)slots.size(), out.data(), st);
  }
};

// A cleared Reads of this thread (k: 0 or 1, two can be live in one proof).
Reads& reads_for(int k) {
  thread_local Reads pool[2];
  pool[k].clear();
  return pool[k];
}

// A tree's witness digests registered with a Reads: (first read, count of digests).
std::pair<size_t, size_t> read_witness(Reads& R, const Tree& t, const std::vector<uint64_t>& q) {
  size_t first = R.n_words, n = 0;
  const uint64_t words = t.words();
  for_each_witness_node(t.height, q, [&](uint32_t k, uint64_t node) {
    R.add(t.layers, words, t.node_word(k, node), 8);
    n++;
  });
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
  std::vector<uint64_t>& w;
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
  uint32_t step = 1;  // the folds from this layer to the next
};

struct Col {
  uint32_t* p;
  uint32_t log;
};

bool same(const qpoint& a, const qpoint& b) { return std::memcmp(&a, &b, sizeof(qpoint)) == 0; }

bool point_less(const qpoint& a, const qpoint& b) {
  const uint32_t ka[8] = {a.x.a.a, a.x.a.b, a.x.b.a, a.x.b.b, a.y.a.a, a.y.a.b, a.y.b.a, a.y.b.b};
  const uint32_t kb[8] = {b.x.a.a, b.x.a.b, b.x.b.a, b.x.b.b, b.y.a.a, b.y.a.b, b.y.b.a, b.y.b.b};
  return std::lexicographical_compare(ka, ka + 8, kb, kb + 8);
}

qpoint add_m31_point(const qpoint& p, const cpoint& g) {
  const qm31 gx = qm(g.x), gy = qm(g.y);
  return {qm31_sub(qm31_mul(p.x, gx), qm31_mul(p.y, gy)), qm31_add(qm31_mul(p.x, gy), qm31_mul(p.y, gx))};
}

qm31 from_partial_evals(const qm31* e) {
  qm31 r = e[0];
  r = qm31_add(r, qm31_mul(e[1], qm31_make(0, 1, 0, 0)));
  r = qm31_add(r, qm31_mul(e[2], qm31_make(0, 0, 1, 0)));
  r = qm31_add(r, qm31_mul(e[3], qm31_make(0, 0, 0, 1)));
  return r;
}

struct ProofConfig {
  uint32_t L, b, pow_bits, log_last_layer_degree_bound, n_queries;
  const uint32_t *tw, *itw;
  uint32_t tw_log;
  uint32_t fold_step = 1;
  // one launch per column for every per-column stage (interpolate, evaluate, running sums,
  // out-of-domain sampling, constraint quotients): the plain form, as a backend without batched
  // overrides runs the trait's default per-column loops
  bool plain = false;
};

}  // namespace

void blake2s_public(const uint8_t* msg, size_t n, uint8_t out[32]) { blake2s(msg, n, out); }

// The prover's device state and the helpers the AIRs use.
struct Prover {
  Arena A;
  cudaStream_t st;
  Channel ch;
  ProofConfig cfg;
  Prover(cudaStream_t s, const ProofConfig& c) : A(s), st(s), cfg(c) {}

  // Evaluations (in place: coefficients) of columns of one size.
  cs_status interpolate(const std::vector<uint32_t*>& cols, uint32_t log) {
    if (cols.empty()) return CS_OK;
    std::vector<uint32_t*> c(cols);
    if (cfg.plain) {
      for (uint32_t* x : c) HP_TRY(cs_interpolate_columns(&x, 1, log, cfg.itw, cfg.tw_log, st));
      return CS_OK;
    }
    return cs_interpolate_columns(c.data(), (uint32_t)c.size(), log, cfg.itw, cfg.tw_log, st);
  }
  // Coefficient columns of one size evaluated on CanonicCoset(to_log) into one new block.
  cs_status evaluate(const std::vector<uint32_t*>& coeffs, uint32_t log, uint32_t to_log, std::vector<uint32_t*>& out) {
    out.clear();
    if (coeffs.empty()) return CS_OK;
    uint32_t* blk = A.alloc(coeffs.size() << to_log);
    if (!blk) return A.status;
    for (size_t j = 0; j < coeffs.size(); j++) out.push_back(blk + (j << to_log));
    std::vector<const uint32_t*> src(coeffs.begin(), coeffs.end());
    if (cfg.plain) {
      for (size_t j = 0; j < src.size(); j++)
        HP_TRY(cs_evaluate_columns(&src[j], &out[j], 1, log, to_log, cfg.tw, cfg.tw_log, st));
      return CS_OK;
    }
    return cs_evaluate_columns(src.data(), out.data(), (uint32_t)coeffs.size(), log, to_log, cfg.tw, cfg.tw_log, st);
  }
  // Columns of any sizes: evaluations src[i] (log size logs[i]) interpolated into dst[i] (which may
  // be src[i]), every size in one call (PolyOps::interpolate_columns over the mixed batch).
  cs_status interpolate_mixed(const std::vector<const uint32_t*>& src, const std::vector<uint32_t*>& dst,
                              const std::vector<uint32_t>& logs) {
    if (src.empty()) return CS_OK;
    if (cfg.plain) {
      for (size_t i = 0; i < src.size(); i++)
        HP_TRY(cs_interpolate_columns_into(&src[i], &dst[i], 1, logs[i], cfg.itw, cfg.tw_log, st));
      return CS_OK;
    }
    return cs_interpolate_columns_multi(src.data(), dst.data(), logs.data(), (uint32_t)src.size(), cfg.itw, cfg.tw_log,
                                        st);
  }
  // Coefficient columns of any sizes evaluated on CanonicCoset(log + blowup) into one new block,
  // every size in one call (PolyOps::evaluate_polynomials over the mixed batch).
  cs_status evaluate_mixed(const std::vector<uint32_t*>& coeffs, const std::vector<uint32_t>& logs,
                           std::vector<uint32_t*>& out) {
    out.clear();
    if (coeffs.empty()) return CS_OK;
    size_t total = 0;
    for (uint32_t l : logs) total += 1ull << (l + cfg.b);
    uint32_t* blk = A.alloc(total);
    if (!blk) return A.status;
    size_t off = 0;
    for (uint32_t l : logs) {
      out.push_back(blk + off);
      off += 1ull << (l + cfg.b);
    }
    std::vector<const uint32_t*> src(coeffs.begin(), coeffs.end());
    if (cfg.plain) {
      for (size_t j = 0; j < src.size(); j++)
        HP_TRY(cs_evaluate_columns(&src[j], &out[j], 1, logs[j], logs[j] + cfg.b, cfg.tw, cfg.tw_log, st));
      return CS_OK;
    }
    return cs_evaluate_columns_multi(src.data(), out.data(), logs.data(), cfg.b, (uint32_t)src.size(), cfg.tw,
                                     cfg.tw_log, st);
  }
  std::vector<uint32_t*>& acc_for(std::map<uint32_t, std::vector<uint32_t*>>& acc, uint32_t el) {
    if (!acc.count(el)) {
      uint32_t* blk = A.alloc(4ull << el);
      if (blk) cudaMemsetAsync(blk, 0, 16ull << el, st);
      acc[el] = {blk, blk + (1ull << el), blk + (2ull << el), blk + (3ull << el)};
    }
    return acc[el];
  }
};

// The AIR-specific parts of a proof, called by prove() between its generic phases.
struct Air {
  virtual ~Air() = default;
  // the trace tree's columns (evaluations on their blown-up domains), in tree order
  virtual cs_status trace(Prover& P, std::vector<Col>& cols) = 0;
  // the mask offsets of every trace column, in tree order (left empty: every column at the point)
  virtual void trace_offsets(std::vector<std::vector<int32_t>>&) const {}
  virtual bool has_interaction() const { return false; }
  virtual bool mix_claimed() const { return false; }
  // the interaction tree's columns, whether each is also sampled at the previous row, and the
  // claimed sums (z, alpha: the lookup elements)
  virtual cs_status interaction(Prover&, const qm31&, const qm31&, std::vector<Col>&, std::vector<bool>&,
                                std::vector<qm31>&) {
    return CS_OK;
  }
  virtual uint32_t n_constraints() const = 0;
  // EvaluationMode::SubDomain's log_expansion (accumulation.rs:42-62): the accumulator holds the
  // evaluation on the subdomain of CanonicCoset(its log size + this); 0 for a canonic coset
  virtual uint32_t log_expansion() const { return 0; }
  // the constraint quotients added to per-size accumulators, powers of the random coefficient given
  virtual cs_status composition(Prover& P, const std::vector<qm31>& powers,
                                std::map<uint32_t, std::vector<uint32_t*>>& acc) = 0;
  // the composition polynomial at the point from the samples (sampled[tree][col][k]), or false for
  // no check
  virtual bool at_point(const qpoint&, uint32_t, const qm31&, const std::vector<std::vector<std::vector<qm31>>>&,
                        qm31&) {
    return false;
  }
};

// prove_ex (crates/stwo/src/prover/mod.rs:39-138) over the trees [preprocessed (empty), trace,
// interaction (if any), composition], FRI with cfg.fold_step folds per layer, the felt stream of the
// StarkProof.
cs_status prove(const ProofConfig& cfg, Air& air, std::vector<uint64_t>& words, std::vector<qm31>& claimed,
                cudaStream_t st) {
  Prover P(st, cfg);
  Arena& A = P.A;
  Channel& ch = P.ch;
  const uint32_t L = cfg.L, b = cfg.b, mldb = L - b;
  // --- preprocessed tree: empty (a single hash of no data at height 0, pcs/mod.rs:83-96)
  uint8_t pre_root[32];
  blake2s(nullptr, 0, pre_root);
  ch.mix_root(pre_root);
  struct TreeCols {
    std::vector<Col> cols;
    std::vector<bool> two;                      // also sampled at the previous row
    std::vector<std::vector<int32_t>> offs;     // the offsets each column is sampled at
    Tree tree;
  };
  // a column sampled at the row, or at the previous row and the row
  const auto offsets_of = [](const std::vector<bool>& two) {
    std::vector<std::vector<int32_t>> o;
    for (bool t : two) o.push_back(t ? std::vector<int32_t>{-1, 0} : std::vector<int32_t>{0});
    return o;
  };
  std::vector<TreeCols> trees;
  // --- trace tree (TreeBuilder::extend_evals + commit)
  trees.emplace_back();
  HP_TRY(air.trace(P, trees.back().cols));
  trees.back().two.assign(trees.back().cols.size(), false);
  air.trace_offsets(trees.back().offs);
  if (trees.back().offs.empty()) trees.back().offs = offsets_of(trees.back().two);
  CS_CHECK_ARG(trees.back().offs.size() == trees.back().cols.size(), "prove: %zu offset lists for %zu columns",
               trees.back().offs.size(), trees.back().cols.size());
  const auto commit_tree = [&](TreeCols& t) -> cs_status {
    std::vector<uint32_t*> c;
    std::vector<uint32_t> l;
    for (const Col& x : t.cols) {
      c.push_back(x.p);
      l.push_back(x.log);
    }
    HP_TRY(commit(A, c, l, L, t.tree));
    return read_root(A, t.tree);
  };
  HP_TRY(commit_tree(trees.back()));
  ch.mix_root(trees.back().tree.root);
  // --- lookup elements and the interaction tree
  if (air.has_interaction()) {
    const qm31 z = ch.draw_secure_felt();
    const qm31 alpha = ch.draw_secure_felt();
    trees.emplace_back();
    HP_TRY(air.interaction(P, z, alpha, trees.back().cols, trees.back().two, claimed));
    trees.back().offs = offsets_of(trees.back().two);
    HP_TRY(commit_tree(trees.back()));
    if (air.mix_claimed()) ch.mix_felts(claimed);
    ch.mix_root(trees.back().tree.root);
  }
  // --- composition polynomial (component_prover.rs:95-116, accumulation.rs:142-180)
  const qm31 random_coeff = ch.draw_secure_felt();
  const std::vector<qm31> pw = powers(random_coeff, air.n_constraints());
  std::map<uint32_t, std::vector<uint32_t*>> sub_acc;
  HP_TRY(air.composition(P, pw, sub_acc));
  std::vector<uint32_t*> acc_cols;
  std::vector<uint32_t> acc_logs;
  for (auto& [el, coords] : sub_acc) {
    acc_cols.insert(acc_cols.end(), coords.begin(), coords.end());
    acc_logs.push_back(el);
  }
  if (acc_logs.size() > 1)
    HP_TRY(cs_lift_and_accumulate(acc_cols.data(), acc_logs.data(), (uint32_t)acc_logs.size(), st));
  const uint32_t comp_log = acc_logs.back();
  std::vector<uint32_t*> accum(acc_cols.end() - 4, acc_cols.end());
  // DomainEvaluationAccumulator::finalize (accumulation.rs:136-180)
  if (air.log_expansion())
    HP_TRY(cs_interpolate_columns_on_subdomain(accum.data(), 4, comp_log, comp_log + air.log_expansion(), cfg.itw,
                                               cfg.tw_log, st));
  else
    HP_TRY(P.interpolate(accum, comp_log));
  const size_t half = 1ull << (comp_log - 1);
  std::vector<uint32_t*> split(accum);
  for (int c = 0; c < 4; c++) split.push_back(accum[c] + half);
  const uint32_t comp_eval_log = (comp_log - 1) + b;
  std::vector<uint32_t*> comp_cols;
  HP_TRY(P.evaluate(split, comp_log - 1, comp_eval_log, comp_cols));
  trees.emplace_back();
  for (uint32_t* c : comp_cols) trees.back().cols.push_back({c, comp_eval_log});
  trees.back().two.assign(8, false);
  trees.back().offs = offsets_of(trees.back().two);
  HP_TRY(commit_tree(trees.back()));
  ch.mix_root(trees.back().tree.root);

  // --- OODS proof of work and point (mod.rs:75-83); the previous row (component.rs:202-214)
  uint64_t oods_pow = 0;
  HP_TRY(cs_grind_blake2s(ch.digest, 16, 1ull << 48, &oods_pow, st));
  ch.mix_u64(oods_pow);
  const qpoint oods = random_point(ch.draw_secure_felt());
  const cpoint g = index_to_point(1u << (31 - mldb));
  const qpoint prev_pt = add_m31_point(oods, {g.x, m31_neg(g.y)});
  // the point `o` trace steps from the OODS point: o G_mldb added (G^-1 is G's conjugate)
  const auto point_at = [&](int32_t o) -> qpoint {
    if (o == 0) return oods;
    if (o == -1) return prev_pt;
    return add_m31_point(oods, index_to_point(((uint32_t)o << (31 - mldb)) & 0x7fffffffu));
  };

  // --- sampled values (pcs/mod.rs:175-214): one weight column per (size, point); values read once
  struct Sample {
    size_t tree, col, slot;
  };
  std::vector<std::pair<std::pair<uint32_t, int32_t>, std::vector<Sample>>> groups;  // (log, offset)
  for (size_t t = 0; t < trees.size(); t++)
    for (size_t c = 0; c < trees[t].cols.size(); c++) {
      const std::vector<int32_t>& pts = trees[t].offs[c];
      for (size_t k = 0; k < pts.size(); k++) {
        const std::pair<uint32_t, int32_t> key{trees[t].cols[c].log, pts[k]};
        auto it = std::find_if(groups.begin(), groups.end(), [&](auto& g) { return g.first == key; });
        if (it == groups.end()) {
          groups.push_back({key, {}});
          it = groups.end() - 1;
        }
        it->second.push_back({t, c, k});
      }
    }
  size_t n_samples = 0;
  for (auto& gr : groups) n_samples += gr.second.size();
  uint32_t* d_samples = A.alloc(4 * n_samples);
  if (!d_samples) return A.status;
  size_t row = 0;
  for (auto& [key, members] : groups) {
    qpoint pt = point_at(key.second);
    for (uint32_t d = key.first; d < L; d++) pt = q_double(pt);
    const uint32_t ls = key.first;
    uint32_t* w = A.alloc(4ull << ls);
    if (!w) return A.status;
    uint32_t* wc[4] = {w, w + (1ull << ls), w + (2ull << ls), w + (3ull << ls)};
    const uint32_t px[4] = {pt.x.a.a, pt.x.a.b, pt.x.b.a, pt.x.b.b}, py[4] = {pt.y.a.a, pt.y.a.b, pt.y.b.a, pt.y.b.b};
    HP_TRY(cs_barycentric_weights(ls, px, py, wc, st));
    std::vector<const uint32_t*> cols;
    for (const Sample& m : members) cols.push_back(trees[m.tree].cols[m.col].p);
    const uint32_t* wcc[4] = {wc[0], wc[1], wc[2], wc[3]};
    if (cfg.plain) {
      for (size_t j = 0; j < cols.size(); j++)
        HP_TRY(cs_barycentric_eval(&cols[j], 1, ls, wcc, d_samples + 4 * (row + j), st));
    } else {
      HP_TRY(cs_barycentric_eval(cols.data(), (uint32_t)cols.size(), ls, wcc, d_samples + 4 * row, st));
    }
    row += members.size();
    A.release(w);
  }
  std::vector<uint32_t> samples(4 * n_samples);
  CS_CUDA(cudaMemcpyAsync(samples.data(), d_samples, 16 * n_samples, cudaMemcpyDeviceToHost, st));
  CS_CUDA(cudaStreamSynchronize(st));
  std::vector<std::vector<std::vector<qm31>>> sampled(trees.size() + 1);  // [0]: the preprocessed tree
  for (size_t t = 0; t < trees.size(); t++) {
    sampled[t + 1].resize(trees[t].cols.size());
    for (size_t c = 0; c < trees[t].cols.size(); c++) sampled[t + 1][c].resize(trees[t].offs[c].size());
  }
  row = 0;
  for (auto& [key, members] : groups)
    for (const Sample& m : members) {
      sampled[m.tree + 1][m.col][m.slot] =
          qm31_make(samples[4 * row], samples[4 * row + 1], samples[4 * row + 2], samples[4 * row + 3]);
      row++;
    }
  {
    std::vector<qm31> all;
    for (auto& tr : sampled)
      for (auto& col : tr) all.insert(all.end(), col.begin(), col.end());
    ch.mix_felts(all);
  }

  // --- FRI quotients (quotient_ops.rs:86-160; periodicity samples, quotients.rs:274-319)
  const qm31 quotient_coeff = ch.draw_secure_felt();
  struct Entry {
    uint32_t log;
    uint32_t* col;
    qpoint pt;
    qm31 value;
  };
  std::vector<Entry> entries;
  for (size_t t = 0; t < trees.size(); t++)
    for (size_t c = 0; c < trees[t].cols.size(); c++) {
      const Col& col = trees[t].cols[c];
      const auto& v = sampled[t + 1][c];
      const std::vector<int32_t>& o = trees[t].offs[c];
      if (o.size() == 2) {
        // the periodicity sample: the second point shifted by the column's period, its value
        const qpoint shifted = add_m31_point(point_at(o[1]), index_to_point(1u << (31 - (L - col.log))));
        entries.push_back({col.log, col.p, shifted, v[1]});
      }
      for (size_t k = 0; k < o.size(); k++) entries.push_back({col.log, col.p, point_at(o[k]), v[k]});
    }
  const std::vector<qm31> qp = powers(quotient_coeff, (uint32_t)entries.size());
  struct Acc {
    qpoint pt;
    uint32_t* cols[4];
    uint32_t log;
    qm31 fl;
  };
  std::vector<Acc> accs;
  std::vector<uint32_t> sizes;
  for (const Entry& e : entries)
    if (std::find(sizes.begin(), sizes.end(), e.log) == sizes.end()) sizes.push_back(e.log);
  std::sort(sizes.begin(), sizes.end());
  for (uint32_t ls : sizes) {
    std::vector<std::pair<qpoint, std::vector<size_t>>> batches;  // by point, in insertion order
    for (size_t k = 0; k < entries.size(); k++) {
      if (entries[k].log != ls) continue;
      auto it = std::find_if(batches.begin(), batches.end(), [&](auto& bt) { return same(bt.first, entries[k].pt); });
      if (it == batches.end()) {
        batches.push_back({entries[k].pt, {}});
        it = batches.end() - 1;
      }
      it->second.push_back(k);
    }
    for (auto& [pt, ks] : batches) {
      std::vector<uint32_t> coeffs(12 * ks.size());
      std::vector<const uint32_t*> cols;
      for (size_t j = 0; j < ks.size(); j++) {
        line_coeffs(pt.y, entries[ks[j]].value, qp[ks[j]], &coeffs[12 * j]);
        cols.push_back(entries[ks[j]].col);
      }
      const uint32_t pl = ls - b;
      uint32_t* blk = A.alloc(4ull << pl);
      if (!blk) return A.status;
      Acc a;
      a.pt = pt;
      a.log = pl;
      for (int c = 0; c < 4; c++) a.cols[c] = blk + ((size_t)c << pl);
      uint32_t fl[4];
      HP_TRY(cs_accumulate_numerators(cols.data(), (uint32_t)cols.size(), ls, b, coeffs.data(), a.cols, fl, st));
      a.fl = qm31_make(fl[0], fl[1], fl[2], fl[3]);
      accs.push_back(a);
    }
  }
  // per point (sorted), lifted and accumulated over ascending sizes
  std::vector<qpoint> points;
  for (const Acc& a : accs)
    if (std::find_if(points.begin(), points.end(), [&](const qpoint& p) { return same(p, a.pt); }) == points.end())
      points.push_back(a.pt);
  std::stable_sort(points.begin(), points.end(), point_less);
  std::vector<const uint32_t*> qaccs;
  std::vector<uint32_t> qlogs, qpts, qfl;
  for (const qpoint& p : points) {
    std::vector<uint32_t*> cols;
    std::vector<uint32_t> logs;
    qm31 fl = qm31_make(0, 0, 0, 0);
    for (const Acc& a : accs)
      if (same(a.pt, p)) {
        cols.insert(cols.end(), a.cols, a.cols + 4);
        logs.push_back(a.log);
        fl = qm31_add(fl, a.fl);
      }
    if (logs.size() > 1) HP_TRY(cs_lift_and_accumulate(cols.data(), logs.data(), (uint32_t)logs.size(), st));
    qaccs.insert(qaccs.end(), cols.end() - 4, cols.end());
    qlogs.push_back(logs.back());
    const uint32_t pw8[8] = {p.x.a.a, p.x.a.b, p.x.b.a, p.x.b.b, p.y.a.a, p.y.a.b, p.y.b.a, p.y.b.b};
    qpts.insert(qpts.end(), pw8, pw8 + 8);
    const uint32_t f4[4] = {fl.a.a, fl.a.b, fl.b.a, fl.b.b};
    qfl.insert(qfl.end(), f4, f4 + 4);
  }
  const uint32_t sub_log = L - b;
  uint32_t* qblk = A.alloc(4ull << sub_log);
  if (!qblk) return A.status;
  uint32_t* qcols[4] = {qblk, qblk + (1ull << sub_log), qblk + (2ull << sub_log), qblk + (3ull << sub_log)};
  HP_TRY(cs_quotients_on_subdomain(qaccs.data(), qlogs.data(), (uint32_t)points.size(), qpts.data(), qfl.data(), L,
                                   b, qcols, st));
  HP_TRY(cs_interpolate_columns_on_subdomain(qcols, 4, sub_log, L, cfg.itw, cfg.tw_log, st));
  std::vector<uint32_t*> quotients;
  HP_TRY(P.evaluate(std::vector<uint32_t*>(qcols, qcols + 4), sub_log, L, quotients));

  const uint32_t last_log = cfg.log_last_layer_degree_bound + b;
  std::vector<FriLayer> layers;
  Tree first_tree;
  std::vector<uint32_t*> cur;
  uint32_t* d_state = nullptr;  // the device channel of the fold_step 1 loop
  if (cfg.fold_step > 1) {
    // --- FRI commit (fri.rs:113-226) with fold_step k: the first layer's circle fold is followed by
    // k - 1 line folds with alpha^2, alpha^4, ..., every inner layer folds k times (alpha, alpha^2,
    // ... : squared_alpha_powers, fri.rs:79-87), the last the 1..k folds left; a layer folded more
    // than once commits packed leaves of 4 values per coordinate (fri.rs:294-305, 357-367). The
    // channel stays on the host.
    const uint32_t k = cfg.fold_step;
    const auto commit_layer = [&](const std::vector<uint32_t*>& ev, uint32_t log, uint32_t step,
                                  Tree& t) -> cs_status {
      if (step > 1 && log >= 2) {
        uint32_t* blk = A.alloc(16ull << (log - 2));
        if (!blk) return A.status;
        std::vector<uint32_t*> packed;
        for (int c = 0; c < 16; c++) packed.push_back(blk + ((size_t)c << (log - 2)));
        const uint32_t* src[4] = {ev[0], ev[1], ev[2], ev[3]};
        HP_TRY(cs_pack_leaves_input(src, log, packed.data(), st));
        HP_TRY(commit(A, packed, std::vector<uint32_t>(16, log - 2), log - 2, t));
        A.release(blk);
      } else {
        HP_TRY(commit(A, ev, std::vector<uint32_t>(4, log), log, t));
      }
      return read_root(A, t);
    };
    const auto words_of = [](const qm31& x, uint32_t* w) {
      w[0] = x.a.a;
      w[1] = x.a.b;
      w[2] = x.b.a;
      w[3] = x.b.b;
    };
    // `steps` folds of the line evaluation `ev` (2^log values) with alpha, alpha^2, alpha^4, ...
    const auto fold = [&](std::vector<uint32_t*>& ev, uint32_t log, qm31 alpha, uint32_t steps) -> cs_status {
      const uint32_t nl = log - steps;
      uint32_t* blk = A.alloc(4ull << nl);
      if (!blk) return A.status;
      std::vector<uint32_t*> nxt = {blk, blk + (1ull << nl), blk + (2ull << nl), blk + (3ull << nl)};
      std::vector<uint32_t> alphas(4 * steps);
      for (uint32_t j = 0; j < steps; j++) {
        words_of(alpha, &alphas[4 * j]);
        alpha = qm31_mul(alpha, alpha);
      }
      const uint32_t* src[4] = {ev[0], ev[1], ev[2], ev[3]};
      HP_TRY(cs_fold_line_steps(src, log, steps, alphas.data(), nxt.data(), cfg.itw, cfg.tw_log, st));
      ev = nxt;
      return CS_OK;
    };
    HP_TRY(commit_layer(quotients, L, k, first_tree));
    ch.mix_root(first_tree.root);
    qm31 alpha = ch.draw_secure_felt();
    uint32_t line_log = L - 1;
    {
      uint32_t* blk = A.alloc(4ull << line_log);
      if (!blk) return A.status;
      cur = {blk, blk + (1ull << line_log), blk + (2ull << line_log), blk + (3ull << line_log)};
      const uint32_t* src[4] = {quotients[0], quotients[1], quotients[2], quotients[3]};
      uint32_t aw[4];
      words_of(alpha, aw);
      HP_TRY(cs_fold_circle_into_line(src, L, aw, cur.data(), cfg.itw, cfg.tw_log, st));
    }
    HP_TRY(fold(cur, line_log, qm31_mul(alpha, alpha), k - 1));
    line_log -= k - 1;
    while (line_log > last_log) {
      FriLayer lay;
      lay.log_size = line_log;
      lay.eval = cur;
      lay.step = line_log > last_log + k ? k : line_log - last_log;
      HP_TRY(commit_layer(cur, line_log, lay.step, lay.tree));
      ch.mix_root(lay.tree.root);
      alpha = ch.draw_secure_felt();
      HP_TRY(fold(cur, line_log, alpha, lay.step));
      line_log -= lay.step;
      layers.push_back(lay);
    }
  } else {
    // --- FRI commit (fri.rs:113-226), fold_step 1, the channel kept on the device for the layer loop
    // 9 state words, then (from word 12, 16-byte aligned) room for the challenges of up to 64 layers
    d_state = A.alloc(12 + 4 * 64);
    if (!d_state) return A.status;
    uint32_t state[9];
    std::memcpy(state, ch.digest, 32);
    state[8] = ch.n_draws;
    CS_CUDA(cudaMemcpyAsync(d_state, state, sizeof(state), cudaMemcpyHostToDevice, st));
    uint32_t* d_felts = d_state + 12;
    uint32_t n_felts = 0;
    HP_TRY(commit(A, quotients, std::vector<uint32_t>(4, L), L, first_tree));
    HP_TRY(cs_channel_mix_root(d_state, first_tree.layers + first_tree.words() - 8, st));
    HP_TRY(cs_channel_draw_secure_felt(d_state, d_felts + 4 * n_felts, st));
    uint32_t line_log = L - 1;
    {
      uint32_t* blk = A.alloc(4ull << line_log);
      if (!blk) return A.status;
      cur = {blk, blk + (1ull << line_log), blk + (2ull << line_log), blk + (3ull << line_log)};
      const uint32_t* src[4] = {quotients[0], quotients[1], quotients[2], quotients[3]};
      HP_TRY(cs_fold_circle_into_line_device_alpha(src, L, d_felts + 4 * n_felts, cur.data(), cfg.itw, cfg.tw_log, st));
      n_felts++;
    }
    while (line_log >= last_log + 1 && n_felts < 64) {  // every layer above the last folds once
      if (!cfg.plain && line_log <= 10 && n_felts + (line_log - last_log) <= 64) {
        // the layers of at most 2^10 values, down to the last layer: one launch (cs_fri_commit_fold_tail)
        const uint32_t n_tail = line_log - last_log;
        std::vector<uint32_t*> evals(cur.begin(), cur.end()), tree_bufs;
        for (uint32_t j = 0; j < n_tail; j++) {
          FriLayer lay;
          lay.log_size = line_log - j;
          lay.eval = std::vector<uint32_t*>(evals.end() - 4, evals.end());
          lay.tree.height = lay.log_size;
          lay.tree.layers = A.alloc(((2ull << lay.log_size) - 1) * 8);
          const uint32_t nl = lay.log_size - 1;
          uint32_t* blk = A.alloc(4ull << nl);
          if (!lay.tree.layers || !blk) return A.status;
          for (int c = 0; c < 4; c++) evals.push_back(blk + ((size_t)c << nl));
          tree_bufs.push_back(lay.tree.layers);
          layers.push_back(lay);
        }
        HP_TRY(cs_fri_commit_fold_tail(d_state, d_felts + 4 * n_felts, evals.data(), tree_bufs.data(), line_log,
                                       n_tail, cfg.itw, cfg.tw_log, st));
        n_felts += n_tail;
        cur.assign(evals.end() - 4, evals.end());
        line_log = last_log;
        break;
      }
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
      HP_TRY(cs_fold_line_device_alpha(src, line_log, d_felts + 4 * n_felts, nxt.data(), cfg.itw, cfg.tw_log, st));
      n_felts++;
      layers.push_back(lay);
      cur = nxt;
      line_log = nl;
    }
  }
  // the state, every layer root and the last layer's evaluation back in one read (with fold_step
  // above 1 the channel and the roots are already on the host: the evaluation alone)
  std::vector<qm31> last_poly;
  {
    const bool device_channel = cfg.fold_step == 1;
    Reads& R = reads_for(0);
    std::vector<Tree*> ts = {&first_tree};
    for (FriLayer& l : layers) ts.push_back(&l.tree);
    if (device_channel) {
      R.add(d_state, 9, 0, 9);
      for (Tree* t : ts)
        R.add(t->layers, t->words(), t->words() - 8, 8);
    }
    const uint32_t last_n = 1u << last_log;
    for (int c = 0; c < 4; c++)
      R.add(cur[c], last_n, 0, last_n);
    HP_TRY(R.run(st));
    size_t o = 0;
    if (device_channel) {
      for (int i = 0; i < 8; i++)
        for (int k = 0; k < 4; k++) ch.digest[4 * i + k] = (uint8_t)(R.out[i] >> (8 * k));
      ch.n_draws = R.out[8];
      o = 9;
      for (Tree* t : ts) {
        for (int i = 0; i < 8; i++)
          for (int k = 0; k < 4; k++) t->root[4 * i + k] = (uint8_t)(R.out[o + i] >> (8 * k));
        o += 8;
      }
    }
    std::vector<qm31> last_values(last_n);
    for (uint32_t i = 0; i < last_n; i++)
      last_values[i] = qm31_make(R.out[o + i], R.out[o + last_n + i], R.out[o + 2 * last_n + i],
                                 R.out[o + 3 * last_n + i]);
    // commit_last_layer (fri.rs:208-226)
    const std::vector<qm31> coeffs = line_interpolate(last_values, last_log);
    const uint32_t bound = 1u << cfg.log_last_layer_degree_bound;
    for (uint32_t i = bound; i < last_n; i++)
      CS_CHECK_ARG(coeffs[i].a.a == 0 && coeffs[i].a.b == 0 && coeffs[i].b.a == 0 && coeffs[i].b.b == 0,
                   "prove: invalid degree in the last FRI layer");
    last_poly.resize(bound);
    for (uint32_t i = 0; i < bound; i++) last_poly[i] = coeffs[bitrev(i, cfg.log_last_layer_degree_bound)];
    ch.mix_felts(last_poly);
  }

  // --- FRI proof of work and queries (fri.rs:229-283)
  uint64_t fri_pow = 0;
  HP_TRY(cs_grind_blake2s(ch.digest, cfg.pow_bits, 1ull << 48, &fri_pow, st));
  ch.mix_u64(fri_pow);
  const std::vector<uint32_t> qraw = ch.draw_queries(L, cfg.n_queries);
  std::vector<uint64_t> queries(qraw.begin(), qraw.end());
  std::sort(queries.begin(), queries.end());
  queries.erase(std::unique(queries.begin(), queries.end()), queries.end());

  // --- decommitments: every read registered, one gather
  Reads& R = reads_for(1);
  struct LayerDec {
    std::vector<uint64_t> positions;
    std::vector<bool> is_witness;
    size_t coord_first;
    std::pair<size_t, size_t> wit;
  };
  // compute_decommitment_positions_and_witness_evals (fri.rs:408-438): every coset of 2^step
  // positions around a query; a packed tree opens the leaves holding them (fri.rs:318-326)
  const auto fri_layer = [&](const std::vector<uint32_t*>& eval, uint32_t log_size, const Tree& t,
                             const std::vector<uint64_t>& q, uint32_t step) {
    LayerDec d;
    std::vector<uint64_t> starts;
    for (uint64_t x : q)
      if (starts.empty() || starts.back() != ((x >> step) << step)) starts.push_back((x >> step) << step);
    for (uint64_t s0 : starts)
      for (uint64_t j = 0; j < (1ull << step); j++) {
        d.positions.push_back(s0 + j);
        d.is_witness.push_back(!std::binary_search(q.begin(), q.end(), s0 + j));
      }
    d.coord_first = R.n_words;
    for (int c = 0; c < 4; c++)  // each coset is a run of 2^step words
      for (uint64_t s0 : starts) R.add(eval[c], 1ull << log_size, s0, 1ull << step);
    if (step > 1 && log_size >= 2) {
      std::vector<uint64_t> leaves;
      for (uint64_t x : d.positions)
        if (leaves.empty() || leaves.back() != (x >> 2)) leaves.push_back(x >> 2);
      d.wit = read_witness(R, t, leaves);
    } else {
      d.wit = read_witness(R, t, d.positions);
    }
    return d;
  };
  // Queries::fold (queries.rs:50-56)
  const auto fold_queries = [](const std::vector<uint64_t>& q, uint32_t n) {
    std::vector<uint64_t> out;
    for (uint64_t x : q)
      if (out.empty() || out.back() != (x >> n)) out.push_back(x >> n);
    return out;
  };
  const LayerDec first_dec = fri_layer(quotients, L, first_tree, queries, cfg.fold_step);
  std::vector<LayerDec> inner_dec;
  std::vector<uint64_t> lq = fold_queries(queries, cfg.fold_step);
  for (FriLayer& l : layers) {
    inner_dec.push_back(fri_layer(l.eval, l.log_size, l.tree, lq, l.step));
    lq = fold_queries(lq, l.step);
  }
  struct TreeDec {
    size_t values_first;
    std::pair<size_t, size_t> wit;
  };
  std::vector<TreeDec> tree_decs;
  for (TreeCols& t : trees) {  // MerkleProverLifted::decommit: queried values per column, then the witness
    TreeDec d;
    d.values_first = R.n_words;
    for (const Col& c : t.cols) {
      const uint32_t shift = L - c.log;
      for (uint64_t q : queries) R.add(c.p, 1ull << c.log, ((q >> (shift + 1)) << 1) + (q & 1));
    }
    d.wit = read_witness(R, t.tree, queries);
    tree_decs.push_back(d);
  }
  HP_TRY(R.run(st));

  // --- sanity check (mod.rs:121-132)
  {
    qm31 expected;
    if (air.at_point(oods, mldb, random_coeff, sampled, expected)) {
      std::vector<qm31> cs;
      for (auto& col : sampled.back()) cs.push_back(col[0]);
      const qm31 left = from_partial_evals(cs.data()), right = from_partial_evals(cs.data() + 4);
      qm31 x = oods.x;
      for (uint32_t i = 0; i + 1 < mldb; i++) x = q_double_x(x);
      const qm31 comp = qm31_add(left, qm31_mul(x, right));
      CS_CHECK_ARG(std::memcmp(&comp, &expected, sizeof(qm31)) == 0,
                   "prove: constraints not satisfied (ProvingError::ConstraintsNotSatisfied)");
    }
  }

  // --- the felt stream (CairoSerialize for StarkProof)
  words.clear();
  Words W{words};
  W.u(cfg.pow_bits);
  W.u(b);
  W.u(cfg.log_last_layer_degree_bound);
  W.u(cfg.n_queries);
  W.u(cfg.fold_step);
  W.u(trees.size() + 1);  // commitments
  W.h(pre_root);
  for (TreeCols& t : trees) W.h(t.tree.root);
  W.u(oods_pow);
  W.u(sampled.size());
  for (auto& tr : sampled) {
    W.u(tr.size());
    for (auto& col : tr) {
      W.u(col.size());
      for (const qm31& v : col) W.q(v);
    }
  }
  W.u(trees.size() + 1);  // decommitments
  W.u(0);
  for (TreeDec& d : tree_decs) W.hw(R.out, d.wit.first, d.wit.second);
  W.u(trees.size() + 1);  // queried values
  W.u(0);
  const size_t nq = queries.size();
  for (size_t t = 0; t < trees.size(); t++) {
    W.u(trees[t].cols.size());
    for (size_t c = 0; c < trees[t].cols.size(); c++) {
      W.u(nq);
      for (size_t i = 0; i < nq; i++) W.u(R.out[tree_decs[t].values_first + c * nq + i]);
    }
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
  W.u(cfg.log_last_layer_degree_bound);
  W.u(fri_pow);
  return CS_OK;
}

// ---------------------------------------------------------------- AIRs

// Wide-Fibonacci components (WideFibonacciEval, crates/examples/src/wide_fibonacci/mod.rs:87-97)
// and single-column LogUp components beside them.
struct FibLookupAir : Air {
  std::vector<uint32_t> n_cols, logs, lookup_logs;
  uint32_t* const* d_trace;
  const uint32_t* const* d_values;  // the LogUp components' looked-up values (trace domain)
  std::vector<std::vector<uint32_t*>> fib_evals;
  std::vector<uint32_t*> lookup_evals;
  std::vector<std::vector<uint32_t*>> inter_evals;
  qm31 z;

  cs_status trace(Prover& P, std::vector<Col>& cols) override {
    // every column of the tree in one interpolate and one evaluate call across sizes: the
    // Wide-Fibonacci columns in place, the LogUp value columns out of place (they stay for the
    // running sums)
    std::vector<const uint32_t*> src;
    std::vector<uint32_t*> coeffs;
    std::vector<uint32_t> tlogs;
    size_t c0 = 0;
    for (size_t k = 0; k < n_cols.size(); k++)
      for (uint32_t j = 0; j < n_cols[k]; j++, c0++) {
        src.push_back(d_trace[c0]);
        coeffs.push_back(d_trace[c0]);
        tlogs.push_back(logs[k]);
      }
    size_t lookup_words = 0;
    for (uint32_t l : lookup_logs) lookup_words += 1ull << l;
    uint32_t* lblk = lookup_words ? P.A.alloc(lookup_words) : nullptr;
    if (lookup_words && !lblk) return P.A.status;
    size_t off = 0;
    for (size_t k = 0; k < lookup_logs.size(); k++) {
      src.push_back(d_values[k]);
      coeffs.push_back(lblk + off);
      tlogs.push_back(lookup_logs[k]);
      off += 1ull << lookup_logs[k];
    }
    HP_TRY(P.interpolate_mixed(src, coeffs, tlogs));
    std::vector<uint32_t*> ev;
    HP_TRY(P.evaluate_mixed(coeffs, tlogs, ev));
    if (lblk) P.A.release(lblk);
    size_t i = 0;
    for (size_t k = 0; k < n_cols.size(); k++) {
      fib_evals.emplace_back(ev.begin() + i, ev.begin() + i + n_cols[k]);
      i += n_cols[k];
    }
    for (size_t k = 0; k < lookup_logs.size(); k++) lookup_evals.push_back(ev[i + k]);
    for (size_t j = 0; j < ev.size(); j++) cols.push_back({ev[j], tlogs[j] + P.cfg.b});
    return CS_OK;
  }
  bool has_interaction() const override { return !lookup_logs.empty(); }
  bool mix_claimed() const override { return true; }
  cs_status interaction(Prover& P, const qm31& zz, const qm31&, std::vector<Col>& cols, std::vector<bool>& two,
                        std::vector<qm31>& claimed) override {
    z = zz;
    const size_t n = lookup_logs.size();
    std::vector<uint32_t*> sums(4 * n);
    for (size_t k = 0; k < n; k++) {
      uint32_t* blk = P.A.alloc(4ull << lookup_logs[k]);
      if (!blk) return P.A.status;
      for (int c = 0; c < 4; c++) sums[4 * k + c] = blk + ((size_t)c << lookup_logs[k]);
    }
    uint32_t* d_claimed = P.A.alloc(4 * n);
    if (!d_claimed) return P.A.status;
    const uint32_t zw[4] = {z.a.a, z.a.b, z.b.a, z.b.b};
    std::vector<const uint32_t*> vals(d_values, d_values + n);
    if (P.cfg.plain) {
      for (size_t k = 0; k < n; k++) {
        uint32_t* out[4] = {sums[4 * k], sums[4 * k + 1], sums[4 * k + 2], sums[4 * k + 3]};
        HP_TRY(cs_logup_running_sum(vals[k], lookup_logs[k], zw, out, d_claimed + 4 * k, P.st));
      }
    } else {
      HP_TRY(cs_logup_running_sums((uint32_t)n, vals.data(), lookup_logs.data(), zw, sums.data(), d_claimed, P.st));
    }
    std::vector<uint32_t> cl(4 * n);
    CS_CUDA(cudaMemcpyAsync(cl.data(), d_claimed, 16 * n, cudaMemcpyDeviceToHost, P.st));
    CS_CUDA(cudaStreamSynchronize(P.st));
    claimed.clear();
    for (size_t k = 0; k < n; k++) claimed.push_back(qm31_make(cl[4 * k], cl[4 * k + 1], cl[4 * k + 2], cl[4 * k + 3]));
    // every running-sum coordinate of every component in one interpolate and one evaluate call
    std::vector<const uint32_t*> src(sums.begin(), sums.end());
    std::vector<uint32_t> slogs;
    for (size_t k = 0; k < n; k++) slogs.insert(slogs.end(), 4, lookup_logs[k]);
    HP_TRY(P.interpolate_mixed(src, sums, slogs));
    std::vector<uint32_t*> ev;
    HP_TRY(P.evaluate_mixed(sums, slogs, ev));
    for (size_t k = 0; k < n; k++) {
      inter_evals.emplace_back(ev.begin() + 4 * k, ev.begin() + 4 * k + 4);
      for (int c = 0; c < 4; c++) {
        cols.push_back({ev[4 * k + c], lookup_logs[k] + P.cfg.b});
        two.push_back(true);
      }
    }
    this->claimed = claimed;
    return CS_OK;
  }
  std::vector<qm31> claimed;
  uint32_t n_constraints() const override {
    uint32_t t = 0;
    for (uint32_t n : n_cols) t += n - 2;
    return t + (uint32_t)lookup_logs.size();
  }
  cs_status composition(Prover& P, const std::vector<qm31>& pw,
                        std::map<uint32_t, std::vector<uint32_t*>>& acc) override {
    const uint32_t total = n_constraints();
    uint32_t start = 0;
    for (size_t k = 0; k < n_cols.size(); k++) {  // each component takes the last powers, reversed
      const uint32_t n = n_cols[k] - 2, el = logs[k] + 1;
      std::vector<uint32_t> rc(4 * n);
      for (uint32_t j = 0; j < n; j++) {
        const qm31 x = pw[total - start - 1 - j];
        rc[4 * j] = x.a.a;
        rc[4 * j + 1] = x.a.b;
        rc[4 * j + 2] = x.b.a;
        rc[4 * j + 3] = x.b.b;
      }
      std::vector<const uint32_t*> ev(fib_evals[k].begin(), fib_evals[k].end());
      HP_TRY(cs_wide_fib_composition(ev.data(), n + 2, el, logs[k], rc.data(), P.acc_for(acc, el).data(), P.st));
      start += n;
    }
    // LogUp components of one size in one pass (cs_logup_compositions), in first-seen size order
    std::vector<uint32_t> order;
    for (uint32_t l : lookup_logs)
      if (std::find(order.begin(), order.end(), l) == order.end()) order.push_back(l);
    for (uint32_t l : order) {
      std::vector<const uint32_t*> vals, inter;
      std::vector<uint32_t> cl, rcs;
      for (size_t k = 0; k < lookup_logs.size(); k++) {
        if (lookup_logs[k] != l) continue;
        vals.push_back(lookup_evals[k]);
        for (int c = 0; c < 4; c++) inter.push_back(inter_evals[k][c]);
        const qm31 w = pw[total - start - 1 - (uint32_t)k];
        const uint32_t ww[4] = {w.a.a, w.a.b, w.b.a, w.b.b};
        const uint32_t cw[4] = {claimed[k].a.a, claimed[k].a.b, claimed[k].b.a, claimed[k].b.b};
        rcs.insert(rcs.end(), ww, ww + 4);
        cl.insert(cl.end(), cw, cw + 4);
      }
      const uint32_t zw[4] = {z.a.a, z.a.b, z.b.a, z.b.b};
      if (P.cfg.plain) {
        for (size_t j = 0; j < vals.size(); j++)
          HP_TRY(cs_logup_composition(vals[j], &inter[4 * j], l + 1, l, zw, &cl[4 * j], &rcs[4 * j],
                                      P.acc_for(acc, l + 1).data(), P.st));
      } else {
        HP_TRY(cs_logup_compositions((uint32_t)vals.size(), vals.data(), inter.data(), l + 1, l, zw, cl.data(),
                                     rcs.data(), P.acc_for(acc, l + 1).data(), P.st));
      }
    }
    return CS_OK;
  }
  bool at_point(const qpoint& oods, uint32_t mldb, const qm31& random_coeff,
                const std::vector<std::vector<std::vector<qm31>>>& sampled, qm31& expected) override {
    qm31 x = oods.x;
    for (uint32_t i = 0; i + 1 < mldb; i++) x = q_double_x(x);
    qm31 acc = qm31_make(0, 0, 0, 0);
    const auto& tr = sampled[1];
    size_t s0 = 0;
    for (size_t k = 0; k < n_cols.size(); k++) {
      for (uint32_t j = 0; j + 2 < n_cols[k]; j++) {
        const qm31 a = tr[s0 + j][0], bb = tr[s0 + j + 1][0], c = tr[s0 + j + 2][0];
        acc = qm31_add(qm31_mul(acc, random_coeff), qm31_sub(c, qm31_add(qm31_mul(a, a), qm31_mul(bb, bb))));
      }
      s0 += n_cols[k];
    }
    for (size_t k = 0; k < lookup_logs.size(); k++) {
      const qm31 v = tr[s0 + k][0];
      qm31 pe[4], ce[4];
      for (int c = 0; c < 4; c++) {
        pe[c] = sampled[2][4 * k + c][0];
        ce[c] = sampled[2][4 * k + c][1];
      }
      const qm31 shift = qm31_mul_m31(claimed[k], m31_inv(1u << lookup_logs[k]));
      const qm31 shifted = qm31_add(qm31_sub(from_partial_evals(ce), from_partial_evals(pe)), shift);
      const qm31 cons = qm31_add(qm31_mul(shifted, qm31_sub(v, z)), q1());
      acc = qm31_add(qm31_mul(acc, random_coeff), cons);
    }
    expected = qm31_mul(acc, qm31_inv(x));
    return true;
  }
};

// Components written against the constraint evaluator (FrameworkComponent, crates/constraint-framework/
// src/component.rs), their constraint quotients from kernels compiled at run time
// (cs_rtc_air_composition) and their constraints at the OODS point from a node program (the
// PointEvaluator's role, crates/constraint-framework/src/point.rs:12-64). A component with LogUp
// relations gets its interaction columns from its fraction kernel (cs_rtc_air_fractions) and the
// LogupTraceGenerator's column calls, after the lookup elements (z, alpha) are drawn; its
// parameters name z, the powers of alpha and the shift claimed sum / 2^n by kind.
struct RtcComponent {
  void* kernel = nullptr;
  uint32_t log_size = 0, col0 = 0, n_cols = 0, degree = 1;
  std::vector<std::vector<int32_t>> offs;  // per trace column
  std::vector<uint32_t> mask_cols, mask_trees, program, constraints, params, param_kinds;
  uint32_t n_batches = 0, inter0 = 0;
  std::vector<uint32_t> frac_cols;
  std::vector<bool> inter_two;
  // filled while proving
  std::vector<uint32_t*> inter_coeffs, inter_evals;
  qm31 claimed = qm31_make(0, 0, 0, 0);
  std::vector<uint32_t> resolved;  // the parameters' words once the lookup elements are drawn
};

struct RtcAir : Air {
  std::vector<RtcComponent> comps;
  uint32_t* const* d_trace = nullptr;
  bool mix = false;
  int32_t sub_e = 0;  // EvaluationMode: SubDomain's log_expansion, or -1 for ExtendToEvalDomain
  std::vector<uint32_t*> coeffs, evals;  // every trace column's coefficients and blown-up evaluations
  qm31 z = qm31_make(0, 0, 0, 0), alpha = qm31_make(0, 0, 0, 0);

  void resolve(RtcComponent& k, bool with_shift) const {
    // kinds: 0 the given value, 1 z, 2 the shift, 3 + i alpha^i
    k.resolved = k.params;
    for (size_t j = 0; j < k.param_kinds.size(); j++) {
      const uint32_t kind = k.param_kinds[j];
      qm31 v;
      if (kind == 0) continue;
      if (kind == 1) {
        v = z;
      } else if (kind == 2) {
        v = with_shift ? qm31_mul_m31(k.claimed, m31_inv(1u << k.log_size)) : qm31_make(0, 0, 0, 0);
      } else {
        v = qm31_make(1, 0, 0, 0);
        for (uint32_t i = 3; i < kind; i++) v = qm31_mul(v, alpha);
      }
      k.resolved[4 * j] = v.a.a;
      k.resolved[4 * j + 1] = v.a.b;
      k.resolved[4 * j + 2] = v.b.a;
      k.resolved[4 * j + 3] = v.b.b;
    }
  }
  bool any_relation() const {
    for (const RtcComponent& k : comps)
      if (k.n_batches) return true;
    return false;
  }

  cs_status trace(Prover& P, std::vector<Col>& cols) override {
    // the columns of a component with relations are interpolated out of place: its fraction
    // kernel reads their trace-domain values after the trace tree is committed
    std::vector<const uint32_t*> src;
    std::vector<uint32_t> tlogs;
    for (const RtcComponent& k : comps) {
      uint32_t* blk = nullptr;  // one block for the coefficients of a component with relations
      if (k.n_batches) {
        blk = P.A.alloc((size_t)k.n_cols << k.log_size);
        if (!blk) return P.A.status;
      }
      for (uint32_t j = 0; j < k.n_cols; j++) {
        src.push_back(d_trace[k.col0 + j]);
        tlogs.push_back(k.log_size);
        coeffs.push_back(blk ? blk + ((size_t)j << k.log_size) : d_trace[k.col0 + j]);
      }
    }
    HP_TRY(P.interpolate_mixed(src, coeffs, tlogs));
    HP_TRY(P.evaluate_mixed(coeffs, tlogs, evals));
    for (size_t j = 0; j < evals.size(); j++) cols.push_back({evals[j], tlogs[j] + P.cfg.b});
    return CS_OK;
  }
  void trace_offsets(std::vector<std::vector<int32_t>>& offs) const override {
    for (const RtcComponent& k : comps) offs.insert(offs.end(), k.offs.begin(), k.offs.end());
  }
  bool has_interaction() const override { return any_relation(); }
  bool mix_claimed() const override { return mix; }
  cs_status interaction(Prover& P, const qm31& zz, const qm31& aa, std::vector<Col>& cols, std::vector<bool>& two,
                        std::vector<qm31>& claimed) override {
    z = zz;
    alpha = aa;
    size_t n_rel = 0;
    for (RtcComponent& k : comps)
      if (k.n_batches) n_rel++;
    uint32_t* d_claimed = P.A.alloc(4 * n_rel);
    if (!d_claimed) return P.A.status;
    size_t r = 0;
    std::vector<const uint32_t*> src;
    std::vector<uint32_t*> dst;
    std::vector<uint32_t> slogs;
    uint32_t inter0 = 0;
    for (RtcComponent& k : comps) {
      if (!k.n_batches) continue;
      const uint32_t n = k.log_size, B = k.n_batches;
      resolve(k, false);
      uint32_t* fr = P.A.alloc((8ull * B) << n);
      uint32_t* ic = P.A.alloc((4ull * B) << n);
      if (!fr || !ic) return P.A.status;
      std::vector<const uint32_t*> fcols;
      for (uint32_t c : k.frac_cols) fcols.push_back(d_trace[k.col0 + c]);
      std::vector<uint32_t*> fout;
      for (uint32_t j = 0; j < 8 * B; j++) fout.push_back(fr + ((size_t)j << n));
      HP_TRY(cs_rtc_air_fractions(k.kernel, fcols.empty() ? nullptr : fcols.data(),
                                  k.resolved.empty() ? nullptr : k.resolved.data(), n, fout.data(), P.st));
      for (uint32_t j = 0; j < 4 * B; j++) k.inter_coeffs.push_back(ic + ((size_t)j << n));
      for (uint32_t b = 0; b < B; b++) {
        const uint32_t* num[4] = {fout[8 * b], fout[8 * b + 1], fout[8 * b + 2], fout[8 * b + 3]};
        const uint32_t* den[4] = {fout[8 * b + 4], fout[8 * b + 5], fout[8 * b + 6], fout[8 * b + 7]};
        const uint32_t* prev[4] = {nullptr, nullptr, nullptr, nullptr};
        if (b) for (int c = 0; c < 4; c++) prev[c] = k.inter_coeffs[4 * (b - 1) + c];
        uint32_t* out[4] = {k.inter_coeffs[4 * b], k.inter_coeffs[4 * b + 1], k.inter_coeffs[4 * b + 2],
                            k.inter_coeffs[4 * b + 3]};
        HP_TRY(cs_logup_gen_col(num, nullptr, den, b ? prev : nullptr, n, out, P.st));
      }
      uint32_t* last[4] = {k.inter_coeffs[4 * (B - 1)], k.inter_coeffs[4 * (B - 1) + 1],
                           k.inter_coeffs[4 * (B - 1) + 2], k.inter_coeffs[4 * (B - 1) + 3]};
      HP_TRY(cs_logup_finalize_last(last, n, d_claimed + 4 * r, P.st));
      P.A.release(fr);
      k.inter0 = inter0;
      inter0 += 4 * B;
      for (uint32_t* c : k.inter_coeffs) {
        src.push_back(c);
        dst.push_back(c);
        slogs.push_back(n);
      }
      r++;
    }
    std::vector<uint32_t> cl(4 * n_rel);
    CS_CUDA(cudaMemcpyAsync(cl.data(), d_claimed, 16 * n_rel, cudaMemcpyDeviceToHost, P.st));
    CS_CUDA(cudaStreamSynchronize(P.st));
    claimed.clear();
    r = 0;
    for (RtcComponent& k : comps) {
      if (!k.n_batches) continue;
      k.claimed = qm31_make(cl[4 * r], cl[4 * r + 1], cl[4 * r + 2], cl[4 * r + 3]);
      claimed.push_back(k.claimed);
      r++;
    }
    // every interaction column of every component in one interpolate and one evaluate call
    HP_TRY(P.interpolate_mixed(src, dst, slogs));
    std::vector<uint32_t*> ev;
    HP_TRY(P.evaluate_mixed(dst, slogs, ev));
    size_t e0 = 0;
    for (RtcComponent& k : comps) {
      if (!k.n_batches) continue;
      for (uint32_t j = 0; j < 4 * k.n_batches; j++) {
        k.inter_evals.push_back(ev[e0 + j]);
        cols.push_back({ev[e0 + j], k.log_size + P.cfg.b});
        two.push_back(k.inter_two[j]);
      }
      e0 += 4 * k.n_batches;
    }
    return CS_OK;
  }
  uint32_t n_constraints() const override {
    uint32_t n = 0;
    for (const RtcComponent& k : comps) n += (uint32_t)k.constraints.size();
    return n;
  }
  uint32_t log_expansion() const override { return sub_e > 0 ? (uint32_t)sub_e : 0; }
  cs_status composition(Prover& P, const std::vector<qm31>& pw,
                        std::map<uint32_t, std::vector<uint32_t*>>& acc) override {
    const uint32_t total = n_constraints();
    uint32_t start = 0;
    for (RtcComponent& k : comps) {  // each component takes the last powers, reversed
      const uint32_t n = (uint32_t)k.constraints.size(), el = k.log_size + k.degree;
      resolve(k, true);
      std::vector<uint32_t> rc(4 * (size_t)n);
      for (uint32_t j = 0; j < n; j++) {
        const qm31 x = pw[total - start - 1 - j];
        rc[4 * j] = x.a.a;
        rc[4 * j + 1] = x.a.b;
        rc[4 * j + 2] = x.b.a;
        rc[4 * j + 3] = x.b.b;
      }
      // get_trace_columns (component_prover.rs:29-56): in SubDomain mode the committed evaluations,
      // whose first 2^el rows are the evaluation domain; in ExtendToEvalDomain mode the columns on
      // CanonicCoset(el), the committed evaluations when that is their domain, else the
      // coefficients evaluated there
      std::vector<uint32_t*> tcols(evals.begin() + k.col0, evals.begin() + k.col0 + k.n_cols), icols = k.inter_evals;
      std::vector<uint32_t*> ext_t, ext_i;
      if (sub_e < 0 && el != k.log_size + P.cfg.b) {
        std::vector<uint32_t*> tc(coeffs.begin() + k.col0, coeffs.begin() + k.col0 + k.n_cols);
        HP_TRY(P.evaluate(tc, k.log_size, el, ext_t));
        tcols = ext_t;
        if (!k.inter_coeffs.empty()) {
          HP_TRY(P.evaluate(k.inter_coeffs, k.log_size, el, ext_i));
          icols = ext_i;
        }
      }
      std::vector<const uint32_t*> table;
      for (size_t i = 0; i < k.mask_cols.size(); i++)
        table.push_back(k.mask_trees[i] == 2 ? icols[k.mask_cols[i]] : tcols[k.mask_cols[i]]);
      HP_TRY(cs_rtc_air_composition_subdomain(k.kernel, table.data(), rc.data(),
                                              k.resolved.empty() ? nullptr : k.resolved.data(), el, k.log_size,
                                              sub_e > 0 ? (uint32_t)sub_e : 0, P.acc_for(acc, el).data(), P.st));
      if (!ext_t.empty()) P.A.release(ext_t[0]);
      if (!ext_i.empty()) P.A.release(ext_i[0]);
      start += n;
    }
    return CS_OK;
  }
  bool at_point(const qpoint& oods, uint32_t mldb, const qm31& random_coeff,
                const std::vector<std::vector<std::vector<qm31>>>& sampled, qm31& expected) override {
    // constraints of log degree 2 or more: no check, as the reference's lifted protocol fails it
    for (const RtcComponent& k : comps)
      if (k.degree > 1) return false;
    qm31 x = oods.x;
    for (uint32_t i = 0; i + 1 < mldb; i++) x = q_double_x(x);
    qm31 acc = qm31_make(0, 0, 0, 0);
    std::vector<qm31> v;
    for (RtcComponent& k : comps) {
      resolve(k, true);
      const size_t n_nodes = k.program.size() / 5;
      v.assign(n_nodes, qm31_make(0, 0, 0, 0));
      for (size_t i = 0; i < n_nodes; i++) {
        const uint32_t* nd = &k.program[5 * i];
        switch (nd[0]) {
          case 0:
            v[i] = nd[3] == 2 ? sampled[2][k.inter0 + nd[1]][nd[2]] : sampled[1][k.col0 + nd[1]][nd[2]];
            break;
          case 1: v[i] = qm31_make(nd[1] % P, 0, 0, 0); break;
          case 2: v[i] = qm31_make(k.resolved[4 * nd[1]], k.resolved[4 * nd[1] + 1], k.resolved[4 * nd[1] + 2],
                                   k.resolved[4 * nd[1] + 3]); break;
          case 3: {
            const qm31 parts[4] = {v[nd[1]], v[nd[2]], v[nd[3]], v[nd[4]]};
            v[i] = from_partial_evals(parts);
            break;
          }
          case 4: v[i] = qm31_sub(qm31_make(0, 0, 0, 0), v[nd[1]]); break;
          case 5: v[i] = qm31_add(v[nd[1]], v[nd[2]]); break;
          case 6: v[i] = qm31_sub(v[nd[1]], v[nd[2]]); break;
          default: v[i] = qm31_mul(v[nd[1]], v[nd[2]]); break;
        }
      }
      for (uint32_t c : k.constraints) acc = qm31_add(qm31_mul(acc, random_coeff), v[c]);
    }
    expected = qm31_mul(acc, qm31_inv(x));
    return true;
  }
};

// The Poseidon2 AIR (crates/examples/src/poseidon/mod.rs:320-379): 1264 trace columns generated on the
// device, 32 interaction columns (the last four also sampled at the previous row), constraint quotients
// on CanonicCoset(n + 2) (ExtendToEvalDomain). No sanity check: the reference's own prove of this AIR
// stops there (lifted protocol, constraint degree 5), and the proof is built as it computes it.
struct PoseidonAir : Air {
  static constexpr uint32_t kCols = 1264, kInter = 32, kConstraints = 1144, kExpand = 2;
  uint32_t log_n = 0;
  std::vector<uint32_t*> trace_vals, trace_coeffs, inter_coeffs;
  uint32_t lookup[8];
  qm31 claimed_sum;

  cs_status trace(Prover& P, std::vector<Col>& cols) override {
    const uint32_t n = log_n;
    uint32_t* blk = P.A.alloc((size_t)kCols << n);
    uint32_t* cblk = P.A.alloc((size_t)kCols << n);
    if (!blk || !cblk) return P.A.status;
    for (uint32_t j = 0; j < kCols; j++) {
      trace_vals.push_back(blk + ((size_t)j << n));
      trace_coeffs.push_back(cblk + ((size_t)j << n));
    }
    HP_TRY(cs_poseidon_trace(n, trace_vals.data(), P.st));
    std::vector<const uint32_t*> src(trace_vals.begin(), trace_vals.end());
    HP_TRY(cs_interpolate_columns_into(src.data(), trace_coeffs.data(), kCols, n, P.cfg.itw, P.cfg.tw_log, P.st));
    std::vector<uint32_t*> ev;
    HP_TRY(P.evaluate(trace_coeffs, n, n + P.cfg.b, ev));
    for (uint32_t* e : ev) cols.push_back({e, n + P.cfg.b});
    return CS_OK;
  }
  bool has_interaction() const override { return true; }
  cs_status interaction(Prover& P, const qm31& z, const qm31& alpha, std::vector<Col>& cols, std::vector<bool>& two,
                        std::vector<qm31>& claimed) override {
    const uint32_t n = log_n;
    const uint32_t lk[8] = {z.a.a, z.a.b, z.b.a, z.b.b, alpha.a.a, alpha.a.b, alpha.b.a, alpha.b.b};
    std::copy(lk, lk + 8, lookup);
    uint32_t* blk = P.A.alloc((size_t)kInter << n);
    if (!blk) return P.A.status;
    for (uint32_t j = 0; j < kInter; j++) inter_coeffs.push_back(blk + ((size_t)j << n));
    std::vector<const uint32_t*> src(trace_vals.begin(), trace_vals.end());
    uint32_t cs[4];
    HP_TRY(cs_poseidon_interaction(src.data(), n, lookup, inter_coeffs.data(), cs, P.st));
    P.A.release(trace_vals[0]);  // the trace values are no longer needed
    claimed_sum = qm31_make(cs[0], cs[1], cs[2], cs[3]);
    claimed = {claimed_sum};
    HP_TRY(P.interpolate(inter_coeffs, n));
    std::vector<uint32_t*> ev;
    HP_TRY(P.evaluate(inter_coeffs, n, n + P.cfg.b, ev));
    for (uint32_t j = 0; j < kInter; j++) {
      cols.push_back({ev[j], n + P.cfg.b});
      two.push_back(j >= kInter - 4);
    }
    return CS_OK;
  }
  uint32_t n_constraints() const override { return kConstraints; }
  cs_status composition(Prover& P, const std::vector<qm31>& pw,
                        std::map<uint32_t, std::vector<uint32_t*>>& acc) override {
    const uint32_t n = log_n, el = n + kExpand;
    // EvaluationMode::infer: constraint log degree 2 > log_blowup 1 -> ExtendToEvalDomain
    std::vector<uint32_t*> tev, iev;
    HP_TRY(P.evaluate(trace_coeffs, n, el, tev));
    HP_TRY(P.evaluate(inter_coeffs, n, el, iev));
    std::vector<uint32_t> rc(4 * kConstraints);
    for (uint32_t j = 0; j < kConstraints; j++) {
      const qm31 x = pw[kConstraints - 1 - j];
      rc[4 * j] = x.a.a;
      rc[4 * j + 1] = x.a.b;
      rc[4 * j + 2] = x.b.a;
      rc[4 * j + 3] = x.b.b;
    }
    const uint32_t cl[4] = {claimed_sum.a.a, claimed_sum.a.b, claimed_sum.b.a, claimed_sum.b.b};
    std::vector<const uint32_t*> t(tev.begin(), tev.end()), i(iev.begin(), iev.end());
    HP_TRY(cs_poseidon_composition(t.data(), i.data(), el, n, lookup, cl, rc.data(), P.acc_for(acc, el).data(), P.st));
    P.A.release(tev[0]);
    P.A.release(iev[0]);
    return CS_OK;
  }
};

}  // namespace hp
}  // namespace cs

using namespace cs;

extern "C" cs_status cs_host_blake2s(const uint8_t* msg, size_t n, uint8_t out[32]) {
  CS_CHECK_ARG((msg != nullptr || n == 0) && out != nullptr, "host_blake2s: null pointer");
  hp::blake2s_public(msg, n, out);
  return CS_OK;
}

namespace {

// This thread's proof words: the vector keeps its capacity across proofs.
std::vector<uint64_t>& proof_words() {
  thread_local std::vector<uint64_t> words;
  return words;
}

cs_status finish(std::vector<uint64_t>& words, uint64_t* h_words, size_t capacity, size_t* n_words) {
  *n_words = words.size();
  CS_CHECK_ARG(h_words == nullptr || capacity >= words.size(), "prove: %zu words do not fit in %zu", words.size(),
               capacity);
  if (h_words != nullptr) std::copy(words.begin(), words.end(), h_words);
  return CS_OK;
}

// max_blowup: the largest log blowup the AIR's evaluation supports (1 for the hand-written AIRs,
// whose constraints run on the committed evaluations)
cs_status check_common(const cs_wide_fib_proof_params& pp, uint32_t max_log, uint32_t max_blowup = 1) {
  CS_CHECK_ARG((pp.flags & ~(uint32_t)CS_PROVE_PLAIN) == 0, "prove: unknown flags 0x%x", pp.flags);
  CS_CHECK_ARG(pp.log_blowup_factor >= 1 && pp.log_blowup_factor <= max_blowup,
               "prove: log_blowup_factor %u outside [1, %u]", pp.log_blowup_factor, max_blowup);
  CS_CHECK_ARG(pp.d_twiddles != nullptr && pp.d_itwiddles != nullptr, "prove: null twiddles");
  CS_CHECK_ARG(pp.pow_bits <= 32 && pp.n_queries >= 1, "prove: bad FRI parameters");
  CS_CHECK_ARG(pp.lifting_log_size == max_log + pp.log_blowup_factor,
               "prove: lifting_log_size must be the largest evaluation size (%u)", max_log + pp.log_blowup_factor);
  CS_CHECK_ARG(pp.lifting_log_size > pp.log_last_layer_degree_bound + pp.log_blowup_factor + 1 &&
                   pp.lifting_log_size <= 28,
               "prove: lifting_log_size %u outside the FRI parameters' range", pp.lifting_log_size);
  CS_CHECK_ARG(pp.twiddle_log_size >= pp.lifting_log_size, "prove: twiddle tree too small");
  // the first layer's k folds must not go below the last layer (fri.rs:143-146)
  const uint32_t k = pp.fold_step ? pp.fold_step : 1;
  CS_CHECK_ARG(k <= 8 && pp.lifting_log_size >= pp.log_last_layer_degree_bound + pp.log_blowup_factor + k,
               "prove: fold_step %u outside [1, 8] or below the last layer", pp.fold_step);
  return CS_OK;
}

hp::ProofConfig config_of(const cs_wide_fib_proof_params& pp) {
  hp::ProofConfig c{pp.lifting_log_size, pp.log_blowup_factor, pp.pow_bits, pp.log_last_layer_degree_bound,
                    pp.n_queries, pp.d_twiddles, pp.d_itwiddles, pp.twiddle_log_size};
  c.plain = (pp.flags & CS_PROVE_PLAIN) != 0;
  c.fold_step = pp.fold_step ? pp.fold_step : 1;
  return c;
}

}  // namespace

extern "C" cs_status cs_prove_wide_fib(const cs_wide_fib_proof_params* params, uint32_t* const* d_trace,
                                       uint64_t* h_words, size_t capacity, size_t* n_words, cs_stream stream) {
  return cs_prove_fib_and_lookups(params, d_trace, 0, nullptr, nullptr, nullptr, h_words, capacity, n_words, stream);
}

extern "C" cs_status cs_prove_fib_and_lookups(const cs_wide_fib_proof_params* params, uint32_t* const* d_trace,
                                              uint32_t n_lookups, const uint32_t* const* d_values,
                                              const uint32_t* h_lookup_log_sizes, uint32_t* h_claimed,
                                              uint64_t* h_words, size_t capacity, size_t* n_words,
                                              cs_stream stream) {
  CS_CHECK_ARG(params != nullptr && d_trace != nullptr && n_words != nullptr, "prove: null pointer");
  const cs_wide_fib_proof_params& pp = *params;
  CS_CHECK_ARG(pp.n_components >= 1 && pp.n_cols != nullptr && pp.log_sizes != nullptr, "prove: no components");
  CS_CHECK_ARG(n_lookups == 0 || (d_values != nullptr && h_lookup_log_sizes != nullptr && h_claimed != nullptr),
               "prove: null lookup table");
  uint32_t max_log = 0, n_total = 0;
  for (uint32_t k = 0; k < pp.n_components; k++) {
    CS_CHECK_ARG(pp.n_cols[k] >= 3 && pp.log_sizes[k] >= 1, "prove: component %u: %u columns of 2^%u", k,
                 pp.n_cols[k], pp.log_sizes[k]);
    max_log = std::max(max_log, pp.log_sizes[k]);
    n_total += pp.n_cols[k];
  }
  for (uint32_t c = 0; c < n_total; c++) CS_CHECK_ARG(d_trace[c] != nullptr, "prove: column %u is null", c);
  for (uint32_t k = 0; k < n_lookups; k++) {
    CS_CHECK_ARG(d_values[k] != nullptr && h_lookup_log_sizes[k] >= 1, "prove: lookup %u is empty", k);
    max_log = std::max(max_log, h_lookup_log_sizes[k]);
  }
  const cs_status cs = check_common(pp, max_log);
  if (cs != CS_OK) return cs;
  hp::FibLookupAir air;
  air.n_cols.assign(pp.n_cols, pp.n_cols + pp.n_components);
  air.logs.assign(pp.log_sizes, pp.log_sizes + pp.n_components);
  if (n_lookups) air.lookup_logs.assign(h_lookup_log_sizes, h_lookup_log_sizes + n_lookups);
  air.d_trace = d_trace;
  air.d_values = d_values;
  std::vector<uint64_t>& words = proof_words();
  std::vector<qm31> claimed;
  const cs_status s = hp::prove(config_of(pp), air, words, claimed, to_stream(stream));
  if (s != CS_OK) return s;
  for (uint32_t k = 0; k < n_lookups; k++) {
    h_claimed[4 * k] = claimed[k].a.a;
    h_claimed[4 * k + 1] = claimed[k].a.b;
    h_claimed[4 * k + 2] = claimed[k].b.a;
    h_claimed[4 * k + 3] = claimed[k].b.b;
  }
  return finish(words, h_words, capacity, n_words);
}

extern "C" cs_status cs_prove_air(const cs_wide_fib_proof_params* params, const cs_air_component* components,
                                  uint32_t n_components, uint32_t* const* d_trace, uint64_t* h_words, size_t capacity,
                                  size_t* n_words, cs_stream stream) {
  CS_CHECK_ARG(params != nullptr && components != nullptr && d_trace != nullptr && n_words != nullptr,
               "prove_air: null pointer");
  CS_CHECK_ARG(n_components >= 1, "prove_air: no components");
  hp::RtcAir air;
  air.d_trace = d_trace;
  air.mix = (params->flags & CS_PROVE_MIX_CLAIMED) != 0;
  uint32_t max_log = 0, col0 = 0;
  for (uint32_t k = 0; k < n_components; k++) {
    const cs_air_component& c = components[k];
    CS_CHECK_ARG(c.kernel != nullptr && c.log_size >= 1 && c.log_size <= 27 && c.n_cols >= 1,
                 "prove_air: component %u: kernel, 2^%u rows, %u columns", k, c.log_size, c.n_cols);
    CS_CHECK_ARG(c.constraint_log_degree == 1 || c.constraint_log_degree == 2,
                 "prove_air: component %u: constraint log degree %u (1 or 2)", k, c.constraint_log_degree);
    CS_CHECK_ARG(c.offsets_start != nullptr && (c.offsets != nullptr || c.offsets_start[c.n_cols] == 0),
                 "prove_air: component %u: null offsets", k);
    CS_CHECK_ARG(c.n_nodes == 0 || c.program != nullptr, "prove_air: component %u: null program", k);
    CS_CHECK_ARG(c.n_constraints == 0 || c.constraints != nullptr, "prove_air: component %u: null constraints", k);
    CS_CHECK_ARG(c.n_masks == 0 || (c.mask_cols != nullptr && c.mask_trees != nullptr),
                 "prove_air: component %u: null mask table", k);
    CS_CHECK_ARG(c.n_params == 0 || (c.params != nullptr && c.param_kinds != nullptr),
                 "prove_air: component %u: null parameters", k);
    CS_CHECK_ARG(c.n_batches <= 1024 && (c.n_batches == 0 || (c.inter_two != nullptr &&
                                                             (c.n_frac_cols == 0 || c.frac_cols != nullptr))),
                 "prove_air: component %u: relation tables", k);
    uint32_t kc = 0, kn = 0, kp = 0;
    const cs_status shape = cs_rtc_kernel_shape(c.kernel, &kc, &kn, &kp);
    if (shape != CS_OK) return shape;
    CS_CHECK_ARG(kc == c.n_masks && kn == c.n_constraints && kp == c.n_params,
                 "prove_air: component %u: the kernel has %u masks, %u constraints, %u parameters", k, kc, kn, kp);
    hp::RtcComponent rc;
    rc.kernel = c.kernel;
    rc.log_size = c.log_size;
    rc.degree = c.constraint_log_degree;
    rc.col0 = col0;
    rc.n_cols = c.n_cols;
    rc.n_batches = c.n_batches;
    for (uint32_t j = 0; j < c.n_cols; j++) {
      CS_CHECK_ARG(c.offsets_start[j] <= c.offsets_start[j + 1], "prove_air: component %u: offsets out of order", k);
      rc.offs.emplace_back(c.offsets + c.offsets_start[j], c.offsets + c.offsets_start[j + 1]);
      for (int32_t o : rc.offs.back())
        CS_CHECK_ARG(o > -(1 << 20) && o < (1 << 20), "prove_air: component %u: offset %d", k, o);
    }
    for (uint32_t j = 0; j < 4 * c.n_batches; j++) rc.inter_two.push_back(c.inter_two[j] != 0);
    rc.frac_cols.assign(c.frac_cols, c.frac_cols + c.n_frac_cols);
    for (uint32_t f : rc.frac_cols) CS_CHECK_ARG(f < c.n_cols, "prove_air: component %u: fraction column %u", k, f);
    rc.mask_cols.assign(c.mask_cols, c.mask_cols + c.n_masks);
    rc.mask_trees.assign(c.mask_trees, c.mask_trees + c.n_masks);
    for (uint32_t i = 0; i < c.n_masks; i++) {
      const bool inter = rc.mask_trees[i] == 2;
      CS_CHECK_ARG((rc.mask_trees[i] == 1 && rc.mask_cols[i] < c.n_cols) ||
                       (inter && rc.mask_cols[i] < 4 * c.n_batches),
                   "prove_air: component %u: mask %u reads column %u of tree %u", k, i, rc.mask_cols[i],
                   rc.mask_trees[i]);
    }
    rc.program.assign(c.program, c.program + 5 * (size_t)c.n_nodes);
    // every operand names an earlier node, every sampled value a column and one of its samples
    for (uint32_t i = 0; i < c.n_nodes; i++) {
      const uint32_t* nd = &rc.program[5 * (size_t)i];
      CS_CHECK_ARG(nd[0] <= 7, "prove_air: component %u: node %u: op %u", k, i, nd[0]);
      const uint32_t n_in = nd[0] == 3 ? 4 : nd[0] == 4 ? 1 : nd[0] >= 5 ? 2 : 0;
      for (uint32_t a = 0; a < n_in; a++)
        CS_CHECK_ARG(nd[1 + a] < i, "prove_air: component %u: node %u reads node %u", k, i, nd[1 + a]);
      if (nd[0] == 0 && nd[3] == 2)
        CS_CHECK_ARG(nd[1] < 4 * c.n_batches && nd[2] < (rc.inter_two[nd[1]] ? 2u : 1u),
                     "prove_air: component %u: node %u: interaction column %u sample %u", k, i, nd[1], nd[2]);
      else if (nd[0] == 0)
        CS_CHECK_ARG(nd[3] <= 1 && nd[1] < c.n_cols && nd[2] < rc.offs[nd[1]].size(),
                     "prove_air: component %u: node %u: column %u offset %u", k, i, nd[1], nd[2]);
      if (nd[0] == 2) CS_CHECK_ARG(nd[1] < c.n_params, "prove_air: component %u: node %u: parameter %u", k, i, nd[1]);
    }
    rc.constraints.assign(c.constraints, c.constraints + c.n_constraints);
    for (uint32_t x : rc.constraints) CS_CHECK_ARG(x < c.n_nodes, "prove_air: component %u: constraint node %u", k, x);
    rc.params.assign(c.params, c.params + 4 * (size_t)c.n_params);
    rc.param_kinds.assign(c.param_kinds, c.param_kinds + c.n_params);
    for (uint32_t j = 0; j < c.n_cols; j++)
      CS_CHECK_ARG(d_trace[col0 + j] != nullptr, "prove_air: column %u is null", col0 + j);
    max_log = std::max(max_log, c.log_size + c.constraint_log_degree - 1);
    col0 += c.n_cols;
    air.comps.push_back(std::move(rc));
  }
  // EvaluationMode::infer (accumulation.rs:42-62): SubDomain when every component's constraint log
  // degree is at most the blowup, by the same log_expansion; else ExtendToEvalDomain
  const uint32_t b = params->log_blowup_factor;
  air.sub_e = -2;
  for (const hp::RtcComponent& rc : air.comps) {
    const int32_t e = rc.degree > b ? -1 : (int32_t)(b - rc.degree);
    if (e < 0 || (air.sub_e != -2 && air.sub_e != e)) {
      air.sub_e = -1;
      break;
    }
    air.sub_e = e;
  }
  cs_wide_fib_proof_params pp = *params;
  pp.flags &= ~CS_PROVE_MIX_CLAIMED;
  const cs_status cs = check_common(pp, max_log, 16);
  if (cs != CS_OK) return cs;
  std::vector<uint64_t>& words = proof_words();
  std::vector<qm31> claimed;
  const cs_status s = hp::prove(config_of(pp), air, words, claimed, to_stream(stream));
  if (s != CS_OK) return s;
  return finish(words, h_words, capacity, n_words);
}

extern "C" cs_status cs_prove_poseidon(uint32_t log_n_rows, const cs_wide_fib_proof_params* params,
                                       uint64_t* h_words, size_t capacity, size_t* n_words, cs_stream stream) {
  CS_CHECK_ARG(params != nullptr && n_words != nullptr, "prove_poseidon: null pointer");
  CS_CHECK_ARG(log_n_rows >= 1 && log_n_rows <= 22, "prove_poseidon: log_n_rows %u outside [1, 22]", log_n_rows);
  // poseidon_pcs_config (mod.rs:305-318): the tree height is log_n_rows + 2 - 1 + log_blowup
  const cs_status cs = check_common(*params, log_n_rows + 1);
  if (cs != CS_OK) return cs;
  hp::PoseidonAir air;
  air.log_n = log_n_rows;
  std::vector<uint64_t>& words = proof_words();
  std::vector<qm31> claimed;
  const cs_status s = hp::prove(config_of(*params), air, words, claimed, to_stream(stream));
  if (s != CS_OK) return s;
  return finish(words, h_words, capacity, n_words);
}

// ---------------------------------------------------------------- GKR batch prover
// prove_batch (crates/stwo/src/prover/lookups/gkr_prover.rs) and its sum-check
// (crates/stwo/src/prover/lookups/sumcheck.rs) in native code over this library's
// GkrOps / MleOps kernels: per sum-check round the device sums of every active
// instance are read back once, the round polynomials and the channel run here,
// and the variable is fixed on the device. The values equal
// proving_gb300.gkr.prove_batch's.

namespace cs {
namespace hp {
namespace {

// One column of a GKR layer: 4 coordinate pointers, or one for base values.
struct GCol {
  const uint32_t* c[4] = {nullptr, nullptr, nullptr, nullptr};
  bool base = false;
  uint32_t* owned = nullptr;  // the allocation holding the coordinates, when this driver made it
};
struct GLayer {
  uint32_t kind = CS_GKR_GRAND_PRODUCT;
  uint32_t n_vars = 0;
  GCol num, den;  // a grand product keeps its column in den
};

const qm31 kOne = qm31_make(1, 0, 0, 0);
const qm31 kZero = qm31_make(0, 0, 0, 0);

bool q_eq(const qm31& a, const qm31& b) { return a.a.a == b.a.a && a.a.b == b.a.b && a.b.a == b.b.a && a.b.b == b.b.b; }
bool q_zero(const qm31& a) { return q_eq(a, kZero); }

qm31 eq1(const qm31& x, const qm31& y) {  // eq for one variable (utils.rs eq)
  return qm31_add(qm31_mul(x, y), qm31_mul(qm31_sub(kOne, x), qm31_sub(kOne, y)));
}

// inverses of nonzero values with one inversion; false when one is zero
bool batch_inverse(std::vector<qm31>& xs) {
  std::vector<qm31> pre(xs.size());
  qm31 acc = kOne;
  for (size_t i = 0; i < xs.size(); i++) {
    if (q_zero(xs[i])) return false;
    pre[i] = acc;
    acc = qm31_mul(acc, xs[i]);
  }
  qm31 inv = qm31_inv(acc);
  for (size_t i = xs.size(); i-- > 0;) {
    const qm31 x = xs[i];
    xs[i] = qm31_mul(inv, pre[i]);
    inv = qm31_mul(inv, x);
  }
  return true;
}

using Poly = std::vector<qm31>;

Poly poly_trim(Poly p) {
  while (!p.empty() && q_zero(p.back())) p.pop_back();
  return p;
}
qm31 poly_eval(const Poly& p, const qm31& x) {
  qm31 acc = kZero;
  for (size_t i = p.size(); i-- > 0;) acc = qm31_add(qm31_mul(acc, x), p[i]);
  return acc;
}

// correct_sum_as_poly_in_first_variable for every k = 1..|y| (see RoundConstants in
// proving_gb300/gkr.py): r(t) = (t - b_k) q(t), q through (x, r(x) / (x - b_k)), x = 0, 1, 2.
struct RoundConstants {
  std::vector<qm31> a, b, eq0, eq2, i0, i1, i2;  // index k
  bool ok = true;
  explicit RoundConstants(const std::vector<qm31>& y) {
    const size_t n = y.size();
    a.resize(n + 1), b.resize(n + 1), eq0.resize(n + 1), eq2.resize(n + 1);
    i0.resize(n + 1), i1.resize(n + 1), i2.resize(n + 1);
    std::vector<qm31> prefix(n);
    qm31 acc = kOne;
    for (size_t i = 0; i < n; i++) prefix[i] = acc = qm31_mul(acc, qm31_sub(kOne, y[i]));
    std::vector<qm31> inv;
    for (size_t k = 1; k <= n; k++) inv.push_back(prefix[n - k]);
    for (size_t k = 1; k <= n; k++) inv.push_back(qm31_sub(kOne, qm31_add(y[n - k], y[n - k])));
    if (!(ok = batch_inverse(inv))) return;
    std::vector<qm31> xb;
    for (size_t k = 1; k <= n; k++) {
      a[k] = inv[k - 1];
      b[k] = qm31_mul(qm31_sub(kOne, y[n - k]), inv[n + k - 1]);
      eq0[k] = eq1(kZero, y[n - k]);
      eq2[k] = eq1(qm31_make(2, 0, 0, 0), y[n - k]);
      for (uint32_t x = 0; x < 3; x++) xb.push_back(qm31_sub(qm31_make(x, 0, 0, 0), b[k]));
    }
    if (!(ok = batch_inverse(xb))) return;
    for (size_t k = 1; k <= n; k++) i0[k] = xb[3 * (k - 1)], i1[k] = xb[3 * (k - 1) + 1], i2[k] = xb[3 * (k - 1) + 2];
  }
  Poly correct(const qm31& f0, const qm31& f2, const qm31& claim, size_t k) const {
    const qm31 r0 = qm31_mul(qm31_mul(f0, eq0[k]), a[k]);
    const qm31 r1 = qm31_sub(claim, r0);
    const qm31 r2 = qm31_mul(qm31_mul(f2, eq2[k]), a[k]);
    const qm31 q0 = qm31_mul(r0, i0[k]), q1 = qm31_mul(r1, i1[k]), q2 = qm31_mul(r2, i2[k]);
    const qm31 c2 = qm31_mul_m31(qm31_add(qm31_sub(q2, qm31_add(q1, q1)), q0), (P + 1) / 2);
    const qm31 c1 = qm31_sub(qm31_sub(q1, q0), c2);
    return poly_trim({qm31_neg(qm31_mul(b[k], q0)), qm31_sub(q0, qm31_mul(b[k], c1)), qm31_sub(c1, qm31_mul(b[k], c2)), c2});
  }
};

struct Oracle {
  GLayer layer;  // the input layer, n_vars = oracle variables + 1
  qm31 corr = kOne;
  qm31 lambda;
  uint32_t n_vars() const { return layer.n_vars - 1; }
};

struct GkrProver {
  Channel& ch;
  Arena& ar;
  cudaStream_t st;

  GCol alloc_secure(uint32_t log_n) {
    GCol col;
    uint32_t* p = ar.alloc(4ull << log_n);
    if (p == nullptr) return col;
    for (int k = 0; k < 4; k++) col.c[k] = p + ((size_t)k << log_n);
    col.owned = p;
    return col;
  }
  void drop(GCol& col) {
    if (col.owned != nullptr) ar.release(col.owned);
    col.owned = nullptr;
  }
  // values 0 .. n-1 of the columns, read back in one synchronisation
  cs_status read(const std::vector<std::pair<const GCol*, uint32_t>>& reqs, std::vector<std::vector<qm31>>& out) {
    std::vector<std::vector<uint32_t>> raw(reqs.size());
    for (size_t r = 0; r < reqs.size(); r++) {
      const GCol& col = *reqs[r].first;
      const uint32_t n = reqs[r].second;
      raw[r].assign(4 * n, 0);
      for (int k = 0; k < (col.base ? 1 : 4); k++)
        CS_CUDA(cudaMemcpyAsync(raw[r].data() + k * n, col.c[k], 4 * n, cudaMemcpyDeviceToHost, st));
    }
    CS_CUDA(cudaStreamSynchronize(st));
    out.assign(reqs.size(), {});
    for (size_t r = 0; r < reqs.size(); r++) {
      const uint32_t n = reqs[r].second;
      for (uint32_t i = 0; i < n; i++)
        out[r].push_back(qm31_make(raw[r][i], raw[r][n + i], raw[r][2 * n + i], raw[r][3 * n + i]));
    }
    return CS_OK;
  }
  static void tables(const GCol& col, const uint32_t* t[4]) {
    for (int k = 0; k < 4; k++) t[k] = col.base ? col.c[0] : col.c[k];
  }

  cs_status next_layer(const GLayer& in, GLayer& out) {
    out.n_vars = in.n_vars - 1;
    out.kind = in.kind == CS_GKR_GRAND_PRODUCT ? CS_GKR_GRAND_PRODUCT : CS_GKR_LOGUP_GENERIC;
    out.den = alloc_secure(out.n_vars);
    if (out.den.owned == nullptr) return CS_ERR_OOM;
    uint32_t* od[4] = {const_cast<uint32_t*>(out.den.c[0]), const_cast<uint32_t*>(out.den.c[1]),
                       const_cast<uint32_t*>(out.den.c[2]), const_cast<uint32_t*>(out.den.c[3])};
    const uint32_t *n[4], *d[4];
    tables(in.num, n);
    tables(in.den, d);
    if (in.kind == CS_GKR_GRAND_PRODUCT) return cs_gkr_next_layer(in.kind, nullptr, d, in.n_vars, nullptr, od, st);
    out.num = alloc_secure(out.n_vars);
    if (out.num.owned == nullptr) return CS_ERR_OOM;
    uint32_t* on[4] = {const_cast<uint32_t*>(out.num.c[0]), const_cast<uint32_t*>(out.num.c[1]),
                       const_cast<uint32_t*>(out.num.c[2]), const_cast<uint32_t*>(out.num.c[3])};
    return cs_gkr_next_layer(in.kind, in.kind == CS_GKR_LOGUP_SINGLES ? nullptr : n, d, in.n_vars, on, od, st);
  }

  cs_status fix(const GCol& src, uint32_t log_n, const qm31& x, GCol& dst) {
    dst = alloc_secure(log_n - 1);
    if (dst.owned == nullptr) return CS_ERR_OOM;
    const uint32_t* s[4];
    tables(src, s);
    uint32_t* d[4] = {const_cast<uint32_t*>(dst.c[0]), const_cast<uint32_t*>(dst.c[1]), const_cast<uint32_t*>(dst.c[2]),
                      const_cast<uint32_t*>(dst.c[3])};
    const uint32_t a[4] = {x.a.a, x.a.b, x.b.a, x.b.b};
    return cs_mle_fix_first_variable(s, src.base ? 1 : 0, log_n, a, d, st);
  }

  // Oracle::fix_first_variable: the eq correction and every column of the layer
  cs_status fix_oracle(Oracle& o, const std::vector<qm31>& y, const qm31& x) {
    const qm31 z0 = y[y.size() - o.n_vars()];
    o.corr = qm31_mul(o.corr, eq1(x, z0));
    GLayer next;
    next.n_vars = o.layer.n_vars - 1;
    next.kind = o.layer.kind == CS_GKR_LOGUP_MULTIPLICITIES ? CS_GKR_LOGUP_GENERIC : o.layer.kind;
    if (o.layer.kind == CS_GKR_LOGUP_GENERIC || o.layer.kind == CS_GKR_LOGUP_MULTIPLICITIES)
      HP_TRY(fix(o.layer.num, o.layer.n_vars, x, next.num));
    HP_TRY(fix(o.layer.den, o.layer.n_vars, x, next.den));
    drop(o.layer.num);  // only what an earlier round of this sum-check made
    drop(o.layer.den);
    o.layer = next;
    return CS_OK;
  }

  cs_status sumcheck(std::vector<qm31> claims, std::vector<Oracle>& oracles, const qm31& lam, const GCol& eq,
                     const std::vector<qm31>& y, const RoundConstants& rc, std::vector<Poly>& round_polys,
                     std::vector<qm31>& assignment) {
    uint32_t n_vars = 0;
    for (const Oracle& o : oracles) n_vars = std::max(n_vars, o.n_vars());
    for (size_t i = 0; i < oracles.size(); i++)
      claims[i] = qm31_mul_m31(claims[i], (uint32_t)((1ull << (n_vars - oracles[i].n_vars())) % P));
    uint32_t* d_sums = ar.alloc(8 * oracles.size());
    if (d_sums == nullptr) return CS_ERR_OOM;
    std::vector<uint32_t> sums(8 * oracles.size());
    const uint32_t* e[4];
    tables(eq, e);
    for (uint32_t rnd = 0; rnd < n_vars; rnd++) {
      const uint32_t remaining = n_vars - rnd;
      std::vector<size_t> active;
      for (size_t i = 0; i < oracles.size(); i++) {
        if (oracles[i].n_vars() != remaining) continue;
        const GLayer& L = oracles[i].layer;
        const uint32_t *n[4], *d[4];
        tables(L.num, n);
        tables(L.den, d);
        const uint32_t l4[4] = {oracles[i].lambda.a.a, oracles[i].lambda.a.b, oracles[i].lambda.b.a,
                                oracles[i].lambda.b.b};
        const bool has_num = L.kind == CS_GKR_LOGUP_GENERIC || L.kind == CS_GKR_LOGUP_MULTIPLICITIES;
        HP_TRY(cs_gkr_sum_as_poly(L.kind, e, has_num ? n : nullptr, d, L.n_vars, l4, d_sums + 8 * active.size(), st));
        active.push_back(i);
      }
      if (!active.empty()) {
        CS_CUDA(cudaMemcpyAsync(sums.data(), d_sums, 32 * active.size(), cudaMemcpyDeviceToHost, st));
        CS_CUDA(cudaStreamSynchronize(st));
      }
      std::vector<Poly> polys;
      for (size_t i = 0, j = 0; i < oracles.size(); i++) {
        Poly p;
        if (j < active.size() && active[j] == i) {
          const uint32_t* w = sums.data() + 8 * j++;
          const qm31 f0 = qm31_mul(qm31_make(w[0], w[1], w[2], w[3]), oracles[i].corr);
          const qm31 f2 = qm31_mul(qm31_make(w[4], w[5], w[6], w[7]), oracles[i].corr);
          p = rc.correct(f0, f2, claims[i], oracles[i].n_vars());
        } else {
          p = poly_trim({qm31_mul_m31(claims[i], (P + 1) / 2)});
        }
        CS_CHECK_ARG(q_eq(qm31_add(poly_eval(p, kZero), poly_eval(p, kOne)), claims[i]) && p.size() <= 4,
                     "gkr_prove_batch: round polynomial inconsistent with its claim (instance %zu, round %u)", i,
                     rnd);
        polys.push_back(p);
      }
      Poly comb;  // p_0 + lam p_1 + ..., no trimming
      for (size_t i = polys.size(); i-- > 0;) {
        Poly next(std::max(comb.size(), polys[i].size()), kZero);
        for (size_t t = 0; t < comb.size(); t++) next[t] = qm31_mul(comb[t], lam);
        for (size_t t = 0; t < polys[i].size(); t++) next[t] = qm31_add(next[t], polys[i][t]);
        comb = next;
      }
      ch.mix_felts(comb);
      const qm31 x = ch.draw_secure_felt();
      for (size_t i = 0; i < oracles.size(); i++) claims[i] = poly_eval(polys[i], x);
      for (size_t i : active) HP_TRY(fix_oracle(oracles[i], y, x));
      round_polys.push_back(comb);
      assignment.push_back(x);
    }
    ar.release(d_sums);
    return CS_OK;
  }

  // prove_batch; the proof and artifact go to `out` in the layout of cs_gkr_prove_batch
  cs_status prove(const std::vector<GLayer>& inputs, Words& out) {
    const size_t n_inst = inputs.size();
    uint32_t n_layers = 0;
    for (const GLayer& L : inputs) n_layers = std::max(n_layers, L.n_vars);
    std::vector<std::vector<GLayer>> layers(n_inst);
    for (size_t i = 0; i < n_inst; i++) {
      layers[i].push_back(inputs[i]);
      while (layers[i].back().n_vars > 0) {
        GLayer next;
        HP_TRY(next_layer(layers[i].back(), next));
        layers[i].push_back(next);
      }
    }
    std::vector<int> cursor(n_inst);  // next layer of each instance, from the output layer down
    for (size_t i = 0; i < n_inst; i++) cursor[i] = (int)inputs[i].n_vars;
    std::vector<std::vector<Poly>> proofs;
    std::vector<std::vector<std::vector<std::pair<qm31, qm31>>>> masks(n_inst);
    std::vector<std::vector<qm31>> outputs(n_inst), claims(n_inst);
    std::vector<bool> has_claims(n_inst, false);
    std::vector<qm31> ood;
    for (uint32_t layer = 0; layer < n_layers; layer++) {
      const uint32_t remaining = n_layers - layer;
      for (size_t i = 0; i < n_inst; i++) {
        if (inputs[i].n_vars != remaining) continue;
        const GLayer& L = layers[i][cursor[i]--];
        std::vector<std::vector<qm31>> v;
        if (L.kind == CS_GKR_GRAND_PRODUCT || L.kind == CS_GKR_LOGUP_SINGLES) {
          HP_TRY(read({{&L.den, 1}}, v));
          claims[i] = L.kind == CS_GKR_GRAND_PRODUCT ? std::vector<qm31>{v[0][0]} : std::vector<qm31>{kOne, v[0][0]};
        } else {
          HP_TRY(read({{&L.num, 1}, {&L.den, 1}}, v));
          claims[i] = {v[0][0], v[1][0]};
        }
        outputs[i] = claims[i];
        has_claims[i] = true;
      }
      for (size_t i = 0; i < n_inst; i++)
        if (has_claims[i]) ch.mix_felts(claims[i]);
      // EqEvals::generate(ood)
      GCol eq = alloc_secure(ood.empty() ? 0 : (uint32_t)ood.size() - 1);
      if (eq.owned == nullptr) return CS_ERR_OOM;
      uint32_t* eqo[4] = {const_cast<uint32_t*>(eq.c[0]), const_cast<uint32_t*>(eq.c[1]), const_cast<uint32_t*>(eq.c[2]),
                          const_cast<uint32_t*>(eq.c[3])};
      if (ood.empty()) {
        const uint32_t one[4] = {1, 0, 0, 0};
        for (int k = 0; k < 4; k++) CS_CUDA(cudaMemcpyAsync(eqo[k], one + k, 4, cudaMemcpyHostToDevice, st));
        CS_CUDA(cudaStreamSynchronize(st));  // the host words live on this stack frame
      } else {
        std::vector<uint32_t> yw;
        for (size_t j = 1; j < ood.size(); j++) yw.insert(yw.end(), {ood[j].a.a, ood[j].a.b, ood[j].b.a, ood[j].b.b});
        const qm31 v = eq1(kZero, ood[0]);
        const uint32_t v4[4] = {v.a.a, v.a.b, v.b.a, v.b.b};
        HP_TRY(cs_gkr_gen_eq_evals(yw.empty() ? nullptr : yw.data(), (uint32_t)ood.size() - 1, v4, eqo, st));
      }
      const RoundConstants rc(ood);
      CS_CHECK_ARG(rc.ok, "gkr_prove_batch: division by zero in the round constants");
      const qm31 alpha = ch.draw_secure_felt();
      const qm31 lam = ch.draw_secure_felt();
      std::vector<Oracle> oracles;
      std::vector<qm31> sc_claims;
      std::vector<size_t> sc_inst;
      for (size_t i = 0; i < n_inst; i++) {
        if (!has_claims[i]) continue;
        Oracle o;
        o.layer = layers[i][cursor[i]--];
        o.layer.num.owned = o.layer.den.owned = nullptr;  // the layer stack keeps its buffers
        o.lambda = lam;
        oracles.push_back(o);
        qm31 c = kZero;  // random_linear_combination (horner)
        for (size_t t = claims[i].size(); t-- > 0;) c = qm31_add(qm31_mul(c, lam), claims[i][t]);
        sc_claims.push_back(c);
        sc_inst.push_back(i);
      }
      std::vector<Poly> round_polys;
      std::vector<qm31> sc_ood;
      HP_TRY(sumcheck(sc_claims, oracles, alpha, eq, ood, rc, round_polys, sc_ood));
      proofs.push_back(round_polys);
      // masks of the constant oracles, one read for all
      std::vector<std::pair<const GCol*, uint32_t>> reqs;
      for (const Oracle& o : oracles) {
        CS_CHECK_ARG(o.layer.kind != CS_GKR_LOGUP_MULTIPLICITIES, "gkr_prove_batch: mask of a multiplicities layer");
        if (o.layer.kind == CS_GKR_LOGUP_GENERIC) reqs.push_back({&o.layer.num, 2});
        reqs.push_back({&o.layer.den, 2});
      }
      std::vector<std::vector<qm31>> mv;
      HP_TRY(read(reqs, mv));
      std::vector<qm31> flat;
      size_t r = 0;
      std::vector<std::vector<std::pair<qm31, qm31>>> layer_masks;
      for (const Oracle& o : oracles) {
        std::vector<std::pair<qm31, qm31>> cols;
        if (o.layer.kind == CS_GKR_LOGUP_SINGLES) cols.push_back({kOne, kOne});
        if (o.layer.kind == CS_GKR_LOGUP_GENERIC) cols.push_back({mv[r][0], mv[r][1]}), r++;
        cols.push_back({mv[r][0], mv[r][1]}), r++;
        std::vector<qm31> m;
        for (const auto& c : cols) m.insert(m.end(), {c.first, c.second});
        ch.mix_felts(m);
        layer_masks.push_back(cols);
      }
      for (Oracle& o : oracles) drop(o.layer.num), drop(o.layer.den);
      ar.release(eq.owned);
      const qm31 x = ch.draw_secure_felt();
      ood = sc_ood;
      ood.push_back(x);
      for (size_t j = 0; j < sc_inst.size(); j++) {
        masks[sc_inst[j]].push_back(layer_masks[j]);
        claims[sc_inst[j]].clear();
        for (const auto& c : layer_masks[j])  // fold_mle_evals
          claims[sc_inst[j]].push_back(qm31_add(qm31_mul(x, qm31_sub(c.second, c.first)), c.first));
      }
    }
    // proof
    out.u(proofs.size());
    for (const auto& rp : proofs) {
      out.u(rp.size());
      for (const Poly& p : rp) {
        out.u(p.size());
        for (const qm31& c : p) out.q(c);
      }
    }
    out.u(n_inst);
    for (size_t i = 0; i < n_inst; i++) {
      out.u(masks[i].size());
      for (const auto& m : masks[i]) {
        out.u(m.size());
        for (const auto& c : m) out.q(c.first), out.q(c.second);
      }
    }
    for (size_t i = 0; i < n_inst; i++) {
      out.u(outputs[i].size());
      for (const qm31& c : outputs[i]) out.q(c);
    }
    // artifact
    out.u(ood.size());
    for (const qm31& c : ood) out.q(c);
    for (size_t i = 0; i < n_inst; i++) {
      out.u(claims[i].size());
      for (const qm31& c : claims[i]) out.q(c);
    }
    for (size_t i = 0; i < n_inst; i++) out.u(inputs[i].n_vars);
    return CS_OK;
  }
};

}  // namespace
}  // namespace hp
}  // namespace cs

extern "C" cs_status cs_gkr_prove_batch(uint32_t n_instances, const uint32_t* h_kinds, const uint32_t* h_n_variables,
                                        const uint32_t* const* h_columns, uint32_t h_channel[9], uint64_t* h_words,
                                        size_t capacity, size_t* n_words, cs_stream stream) {
  CS_CHECK_ARG(n_instances >= 1 && h_kinds != nullptr && h_n_variables != nullptr && h_columns != nullptr &&
                   h_channel != nullptr && n_words != nullptr,
               "gkr_prove_batch: null pointer or no instance");
  std::vector<hp::GLayer> inputs(n_instances);
  for (uint32_t i = 0; i < n_instances; i++) {
    hp::GLayer& L = inputs[i];
    L.kind = h_kinds[i];
    L.n_vars = h_n_variables[i];
    CS_CHECK_ARG(L.kind <= CS_GKR_LOGUP_SINGLES, "gkr_prove_batch: unknown layer kind %u", L.kind);
    CS_CHECK_ARG(L.n_vars >= 1 && L.n_vars <= 29, "gkr_prove_batch: %u variables (1..29)", L.n_vars);
    const uint32_t* const* c = h_columns + 8 * (size_t)i;
    for (int k = 0; k < 4; k++) {
      L.den.c[k] = c[4 + k];
      CS_CHECK_ARG(c[4 + k] != nullptr, "gkr_prove_batch: instance %u: null column", i);
    }
    if (L.kind == CS_GKR_LOGUP_GENERIC)
      for (int k = 0; k < 4; k++) {
        L.num.c[k] = c[k];
        CS_CHECK_ARG(c[k] != nullptr, "gkr_prove_batch: instance %u: null numerator", i);
      }
    if (L.kind == CS_GKR_LOGUP_MULTIPLICITIES) {
      L.num.c[0] = c[0];
      L.num.base = true;
      CS_CHECK_ARG(c[0] != nullptr, "gkr_prove_batch: instance %u: null numerator", i);
    }
  }
  const cudaStream_t st = to_stream(stream);
  hp::Channel ch;
  for (int i = 0; i < 8; i++)
    for (int b = 0; b < 4; b++) ch.digest[4 * i + b] = (uint8_t)(h_channel[i] >> (8 * b));
  ch.n_draws = h_channel[8];
  std::vector<uint64_t>& proof = proof_words();
  proof.clear();
  hp::Words words{proof};
  cs_status s;
  {
    hp::Arena arena(st);
    hp::GkrProver prover{ch, arena, st};
    s = prover.prove(inputs, words);
    if (s == CS_OK && arena.status != CS_OK) s = arena.status;
  }
  if (s != CS_OK) return s;
  for (int i = 0; i < 8; i++)
    h_channel[i] = (uint32_t)ch.digest[4 * i] | ((uint32_t)ch.digest[4 * i + 1] << 8) |
                   ((uint32_t)ch.digest[4 * i + 2] << 16) | ((uint32_t)ch.digest[4 * i + 3] << 24);
  h_channel[8] = ch.n_draws;
  return finish(words.w, h_words, capacity, n_words);
}
