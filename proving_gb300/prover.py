"""The reference's generic prover, restated on the host over a backend.

The reference prover is generic over its backend (`prove_ex`,
crates/stwo/src/prover/mod.rs:39-138); this module restates that caller for
the Wide-Fibonacci AIR so that the CUDA backend runs inside a whole proof:
the commitment scheme (crates/stwo/src/prover/pcs/mod.rs:83-398), DEEP
quotients (crates/stwo/src/prover/pcs/quotient_ops.rs:86-160), FRI commit and
decommit (crates/stwo/src/prover/fri.rs:113-438), lifted Merkle decommitment
(crates/stwo/src/prover/vcs_lifted/prover.rs:97-162), the Blake2s channel
(crates/stwo/src/core/channel/blake2s.rs:16-118) and query sampling
(crates/stwo/src/core/queries.rs:11-58). Every mix and draw happens in the
reference's order. The device work goes through an `ops` object: `GpuOps`
below drives libstwo_cuda.so; the tests drive the same code with the CPU
oracle to compare proofs byte for byte.
"""
from __future__ import annotations

import functools
import hashlib
import struct
from dataclasses import dataclass, field

import numpy as np

P = (1 << 31) - 1

# ------------------------------------------------------------ QM31 scalars
# Host arithmetic on single QM31 values (tuples of 4 ints): channel draws,
# line coefficients and random powers.


def m_inv(a: int) -> int:
    return pow(a, P - 2, P)


def cm_mul(x, y):
    return ((x[0] * y[0] - x[1] * y[1]) % P, (x[0] * y[1] + x[1] * y[0]) % P)


def qm(a, b=0, c=0, d=0):
    return (a % P, b % P, c % P, d % P)


def qm_add(x, y):
    return tuple((a + b) % P for a, b in zip(x, y))


def qm_sub(x, y):
    return tuple((a - b) % P for a, b in zip(x, y))


def qm_neg(x):
    return tuple((-a) % P for a in x)


def qm_mul(x, y):
    # (a + b u)(c + d u) = (ac + (2+i) bd) + (ad + bc) u  (crates/stwo/src/core/fields/qm31.rs:75-81)
    a, b = (x[0], x[1]), (x[2], x[3])
    c, d = (y[0], y[1]), (y[2], y[3])
    ac, bd, ad, bc = cm_mul(a, c), cm_mul(b, d), cm_mul(a, d), cm_mul(b, c)
    rbd = cm_mul((2, 1), bd)
    return ((ac[0] + rbd[0]) % P, (ac[1] + rbd[1]) % P, (ad[0] + bc[0]) % P, (ad[1] + bc[1]) % P)


def qm_mul_m31(x, m: int):
    return tuple((a * m) % P for a in x)


def qm_inv(x):
    # (a + b u)^-1 = (a - b u) / (a^2 - (2+i) b^2)  (qm31.rs:113-122)
    a, b = (x[0], x[1]), (x[2], x[3])
    b2 = cm_mul(b, b)
    ib2 = ((-b2[1]) % P, b2[0])
    a2 = cm_mul(a, a)
    den = ((a2[0] - 2 * b2[0] - ib2[0]) % P, (a2[1] - 2 * b2[1] - ib2[1]) % P)
    n = m_inv((den[0] * den[0] + den[1] * den[1]) % P)
    di = ((den[0] * n) % P, (-den[1] * n) % P)
    r0 = cm_mul(a, di)
    r1 = cm_mul(((-b[0]) % P, (-b[1]) % P), di)
    return (r0[0], r0[1], r1[0], r1[1])


def qm_conj(x):
    """Conjugate with respect to CM31: (a + b u) -> (a - b u)."""
    return (x[0], x[1], (-x[2]) % P, (-x[3]) % P)


def q_double_x(x):
    s = qm_mul(x, x)
    return qm_sub(qm_add(s, s), qm(1))


def m_double_x(x: int) -> int:
    return (2 * x * x - 1) % P


def from_partial_evals(ev):
    """QM31::from_partial_evals (crates/stwo/src/core/fields/qm31.rs:48-54)."""
    r = ev[0]
    r = qm_add(r, qm_mul(ev[1], qm(0, 1, 0, 0)))
    r = qm_add(r, qm_mul(ev[2], qm(0, 0, 1, 0)))
    r = qm_add(r, qm_mul(ev[3], qm(0, 0, 0, 1)))
    return r


def qv_times_i(x):
    """x i for QM31 arrays: (c0 + c1 i) + (c2 + c3 i) u -> (-c1 + c0 i) + (-c3 + c2 i) u."""
    return np.stack([(-x[..., 1]) % P, x[..., 0], (-x[..., 3]) % P, x[..., 2]], axis=-1)


def qv_times_u(x):
    """x u for QM31 arrays: (A + B u) u = (2 + i) B + A u."""
    b0, b1 = x[..., 2], x[..., 3]
    return np.stack([(2 * b0 - b1) % P, (b0 + 2 * b1) % P, x[..., 0], x[..., 1]], axis=-1)


def qv_partial_evals(e):
    """from_partial_evals over arrays: e[..., j, :] are the 4 coordinate values; returns
    e0 + e1 i + e2 u + e3 i u."""
    e = np.asarray(e, np.int64)
    return (e[..., 0, :] + qv_times_i(e[..., 1, :]) + qv_times_u(e[..., 2, :])
            + qv_times_u(qv_times_i(e[..., 3, :]))) % P


def secure_powers(felt, n: int):
    """felt^0 .. felt^(n-1) (generate_secure_powers, crates/stwo/src/prover/air/accumulation.rs:183-200),
    built by doubling: the powers below 2^k times felt^(2^k) give the next 2^k."""
    if n <= 0:
        return []
    pw = np.zeros((1, 4), np.int64)
    pw[0, 0] = 1
    step = np.asarray(felt, np.int64)
    while pw.shape[0] < n:
        pw = np.concatenate([pw, qv_mul(pw, step[None])], axis=0)
        step = qv_mul(step, step)
    return [tuple(r) for r in pw[:n].tolist()]


# ------------------------------------------------------------ QM31 arrays
# The same arithmetic on numpy int64 arrays of shape (..., 4) with canonical
# coordinates: products of two words stay below 2^62 and a sum of two below 2^63.


def qv(x):
    return np.asarray(x, dtype=np.int64).reshape(-1, 4) if np.ndim(x) == 1 else np.asarray(x, dtype=np.int64)


def _cm_mul_v(p0, p1, q0, q1):
    return (p0 * q0 - p1 * q1) % P, (p0 * q1 + p1 * q0) % P


def qv_mul(x, y):
    x, y = np.asarray(x, np.int64), np.asarray(y, np.int64)
    ac0, ac1 = _cm_mul_v(x[..., 0], x[..., 1], y[..., 0], y[..., 1])
    bd0, bd1 = _cm_mul_v(x[..., 2], x[..., 3], y[..., 2], y[..., 3])
    ad0, ad1 = _cm_mul_v(x[..., 0], x[..., 1], y[..., 2], y[..., 3])
    bc0, bc1 = _cm_mul_v(x[..., 2], x[..., 3], y[..., 0], y[..., 1])
    r0, r1 = (2 * bd0 - bd1) % P, (bd0 + 2 * bd1) % P
    return np.stack([(ac0 + r0) % P, (ac1 + r1) % P, (ad0 + bc0) % P, (ad1 + bc1) % P], axis=-1)


def qv_sub(x, y):
    return (np.asarray(x, np.int64) - np.asarray(y, np.int64)) % P


def qv_add(x, y):
    return (np.asarray(x, np.int64) + np.asarray(y, np.int64)) % P


def qv_conj(x):
    x = np.asarray(x, np.int64)
    return np.stack([x[..., 0], x[..., 1], (-x[..., 2]) % P, (-x[..., 3]) % P], axis=-1)


def qv_sum(x):
    """Sum over the leading axis, reduced."""
    return np.asarray(x, np.int64).sum(axis=0) % P


# ------------------------------------------------------------ circle points

def cpoint_add(p, q):
    return ((p[0] * q[0] - p[1] * q[1]) % P, (p[0] * q[1] + p[1] * q[0]) % P)


def index_to_point(idx: int):
    r, cur = (1, 0), (2, 1268011823)
    idx &= (1 << 31) - 1
    while idx:
        if idx & 1:
            r = cpoint_add(r, cur)
        cur = cpoint_add(cur, cur)
        idx >>= 1
    return r


def qpoint_add(p, q):
    return (qm_sub(qm_mul(p[0], q[0]), qm_mul(p[1], q[1])), qm_add(qm_mul(p[0], q[1]), qm_mul(p[1], q[0])))


def random_point(t):
    """CirclePoint::get_random_point from a drawn t (crates/stwo/src/core/circle.rs:150-160)."""
    t2 = qm_mul(t, t)
    inv = qm_inv(qm_add(t2, qm(1)))
    return (qm_mul(qm_sub(qm(1), t2), inv), qm_mul(qm_add(t, t), inv))


def canonic_domain_point(log_size: int, j: int):
    """CanonicCoset(log_size).circle_domain().at(j) (crates/stwo/src/core/poly/circle/domain.rs:148-160)."""
    half_init, half_step, hs = 1 << (31 - (log_size + 1)), 1 << (31 - (log_size - 1)), 1 << (log_size - 1)
    mask = (1 << 31) - 1
    if j < hs:
        return index_to_point((half_init + j * half_step) & mask)
    return index_to_point((-(half_init + (j - hs) * half_step)) & mask)


def bit_reverse_index(i: int, log_size: int) -> int:
    if log_size == 0:
        return i
    return int(format(i, f"0{log_size}b")[::-1], 2)


# ------------------------------------------------------------ channel

class Blake2sChannel:
    """Blake2sChannel (crates/stwo/src/core/channel/blake2s.rs:16-118), hashlib's Blake2s-256."""

    POW_PREFIX = 0x12345678

    def __init__(self, digest: bytes = bytes(32)):
        self.digest = digest
        self.n_draws = 0
        self.log = []  # transcript: (op, data) pairs, for diffing two provers

    def _update(self, d: bytes):
        self.digest = d
        self.n_draws = 0

    def mix_u32s(self, words):
        h = hashlib.blake2s(self.digest)
        h.update(b"".join(struct.pack("<I", int(w) & 0xFFFFFFFF) for w in words))
        self._update(h.digest())
        self.log.append(("mix_u32s", len(words)))

    def mix_u64(self, v: int):
        self.mix_u32s([v & 0xFFFFFFFF, v >> 32])

    def mix_felts(self, felts):
        self.mix_u32s([w for f in felts for w in f])

    def mix_root(self, root: bytes):
        """Blake2sMerkleChannel::mix_hash (crates/stwo/src/core/vcs_lifted/blake2_merkle.rs:56-58)."""
        self._update(hashlib.blake2s(self.digest + root).digest())
        self.log.append(("mix_root", root.hex()))

    def draw_u32s(self):
        h = hashlib.blake2s(self.digest + struct.pack("<I", self.n_draws) + b"\x00").digest()
        self.n_draws += 1
        return list(struct.unpack("<8I", h))

    def draw_secure_felt(self):
        f = [w % P for w in self.draw_u32s()]
        return tuple((f[2 * i] + 2 * f[2 * i + 1]) % P for i in range(4))

    def draw_queries(self, log_domain_size: int, n_queries: int):
        mask, out = (1 << log_domain_size) - 1, []
        while len(out) < n_queries:
            for w in self.draw_u32s():
                out.append(w & mask)
                if len(out) == n_queries:
                    break
        return out

    def verify_pow_nonce(self, n_bits: int, nonce: int) -> bool:
        pre = hashlib.blake2s(struct.pack("<I", self.POW_PREFIX) + self.digest + struct.pack("<I", n_bits)).digest()
        h = hashlib.blake2s(pre + struct.pack("<Q", nonce)).digest()
        v = int.from_bytes(h[:16], "little")
        return v == 0 or (v & -v).bit_length() - 1 >= n_bits


# ------------------------------------------------------------ configuration

@dataclass(frozen=True)
class FriParams:
    """FriParams (crates/stwo/src/core/fri.rs:31-100)."""
    pow_bits: int = 10
    log_blowup_factor: int = 1
    log_last_layer_degree_bound: int = 0
    n_queries: int = 70
    fold_step: int = 1

    def last_layer_domain_size(self) -> int:
        return 1 << (self.log_last_layer_degree_bound + self.log_blowup_factor)


@dataclass(frozen=True)
class PcsConfig:
    """PcsConfig (crates/stwo/src/core/pcs/mod.rs:43-76)."""
    fri_params: FriParams
    trace_lifting_log_size: int
    preprocessed_lifting_log_size: int = 0

    def lifting_log_size(self, tree_index: int) -> int:
        return self.preprocessed_lifting_log_size if tree_index == 0 else self.trace_lifting_log_size


OODS_POW_BITS = 16  # crates/stwo/src/core/proof_of_work.rs:8


# ------------------------------------------------------------ complex-conjugate lines

def line_coeffs(py, value, alpha):
    """complex_conjugate_line_coeffs (crates/stwo/src/core/constraints.rs:119-135), scaled by alpha."""
    a = qm_sub(qm_conj(value), value)
    c = qm_sub(qm_conj(py), py)
    b = qm_sub(qm_mul(value, c), qm_mul(a, py))
    return (qm_mul(alpha, a), qm_mul(alpha, b), qm_mul(alpha, c))


def line_coeffs_v(py, values, alphas):
    """line_coeffs for n sampled values: (n, 3, 4) words (a, b, c per column). py: the sample
    point's y, one for all values or one per value."""
    v, al = np.asarray(values, np.int64), np.asarray(alphas, np.int64)
    pyv = np.broadcast_to(np.asarray(py, np.int64), v.shape)
    a = qv_sub(qv_conj(v), v)
    c = qv_sub(qv_conj(pyv), pyv)
    b = qv_sub(qv_mul(v, c), qv_mul(a, pyv))
    return np.stack([qv_mul(al, a), qv_mul(al, b), qv_mul(al, c)], axis=1)


# ------------------------------------------------------------ decommitment reads

class Reads:
    """Every device read a decommitment makes, collected first and performed in
    one batched call (ops.gather_many): column values at positions and Merkle
    digests at (layer, node). Handles index the results of `run`."""

    def __init__(self):
        self.items = []
        self.out = None

    def values(self, col, idx) -> int:
        self.items.append(("col", col, np.asarray(idx, dtype=np.int64)))
        return len(self.items) - 1

    def block(self, cols, idx) -> int:
        """The same positions of several columns: the result is (len(cols), len(idx))."""
        self.items.append(("cols", list(cols), np.asarray(idx, dtype=np.int64)))
        return len(self.items) - 1

    def digests(self, tree, layer_log: int, nodes) -> int:
        self.items.append(("dig", tree, layer_log, np.asarray(nodes, dtype=np.int64)))
        return len(self.items) - 1

    def tree_digests(self, tree, layers) -> int:
        """Digests of several layers of one tree, [(layer_log, nodes)], as one (n, 8) result in
        that order."""
        self.items.append(("digs", tree, [(k, np.asarray(nodes, dtype=np.int64)) for k, nodes in layers]))
        return len(self.items) - 1

    def run(self, ops):
        self.out = ops.gather_many(self.items)

    def __getitem__(self, h: int):
        return self.out[h]


def merkle_witness_nodes(height: int, query_positions):
    """The witness of MerkleProverLifted::decommit (crates/stwo/src/prover/vcs_lifted/prover.rs:119-150)
    per layer, walking down from the leaves: [(layer log size, sibling nodes)], the sibling of
    every queried node whose sibling is not queried, in node order. All layers at once: row k holds
    the sorted queries shifted down k layers; a node's sibling is present iff it sits next to the
    node's run of equal values."""
    q = np.unique(np.asarray(query_positions, dtype=np.int64))
    if height == 0 or q.size == 0:
        return []
    r = q[None, :] >> np.arange(height, dtype=np.int64)[:, None]
    n = r.shape[1]
    first = np.ones(r.shape, bool)
    first[:, 1:] = r[:, 1:] != r[:, :-1]
    last = np.ones(r.shape, bool)
    last[:, :-1] = r[:, :-1] != r[:, 1:]
    next_is_sib = np.zeros(r.shape, bool)
    next_is_sib[:, :-1] = r[:, 1:] == r[:, :-1] + 1
    prev_is_sib = np.zeros(r.shape, bool)
    prev_is_sib[:, 1:] = r[:, :-1] == r[:, 1:] - 1
    even = (r & 1) == 0
    need = (last & even & ~next_is_sib) | (first & ~even & ~prev_is_sib)
    out = []
    rows, cols = np.nonzero(need)
    if rows.size == 0:
        return out
    sib = r[rows, cols] ^ 1
    bounds = np.searchsorted(rows, np.arange(height + 1))
    for k in range(height):
        if bounds[k + 1] > bounds[k]:
            out.append((height - k, sib[bounds[k]:bounds[k + 1]]))
    return out


class MerkleDecommit:
    """MerkleProverLifted::decommit (crates/stwo/src/prover/vcs_lifted/prover.rs:97-162) in two
    steps: the constructor registers the queried values (col[(pos >> (shift + 1) << 1) + (pos & 1)]
    for a column of log size L - shift) and the witness digests with a Reads; `result` assembles
    them once the Reads has run."""

    def __init__(self, reads: Reads, tree, query_positions, columns, ops):
        L = tree.height
        q = np.asarray(query_positions, dtype=np.int64)
        # columns of one log size read the same positions: one read per run of equal sizes
        self.value_handles = []
        i = 0
        while i < len(columns):
            ls = ops.log_size(columns[i])
            j = i + 1
            while j < len(columns) and ops.log_size(columns[j]) == ls:
                j += 1
            shift = L - ls
            self.value_handles.append(reads.block(columns[i:j], ((q >> (shift + 1)) << 1) + (q & 1)))
            i = j
        self.witness_handle = reads.tree_digests(tree, merkle_witness_nodes(L, q))
        self.reads = reads

    def result(self):
        queried = [row for h in self.value_handles for row in self.reads[h].tolist()]
        b = np.ascontiguousarray(self.reads[self.witness_handle], dtype="<u4").tobytes()
        return queried, [b[i:i + 32] for i in range(0, len(b), 32)]


# ------------------------------------------------------------ FRI

def decommitment_positions(query_positions, fold_step: int):
    """compute_decommitment_positions_and_witness_evals (crates/stwo/src/prover/fri.rs:408-438)
    without the values: the positions to open (every coset of 2^fold_step around a query) and,
    per position, whether its value goes to the witness (it is not itself a query)."""
    q = np.asarray(query_positions, dtype=np.int64)
    starts = np.unique(q >> fold_step) << fold_step
    positions = (starts[:, None] + np.arange(1 << fold_step)).reshape(-1)
    return positions, ~np.isin(positions, q)


class FriLayerDecommit:
    """One FRI layer's decommitment (FriLayerProver::decommit, crates/stwo/src/prover/fri.rs:380-406):
    the witness values of the opened cosets and the Merkle witness of their positions."""

    def __init__(self, reads: Reads, column, tree, query_positions, fold_step: int, ops):
        self.positions, self.is_witness = decommitment_positions(query_positions, fold_step)
        self.coord_handles = [reads.values(c, self.positions) for c in ops.secure_coords(column)]
        # a packed tree opens the leaves holding the positions (fri.rs:318-326)
        packed = packs_leaves(fold_step, ops.secure_len(column).bit_length() - 1)
        merkle_positions = np.unique(self.positions >> LOG_PACKED_LEAF_SIZE) if packed else self.positions
        self.merkle = MerkleDecommit(reads, tree, merkle_positions, [], ops)
        self.reads = reads
        self.tree = tree

    def result(self):
        coords = np.stack([self.reads[h] for h in self.coord_handles], axis=1)[self.is_witness]
        witness = [tuple(r) for r in coords.tolist()]
        _, dec = self.merkle.result()
        return {"fri_witness": witness, "decommitment": dec, "commitment": self.tree.root}


def fold_queries(positions, n_folds: int):
    """Queries::fold (crates/stwo/src/core/queries.rs:50-56)."""
    out = []
    for q in positions:
        f = q >> n_folds
        if not out or out[-1] != f:
            out.append(f)
    return out


# ------------------------------------------------------------ the proof

@dataclass
class StarkProof:
    """CommitmentSchemeProof (crates/stwo/src/core/pcs/quotients.rs:26-36) + FriProof (crates/stwo/src/core/fri.rs)."""
    config: PcsConfig
    commitments: list = field(default_factory=list)          # roots (bytes)
    oods_proof_of_work: int = 0
    sampled_values: list = field(default_factory=list)       # per tree, per column, list of QM31
    decommitments: list = field(default_factory=list)        # per tree, list of hash witness (bytes)
    queried_values: list = field(default_factory=list)       # per tree, per column, list of M31
    fri_first_layer: dict = field(default_factory=dict)
    fri_inner_layers: list = field(default_factory=list)
    fri_last_layer_poly: list = field(default_factory=list)
    fri_proof_of_work: int = 0

    def to_words(self) -> list:
        """A felt stream in the field order of CairoSerialize for StarkProof
        (crates/cairo-serialize/src/serialize.rs:99-210): vectors are a length
        followed by items, QM31 = 4 words, Blake2s hash = 8 LE words, u64 = one felt;
        the pcs config is its 5 FRI parameters only (the lifting log sizes are not
        serialized, serialize.rs:111-119); the last-layer LinePoly is its coefficients
        followed by log2 of their number (serialize.rs:61-66)."""
        w = []

        def vec(items, f):
            w.append(len(items))
            for it in items:
                f(it)

        def h(b):
            w.extend(struct.unpack("<8I", b))

        def q(x):
            w.extend(x)

        fp = self.config.fri_params
        w.extend([fp.pow_bits, fp.log_blowup_factor, fp.log_last_layer_degree_bound, fp.n_queries, fp.fold_step])
        vec(self.commitments, h)
        w.append(self.oods_proof_of_work)
        vec(self.sampled_values, lambda tree: vec(tree, lambda col: vec(col, q)))
        vec(self.decommitments, lambda wit: vec(wit, h))
        vec(self.queried_values, lambda tree: vec(tree, lambda col: vec(col, w.append)))

        def layer(lp):
            vec(lp["fri_witness"], q)
            vec(lp["decommitment"], h)
            h(lp["commitment"])

        layer(self.fri_first_layer)
        vec(self.fri_inner_layers, layer)
        vec(self.fri_last_layer_poly, q)
        w.append(len(self.fri_last_layer_poly).bit_length() - 1)
        w.append(self.fri_proof_of_work)
        return w

    def to_bytes(self) -> bytes:
        return b"".join(struct.pack("<Q", int(x)) for x in self.to_words())


def prove_wide_fib(ops, trace, log_n_rows: int, config: PcsConfig, channel: Blake2sChannel, twiddles):
    """Commits the (empty) preprocessed tree and the Wide-Fibonacci trace, then
    runs prove_ex (crates/stwo/src/prover/mod.rs:39-138). `trace`: the
    column evaluations on CanonicCoset(log_n_rows), as ops columns (consumed)."""
    return prove_wide_fib_components(ops, [trace], [log_n_rows], config, channel, twiddles)


def prove_wide_fib_components(ops, traces, log_sizes, config: PcsConfig, channel: Blake2sChannel, twiddles):
    """Several WideFibonacciComponents of different sizes in one proof, their traces committed in one
    lifted tree (as test_e2e_lifted_fib_prove, crates/examples/src/wide_fibonacci/mod.rs:495-577):
    the empty preprocessed tree, the trace tree, then prove_ex (crates/stwo/src/prover/mod.rs:39-138).
    traces[i]: component i's column evaluations on CanonicCoset(log_sizes[i]) (consumed)."""
    fp = config.fri_params
    b = fp.log_blowup_factor
    L = config.trace_lifting_log_size

    # --- preprocessed tree: empty, a single hash of no data at height 0 (pcs/mod.rs:83-96)
    pre_root = hashlib.blake2s(b"").digest()
    channel.mix_root(pre_root)

    # --- trace tree (TreeBuilder::extend_evals + commit, pcs/mod.rs:325-349, 360-386): every
    # component's columns, in component order, lifted to the tree height
    comp_evals_by = []
    for trace, log_n in zip(traces, log_sizes):
        ops.interpolate(trace, twiddles)
        comp_evals_by.append(ops.evaluate(trace, log_n + b, twiddles))
    trace_evals = [c for ev in comp_evals_by for c in ev]
    n_cols = len(trace_evals)
    trace_tree = ops.merkle_commit(trace_evals, L)
    channel.mix_root(trace_tree.root)

    # --- prove_ex: composition polynomial (air/component_prover.rs:95-116)
    random_coeff = channel.draw_secure_felt()
    # EvaluationMode::infer: constraint log degree 1 <= blowup for every component -> SubDomain{b - 1}
    if b != 1:
        raise NotImplementedError("the Wide-Fibonacci prover supports log_blowup_factor = 1")
    n_cons = [len(t) - 2 for t in traces]
    total = sum(n_cons)
    powers = ops.secure_powers(random_coeff, total)
    # DomainEvaluationAccumulator::columns (air/accumulation.rs:102-122): each component in turn takes
    # the last n of the remaining powers, reversed (component_prover.rs:194), so constraint k of the
    # component whose constraints start at global index g gets alpha^(total - 1 - g - k)
    sub_acc = {}
    start = 0
    for evals, log_n, n in zip(comp_evals_by, log_sizes, n_cons):
        rc = list(reversed(powers[total - start - n:total - start]))
        eval_log = log_n + 1
        if eval_log not in sub_acc:
            sub_acc[eval_log] = ops.secure_zeros(1 << eval_log)
        ops.wide_fib_composition(evals, log_n, rc, sub_acc[eval_log])
        start += n
    # finalize (accumulation.rs:142-180): lift and accumulate ascending sizes, interpolate on the
    # largest canonic domain
    accs = [sub_acc[k] for k in sorted(sub_acc)]
    accum = accs[0] if len(accs) == 1 else ops.lift_and_accumulate(accs)
    comp_log = max(sub_acc)
    comp_coeffs = ops.interpolate_secure(accum, twiddles)
    left, right = ops.split_at_mid(comp_coeffs)
    comp_polys = left + right  # extend_polys(left coords), extend_polys(right coords)
    comp_evals = ops.evaluate(comp_polys, (comp_log - 1) + b, twiddles)
    comp_tree = ops.merkle_commit(comp_evals, L)
    channel.mix_root(comp_tree.root)

    # --- OODS proof of work and point (mod.rs:75-83)
    oods_pow = ops.grind(channel.digest, OODS_POW_BITS)
    channel.mix_u64(oods_pow)
    oods = random_point(channel.draw_secure_felt())

    # --- prove_values (pcs/mod.rs:224-315)
    lifting = L
    columns = [[], trace_evals, comp_evals]
    sample_points = [[], [[oods]] * n_cols, [[oods]] * 8]
    sampled = sample_values(ops, columns, sample_points, lifting)
    channel.mix_felts([v for tree in sampled for col in tree for v in col])

    quotient_coeff = channel.draw_secure_felt()
    quotients = compute_fri_quotients(ops, columns, sample_points, sampled, quotient_coeff, lifting, b, twiddles)

    # --- FRI commit (fri.rs:113-226)
    fri = fri_commit(ops, channel, fp, quotients, lifting, twiddles)

    # --- FRI decommit (fri.rs:229-283) and tree decommitments (pcs/mod.rs:259-287): every value and
    # digest the proof opens is read from the device in one batched call
    fri_pow = ops.grind(channel.digest, fp.pow_bits)
    channel.mix_u64(fri_pow)
    unsorted = channel.draw_queries(lifting, fp.n_queries)
    queries = sorted(set(unsorted))
    reads = Reads()
    first = FriLayerDecommit(reads, quotients, fri["first"]["tree"], queries, fp.fold_step, ops)
    inner = []
    layer_queries = fold_queries(queries, fp.fold_step)
    for layer in fri["inner"]:
        inner.append(FriLayerDecommit(reads, layer["eval"], layer["tree"], layer_queries, layer["fold_step"], ops))
        layer_queries = fold_queries(layer_queries, layer["fold_step"])
    trees = [MerkleDecommit(reads, tree, queries, cols, ops)
             for tree, cols in ((trace_tree, trace_evals), (comp_tree, comp_evals))]
    reads.run(ops)

    proof = StarkProof(config=config)
    proof.fri_first_layer = first.result()
    proof.fri_inner_layers = [d.result() for d in inner]
    proof.fri_last_layer_poly = fri["last_poly"]
    proof.fri_proof_of_work = fri_pow
    # the empty preprocessed tree has height 0: no values, no witness
    proof.commitments = [pre_root, trace_tree.root, comp_tree.root]
    proof.oods_proof_of_work = oods_pow
    proof.sampled_values = sampled
    proof.decommitments = [[]]
    proof.queried_values = [[]]
    for d in trees:
        qv, wit = d.result()
        proof.queried_values.append(qv)
        proof.decommitments.append(wit)

    # --- sanity check: composition value at the OODS point (mod.rs:121-132)
    max_log_degree_bound = lifting - b
    comp = sampled[2]
    left_v = from_partial_evals([comp[k][0] for k in range(4)])
    right_v = from_partial_evals([comp[k][0] for k in range(4, 8)])
    x = oods[0]
    for _ in range(max_log_degree_bound - 1):
        x = q_double_x(x)
    composition_oods = qm_add(left_v, qm_mul(x, right_v))
    mask = [c[0] for c in sampled[1]]
    expected = wide_fib_components_at_point(oods, mask, [len(t) for t in traces], random_coeff, max_log_degree_bound)
    if composition_oods != expected:
        raise RuntimeError("constraints not satisfied (ProvingError::ConstraintsNotSatisfied)")
    return proof


def _size_groups(logs):
    """Indices grouped by log size, in first-seen order."""
    groups = {}
    for i, log_n in enumerate(logs):
        groups.setdefault(log_n, []).append(i)
    return groups


def _evaluate_grouped(ops, coeffs, logs, log_blowup: int, twiddles):
    """Coefficient columns of several sizes evaluated on their blown-up domains, one batched call per
    size; returned in the input order."""
    out = [None] * len(coeffs)
    for log_n, idx in _size_groups(logs).items():
        for i, e in zip(idx, ops.evaluate([coeffs[i] for i in idx], log_n + log_blowup, twiddles)):
            out[i] = e
    return out


def prove_fib_and_lookups(ops, fib_traces, fib_logs, lookup_values, lookup_logs, config: PcsConfig,
                          channel: Blake2sChannel, twiddles, generic: bool = False):
    """Wide-Fibonacci components and single-column LogUp components in one proof (the batched mixed-size
    trace: components of different sizes in one lifted tree, plus LogUp interaction columns). Follows
    the example provers' flow (crates/examples/src/poseidon/mod.rs:336-379): the empty preprocessed
    tree; the trace tree (every Wide-Fibonacci column, then each LogUp component's value column);
    the lookup elements (z, alpha; crates/constraint-framework/src/logup.rs:70-79); the interaction
    tree (each LogUp component's running-sum column, LogupTraceGenerator), after the claimed sums are
    mixed into the channel; then prove_ex. A LogUp
    component's relation entry has multiplicity -1 and values [v], so its fractions are 1 / (z - v)
    and its one constraint is (cur - prev + claimed / 2^n) (v - z) + 1 (finalize_logup). Returns the
    proof with `claimed_sums` (one per LogUp component, part of the statement, not serialized).
    generic=True evaluates the constraints through the generic path (proving_gb300.framework: the
    AIRs written against the constraint evaluator, compiled at run time) instead of the
    hand-written kernels; the proof is the same."""
    fp = config.fri_params
    b = fp.log_blowup_factor
    L = config.trace_lifting_log_size
    if b != 1:
        raise NotImplementedError("log_blowup_factor = 1 (SubDomain evaluation with log_expansion 0)")

    pre_root = hashlib.blake2s(b"").digest()
    channel.mix_root(pre_root)

    # --- trace tree: every stage batched per column size across all components
    fib_cols = [c for t in fib_traces for c in t]
    fib_col_logs = [log_n for t, log_n in zip(fib_traces, fib_logs) for _ in t]
    ops.interpolate(fib_cols, twiddles)
    lookup_coeffs = [None] * len(lookup_values)
    for log_n, idx in _size_groups(lookup_logs).items():
        # out of place: the values stay for the interaction trace
        for i, c in zip(idx, ops.interpolate_into([lookup_values[i] for i in idx], twiddles)):
            lookup_coeffs[i] = c
    trace_cols = _evaluate_grouped(ops, fib_cols + lookup_coeffs, fib_col_logs + list(lookup_logs), b, twiddles)
    fib_evals, start = [], 0
    for t in fib_traces:
        fib_evals.append(trace_cols[start:start + len(t)])
        start += len(t)
    lookup_ext = trace_cols[start:]
    trace_tree = ops.merkle_commit(trace_cols, L)
    channel.mix_root(trace_tree.root)

    # --- lookup elements and the interaction tree
    z = channel.draw_secure_felt()
    channel.draw_secure_felt()  # alpha: drawn with z; a one-value relation does not use it
    sums, claimed = ops.logup_running_sums(lookup_values, z)
    inter_coeffs = [c for col in sums for c in ops.secure_coords(col)]
    inter_logs = [log_n for log_n in lookup_logs for _ in range(4)]
    ops.interpolate(inter_coeffs, twiddles)
    inter_cols = _evaluate_grouped(ops, inter_coeffs, inter_logs, b, twiddles)
    inter_ext = [inter_cols[4 * k:4 * k + 4] for k in range(len(lookup_values))]
    inter_tree = ops.merkle_commit(inter_cols, L)
    # the claimed sums are part of the statement: mixed before the interaction commitment, as the
    # state-machine example does with its second statement (crates/examples/src/state_machine/mod.rs:82-86)
    channel.mix_felts(claimed)
    channel.mix_root(inter_tree.root)

    # --- composition polynomial: components in order take the last powers, reversed
    random_coeff = channel.draw_secure_felt()
    n_cons = [len(t) - 2 for t in fib_traces] + [1] * len(lookup_values)
    total = sum(n_cons)
    powers = ops.secure_powers(random_coeff, total)
    sub_acc, start = {}, 0

    def acc_for(eval_log):
        if eval_log not in sub_acc:
            sub_acc[eval_log] = ops.secure_zeros(1 << eval_log)
        return sub_acc[eval_log]

    if generic:
        from . import framework as fw
        lookup_air = fw.compile_air("single_lookup", fw.single_lookup_air)
    for evals, log_n, n in zip(fib_evals, fib_logs, n_cons):
        rc = list(reversed(powers[total - start - n:total - start]))
        if generic:
            air = fw.compile_air(f"wide_fib_{n + 2}", fw.wide_fib_air, n + 2)
            ops.air_composition(air, {1: evals}, log_n, {}, rc, acc_for(log_n + 1))
        else:
            ops.wide_fib_composition(evals, log_n, rc, acc_for(log_n + 1))
        start += n
    lookup_rc = []
    for k in range(len(lookup_logs)):
        lookup_rc.append(powers[total - start - 1])
        start += 1
    for log_n, idx in _size_groups(lookup_logs).items():
        if generic:
            for k in idx:
                shift = tuple(int(c) * m_inv(1 << log_n) % P for c in claimed[k])
                ops.air_composition(lookup_air, {1: [lookup_ext[k]], 2: inter_ext[k]}, log_n,
                                    {"z": z, "shift": shift}, [lookup_rc[k]], acc_for(log_n + 1))
            continue
        # every LogUp component of one size in one pass over the evaluation domain
        ops.logup_compositions([lookup_ext[k] for k in idx], [inter_ext[k] for k in idx], log_n, z,
                               [claimed[k] for k in idx], [lookup_rc[k] for k in idx], acc_for(log_n + 1))
    accs = [sub_acc[k] for k in sorted(sub_acc)]
    accum = accs[0] if len(accs) == 1 else ops.lift_and_accumulate(accs)
    comp_log = max(sub_acc)
    comp_coeffs = ops.interpolate_secure(accum, twiddles)
    left, right = ops.split_at_mid(comp_coeffs)
    comp_evals = ops.evaluate(left + right, (comp_log - 1) + b, twiddles)
    comp_tree = ops.merkle_commit(comp_evals, L)
    channel.mix_root(comp_tree.root)

    # --- OODS
    oods_pow = ops.grind(channel.digest, OODS_POW_BITS)
    channel.mix_u64(oods_pow)
    oods = random_point(channel.draw_secure_felt())
    lifting = L
    mldb = lifting - b
    g = m31_subgroup_generator(mldb)
    prev_pt = qpoint_add_m31(oods, (g[0], (-g[1]) % P))
    columns = [[], trace_cols, inter_cols, comp_evals]
    sample_points = [[], [[oods]] * len(trace_cols), [[prev_pt, oods]] * len(inter_cols), [[oods]] * 8]
    sampled = sample_values(ops, columns, sample_points, lifting)
    channel.mix_felts([v for tree in sampled for col in tree for v in col])
    quotient_coeff = channel.draw_secure_felt()
    quotients = compute_fri_quotients(ops, columns, sample_points, sampled, quotient_coeff, lifting, b, twiddles)
    fri = fri_commit(ops, channel, fp, quotients, lifting, twiddles)

    fri_pow = ops.grind(channel.digest, fp.pow_bits)
    channel.mix_u64(fri_pow)
    queries = sorted(set(channel.draw_queries(lifting, fp.n_queries)))
    reads = Reads()
    first = FriLayerDecommit(reads, quotients, fri["first"]["tree"], queries, fp.fold_step, ops)
    inner = []
    layer_queries = fold_queries(queries, fp.fold_step)
    for layer in fri["inner"]:
        inner.append(FriLayerDecommit(reads, layer["eval"], layer["tree"], layer_queries, layer["fold_step"], ops))
        layer_queries = fold_queries(layer_queries, layer["fold_step"])
    trees = [MerkleDecommit(reads, tree, queries, cols, ops)
             for tree, cols in ((trace_tree, trace_cols), (inter_tree, inter_cols), (comp_tree, comp_evals))]
    reads.run(ops)
    proof = StarkProof(config=config)
    proof.fri_first_layer = first.result()
    proof.fri_inner_layers = [d.result() for d in inner]
    proof.fri_last_layer_poly = fri["last_poly"]
    proof.fri_proof_of_work = fri_pow
    proof.commitments = [pre_root, trace_tree.root, inter_tree.root, comp_tree.root]
    proof.oods_proof_of_work = oods_pow
    proof.sampled_values = sampled
    proof.decommitments = [[]]
    proof.queried_values = [[]]
    for d in trees:
        qv, wit = d.result()
        proof.queried_values.append(qv)
        proof.decommitments.append(wit)
    proof.claimed_sums = claimed

    # --- sanity check (mod.rs:121-132)
    comp = sampled[3]
    left_v = from_partial_evals([comp[k][0] for k in range(4)])
    right_v = from_partial_evals([comp[k][0] for k in range(4, 8)])
    x = oods[0]
    for _ in range(mldb - 1):
        x = q_double_x(x)
    composition_oods = qm_add(left_v, qm_mul(x, right_v))
    expected = fib_and_lookups_at_point(oods, sampled, [len(t) for t in fib_traces], lookup_logs, z, claimed,
                                        random_coeff, mldb, powers)
    if composition_oods != expected:
        raise RuntimeError("constraints not satisfied (ProvingError::ConstraintsNotSatisfied)")
    return proof


def fib_and_lookups_at_point(point, sampled, n_cols_per_fib, lookup_logs, z, claimed, random_coeff,
                             max_log_degree_bound: int, powers=None):
    """The composition polynomial at the point from the sampled values (Components::
    eval_composition_polynomial_at_point): the Wide-Fibonacci constraints, then each LogUp
    component's (cur - prev + claimed / 2^n) (v - z) + 1, Horner-combined, over V(mldb) at the point."""
    x = point[0]
    for _ in range(max_log_degree_bound - 1):
        x = q_double_x(x)
    den_inv = qm_inv(x)
    m = np.asarray([c[0] for c in sampled[1]], np.int64)
    # every Wide-Fibonacci constraint c - (a^2 + b^2) at once, component after component
    starts = np.cumsum([0] + list(n_cols_per_fib))[:-1]
    i0 = np.concatenate([st + np.arange(n - 2) for st, n in zip(starts, n_cols_per_fib)]).astype(np.int64)
    sq = qv_mul(m, m)
    cons = [qv_sub(m[i0 + 2], qv_add(sq[i0], sq[i0 + 1]))]
    start = int(sum(n_cols_per_fib))
    n_look = len(lookup_logs)
    if n_look:
        # every LogUp component at once: samples (component, coordinate, prev / cur, QM31)
        smp = np.asarray(sampled[2], np.int64).reshape(n_look, 4, 2, 4)
        prev, cur = qv_partial_evals(smp[:, :, 0]), qv_partial_evals(smp[:, :, 1])
        inv_n = np.asarray([m_inv(1 << log_n) for log_n in lookup_logs], np.int64)
        shift = np.asarray(claimed, np.int64) * inv_n[:, None] % P
        shifted = qv_add(qv_sub(cur, prev), shift)
        v = m[start:start + n_look]
        one = np.asarray([1, 0, 0, 0], np.int64)
        cons.append(qv_add(qv_mul(shifted, qv_sub(v, np.asarray(z, np.int64))), one))
    cons = np.concatenate(cons, axis=0)
    if powers is None:
        powers = secure_powers(random_coeff, len(cons))
    total = qv_sum(qv_mul(cons, np.asarray(list(reversed(powers[:len(cons)])), np.int64)))
    return qm_mul(tuple(int(t) for t in total), den_inv)


def q_double_point(pt):
    """CirclePoint::double over QM31."""
    return (q_double_x(pt[0]), qm_mul(qm(2), qm_mul(pt[0], pt[1])))


def sample_values(ops, columns, sample_points, lifting: int):
    """CommitmentSchemeProver::compute_samples (crates/stwo/src/prover/pcs/mod.rs:175-214): every
    column at every one of its sample points, each point doubled lifting - log_size times (the
    column is committed lifted). One barycentric weight column per (log size, point) across all
    trees; every evaluation is launched before the values are read back once.
    Returns per tree, per column, the list of QM31 values."""
    groups = {}
    for ti, (tree_cols, pts) in enumerate(zip(columns, sample_points)):
        for ci, col in enumerate(tree_cols):
            ls = ops.log_size(col)
            for si, pt in enumerate(pts[ci]):
                groups.setdefault((ls, pt), []).append((ti, ci, si))
    doublings = {}  # point -> [point, 2 point, 4 point, ...]
    pending = []
    for (log_size, pt), members in groups.items():
        chain = doublings.setdefault(pt, [pt])
        while len(chain) <= lifting - log_size:
            chain.append(q_double_point(chain[-1]))
        w = ops.barycentric_weights(log_size, chain[lifting - log_size])
        pending.append((members, ops.barycentric_eval_lazy([columns[ti][ci] for ti, ci, _ in members], w)))
    results = ops.fetch_evals([h for _, h in pending])
    sampled = [[[None] * len(p_) for p_ in pts] for pts in sample_points]
    for (members, _), res in zip(pending, results):
        for (ti, ci, si), v in zip(members, res):
            sampled[ti][ci][si] = v
    return sampled


@functools.lru_cache(maxsize=64)
def m31_subgroup_generator(log_size: int):
    """The generator G_log_size of the circle subgroup of order 2^log_size, as an M31 point."""
    return index_to_point(1 << (31 - log_size))


def qpoint_add_m31(p, g):
    """p + g for a QM31 point p and an M31 point g."""
    return qpoint_add(p, (qm(g[0]), qm(g[1])))


def wide_fib_components_at_point(point, mask, n_cols_per_component, random_coeff, max_log_degree_bound: int):
    """Components::eval_composition_polynomial_at_point (crates/stwo/src/core/air/components.rs:54-75) for
    Wide-Fibonacci components in order: one Horner accumulation over all their constraints, each
    divided by V(CanonicCoset(max_log_degree_bound)) at the point."""
    x = point[0]
    for _ in range(max_log_degree_bound - 1):
        x = q_double_x(x)
    den_inv = qm_inv(x)
    m = np.asarray(mask, np.int64)
    cons, start = [], 0
    for n in n_cols_per_component:
        a, b, c = m[start:start + n - 2], m[start + 1:start + n - 1], m[start + 2:start + n]
        cons.append(qv_sub(c, qv_add(qv_mul(a, a), qv_mul(b, b))))
        start += n
    cons = np.concatenate(cons, axis=0)
    powers = np.asarray(list(reversed(secure_powers(random_coeff, len(cons)))), np.int64)
    total = qv_sum(qv_mul(cons, powers))
    return qm_mul(tuple(int(v) for v in total), den_inv)


def compute_fri_quotients(ops, columns, sample_points, sampled, random_coeff, lifting: int, log_blowup: int,
                          twiddles):
    """compute_fri_quotients (crates/stwo/src/prover/pcs/quotient_ops.rs:86-160): every sample of every
    column with its random power, grouped by column size and sample point, accumulated, lifted and
    combined into the FRI quotient column."""
    n_samples = sum(len(c) + (1 if len(c) == 2 else 0) for tree in sampled for c in tree)
    pows = ops.secure_powers(random_coeff, n_samples)
    entries = []  # (log size, column, point, value) in tree/column order; entry k has power k
    shifted = {}  # (point, log period) -> the point shifted by the period
    for tree_cols, pts, vals in zip(columns, sample_points, sampled):
        for col, cp, cv in zip(tree_cols, pts, vals):
            ls = ops.log_size(col)
            if len(cp) == 2:
                # build_samples_with_randomness_and_periodicity (crates/stwo/src/core/pcs/quotients.rs:274-319):
                # a column sampled at (previous row, point) also opens the point shifted by the
                # period G_(lifting - log size), with the point's value, first
                key = (cp[1], lifting - ls)
                if key not in shifted:
                    shifted[key] = qpoint_add_m31(cp[1], m31_subgroup_generator(lifting - ls))
                entries.append((ls, col, shifted[key], cv[1]))
            for p_, v_ in zip(cp, cv):
                entries.append((ls, col, p_, v_))
    # every sample's line coefficients in one vectorized pass
    all_coeffs = line_coeffs_v(np.asarray([e[2][1] for e in entries], np.int64),
                               [e[3] for e in entries], pows[:len(entries)])
    # stable sort by column log size, group by size, batch by point in insertion order
    by_size = {}
    for k, e in enumerate(entries):
        by_size.setdefault(e[0], []).append(k)
    accs = []  # (point, partial numerator column, first linear term)
    for ls in sorted(by_size):
        batches = {}
        for k in by_size[ls]:
            batches.setdefault(entries[k][2], []).append(k)
        for p_, ks in batches.items():
            part, first_linear = ops.accumulate_numerators([entries[k][1] for k in ks], all_coeffs[ks], log_blowup)
            accs.append((p_, part, tuple(int(x) for x in first_linear)))
    # group per sample point (sorted by (x, y)), lift and accumulate ascending sizes
    per_point = {}
    for p_, part, fl in accs:
        per_point.setdefault(p_, []).append((part, fl))
    points, parts, fls = [], [], []
    for p_ in sorted(per_point, key=lambda pt: (pt[0], pt[1])):
        items = per_point[p_]
        fl = qm(0)
        for _, f in items:
            fl = qm_add(fl, f)
        col = ops.lift_and_accumulate([part for part, _ in sorted(items, key=lambda it: ops.secure_len(it[0]))])
        points.append(p_)
        parts.append(col)
        fls.append(fl)
    return ops.compute_quotients_and_combine(parts, points, fls, lifting, log_blowup, twiddles)


class HostFriChannel:
    """The FRI commit loop's view of the channel when the channel lives on the host."""

    def __init__(self, channel):
        self.channel = channel

    def mix_root(self, tree):
        self.channel.mix_root(tree.root)

    def draw(self):
        return self.channel.draw_secure_felt()

    def finish(self):
        pass


LOG_PACKED_LEAF_SIZE = 2  # crates/stwo/src/core/vcs_lifted/verifier.rs:16


def squared_alpha_powers(alpha, n: int) -> list:
    """squared_alpha_powers (crates/stwo/src/prover/fri.rs:79-87): alpha, alpha^2, alpha^4, ..."""
    out = []
    for _ in range(n):
        out.append(alpha)
        alpha = qm_mul(alpha, alpha)
    return out


def packs_leaves(fold_step: int, log_size: int) -> bool:
    """Whether a FRI layer's tree has leaves of 2^LOG_PACKED_LEAF_SIZE consecutive values
    (FriFirstLayerProver::new / FriInnerLayerProver::new, fri.rs:294-305, 357-367)."""
    return fold_step > 1 and log_size >= LOG_PACKED_LEAF_SIZE


def _commit_layer(ops, column, log_size: int, fold_step: int):
    """A FRI layer's lifted Merkle tree over its 4 coordinate columns, or, with packed leaves,
    over the 16 columns of pack_leaves_input at 2^(log_size - 2) rows."""
    cols = ops.secure_columns(column)
    if packs_leaves(fold_step, log_size):
        return ops.merkle_commit(ops.pack_leaves(cols), log_size - LOG_PACKED_LEAF_SIZE)
    return ops.merkle_commit(cols, log_size)


def fri_layers(ops, ch, fp: FriParams, column, log_size: int, twiddles):
    """The layer loop of FriProver::commit (crates/stwo/src/prover/fri.rs:113-206): commit a
    layer, mix its root, draw the challenge, fold. The first layer's circle fold is followed by
    fold_step - 1 line folds with alpha^2, alpha^4, ...; every inner layer folds fold_step times
    (alpha, alpha^2, ...), the last one the 1..fold_step folds left. Returns (first tree, inner
    layers, the last evaluation); the channel `ch` is finished by the caller."""
    k = fp.fold_step

    def fold(layer, alpha, steps):
        if steps == 1:
            return ops.fold_line(layer, alpha, twiddles)
        return ops.fold_line_steps(layer, squared_alpha_powers(alpha, steps), twiddles)

    first_tree = _commit_layer(ops, column, log_size, k)
    ch.mix_root(first_tree)
    alpha = ch.draw()
    layer = ops.fold_circle_into_line(column, alpha, twiddles)
    line_log = log_size - 1
    if k > 1:
        layer = fold(layer, qm_mul(alpha, alpha), k - 1)
        line_log -= k - 1
    last_log = (fp.last_layer_domain_size()).bit_length() - 1
    if line_log < last_log:
        raise ValueError("the circle-to-line fold results in a smaller line domain than the last layer")
    inner = []
    if line_log == last_log:
        return first_tree, inner, layer
    while line_log > last_log + k:
        tree = _commit_layer(ops, layer, line_log, k)
        ch.mix_root(tree)
        alpha = ch.draw()
        inner.append({"tree": tree, "eval": layer, "fold_step": k})
        layer = fold(layer, alpha, k)
        line_log -= k
    last_step = line_log - last_log
    tree = _commit_layer(ops, layer, line_log, last_step)
    ch.mix_root(tree)
    alpha = ch.draw()
    inner.append({"tree": tree, "eval": layer, "fold_step": last_step})
    layer = fold(layer, alpha, last_step)
    return first_tree, inner, layer


def fri_commit(ops, channel, fp: FriParams, column, log_size: int, twiddles):
    """FriProver::commit (crates/stwo/src/prover/fri.rs:113-226). With fold_step 1 the ops may run
    the layer loop themselves (ops.fri_layers: the channel kept on the device, so that mixing each
    root and drawing each challenge needs no host round trip); a larger fold_step squares each
    challenge on the host."""
    if hasattr(ops, "fri_layers") and fp.fold_step == 1:
        first_tree, inner, layer = ops.fri_layers(channel, fp, column, log_size, twiddles)
    else:
        ch = HostFriChannel(channel)
        first_tree, inner, layer = fri_layers(ops, ch, fp, column, log_size, twiddles)
        ch.finish()
    last_log = (fp.last_layer_domain_size()).bit_length() - 1
    # commit_last_layer (fri.rs:208-226): interpolate the last evaluation on its line domain
    values = ops.gather_secure(layer, list(range(fp.last_layer_domain_size())))
    coeffs = line_interpolate(values, last_log)
    bound = 1 << fp.log_last_layer_degree_bound
    if any(c != qm(0) for c in coeffs[bound:]):
        raise RuntimeError("invalid degree in the last FRI layer")
    # LinePoly::from_ordered_coefficients stores them bit-reversed; that order is mixed
    last_poly = [coeffs[:bound][bit_reverse_index(i, fp.log_last_layer_degree_bound)] for i in range(bound)]
    channel.mix_felts(last_poly)
    return {"first": {"tree": first_tree}, "inner": inner, "last_poly": last_poly}


def line_interpolate(values, log_size: int):
    """LineEvaluation::interpolate + LinePoly::into_ordered_coefficients
    (crates/stwo/src/prover/line.rs:54-99, crates/stwo/src/core/poly/line.rs:151-154)
    for an evaluation on LineDomain(half_odds(log_size)) given in bit-reversed
    order; returns the coefficients in natural order."""
    n = 1 << log_size
    v = [values[bit_reverse_index(i, log_size)] for i in range(n)]
    mask = (1 << 31) - 1
    init, step, dom_log = 1 << (31 - (log_size + 2)), 1 << (31 - log_size), log_size
    while dom_log > 0:
        size = 1 << dom_log
        xs = [index_to_point((init + i * step) & mask)[0] for i in range(size // 2)]
        for start in range(0, n, size):
            for i in range(size // 2):
                a, c = v[start + i], v[start + size // 2 + i]
                v[start + i] = qm_add(a, c)
                v[start + size // 2 + i] = qm_mul_m31(qm_sub(a, c), m_inv(xs[i]))
        init, step, dom_log = (init * 2) & mask, (step * 2) & mask, dom_log - 1
    ninv = m_inv(n % P)
    v = [qm_mul_m31(x, ninv) for x in v]
    return [v[bit_reverse_index(i, log_size)] for i in range(n)]


# ------------------------------------------------------------ GPU ops

class GpuMerkle:
    def __init__(self, prover, height: int):
        self.t = prover
        self.height = height
        self._root = None

    @property
    def root(self) -> bytes:
        if self._root is None:
            self._root = self.t.root()
        return self._root

    def hashes(self, layer_log: int, idx):
        import torch
        lay = self.t.layer(layer_log)
        sel = lay[torch.as_tensor(idx, device=lay.device, dtype=torch.long)]
        arr = sel.cpu().numpy().astype("<i4")
        return [arr[i].tobytes() for i in range(arr.shape[0])]


class GpuOps:
    """Device operations of the prover through libstwo_cuda.so (proving_gb300.backend)."""

    def __init__(self):
        from . import backend as be
        self.be = be
        self.B = be.CudaBackend
        self._fri_graphs = {}

    def secure_powers(self, felt, n):
        """felt^0 .. felt^(n-1) on the host (cs_generate_secure_powers)."""
        return [tuple(r) for r in self.B.generate_secure_powers(np.asarray(felt, np.uint32), n).tolist()]

    def twiddles(self, root_log_domain: int):
        return self.B.precompute_twiddles(self.be.canonic_half_coset(root_log_domain))

    def columns_from_host(self, cols):
        return [self.be.BaseColumn.from_cpu(c) for c in cols]

    def log_size(self, col) -> int:
        return col.log_size

    def interpolate(self, cols, tw):
        self.B.interpolate_columns(cols, tw)

    def interpolate_into(self, cols, tw):
        """Coefficients of the evaluations `cols` in new columns (one device block); cols are kept."""
        return self.B.interpolate_columns_into(cols, tw, out=self._block(len(cols), cols[0].log_size))

    def evaluate(self, coeffs, log_size, tw):
        return self.B.evaluate_polynomials(coeffs, log_size, tw, out=self._block(len(coeffs), log_size))

    def _block(self, n_cols, log_size):
        import torch
        blk = torch.empty((n_cols, 1 << log_size), dtype=torch.int32, device="cuda")
        return self.be.BaseColumn.rows_of(blk)

    def merkle_commit(self, cols, L):
        return GpuMerkle(self.B.merkle_commit(cols, L), L)

    # single-column LogUp components
    def logup_running_sum(self, values, z):
        return self.B.logup_running_sum(values, np.asarray(z, np.uint32))

    def logup_running_sums(self, values, z):
        """Every column's running sum in one batch of launches; the claimed sums read back once."""
        cols, claimed = self.B.logup_running_sums(values, np.asarray(z, np.uint32))
        return cols, [tuple(int(x) for x in row) for row in claimed.cpu().numpy().view(np.uint32)]

    def air_composition(self, air, columns_by_interaction, trace_log, params, rc, accum, log_expansion=0):
        """An AIR's constraint quotients through the generic path (run-time compiled kernel)."""
        from .framework import CompiledAir
        CompiledAir.get(air).composition(columns_by_interaction, trace_log, params, rc, accum, log_expansion)

    def air_fractions(self, air, columns_by_interaction, log_n, params):
        """An AIR's LogUp batch fractions on the trace domain (run-time compiled kernel)."""
        from .framework import CompiledAir
        return CompiledAir.get(air).fractions(columns_by_interaction, log_n, params)

    def logup_generator(self, log_n):
        return self.be.LogupTraceGenerator(log_n)

    def interpolate_secure_on_subdomain(self, accum, domain_log_size, tw):
        """The accumulator interpolated on the subdomain of its size of CanonicCoset(domain_log_size)
        (DomainEvaluationAccumulator::finalize in SubDomain mode), in place."""
        self.B.interpolate_on_subdomain(accum.columns, domain_log_size, tw)
        return accum.columns

    def logup_compositions(self, values_evals, inter_evals, trace_log, z, claimed, rcs, accum):
        self.B.logup_compositions(values_evals, [self.be.SecureColumnByCoords(it) for it in inter_evals], trace_log,
                                  z, claimed, [[int(w) for w in r] for r in rcs], accum)

    def logup_composition(self, values_eval, inter_eval, trace_log, z, claimed, rc, accum):
        self.B.logup_composition(values_eval, self.be.SecureColumnByCoords(inter_eval), trace_log, z, claimed, rc,
                                 accum)

    # Poseidon2 AIR (crates/examples/src/poseidon/mod.rs)
    def poseidon_trace(self, log_n):
        return self.B.poseidon_trace(log_n)

    def poseidon_interaction(self, trace, lookup):
        return self.B.poseidon_interaction(trace, lookup)

    def poseidon_composition(self, trace_evals, inter_evals, trace_log, lookup, claimed, rc, accum):
        self.B.poseidon_composition(trace_evals, inter_evals, trace_log, lookup, claimed, rc, accum)

    def gather(self, col, idx):
        import torch
        t = col.data[torch.as_tensor(idx, device=col.data.device, dtype=torch.long)]
        return t.cpu().numpy().view(np.uint32)

    def secure_zeros(self, n):
        return self.be.SecureColumnByCoords.zeros(n)

    def secure_len(self, col) -> int:
        return len(col)

    def secure_columns(self, col):
        return col.columns

    def secure_coords(self, col):
        return col.columns

    def gather_many(self, items):
        """Column values ("col", col, idx) and Merkle digests ("dig", tree, layer_log, nodes), read in
        one cs_gather_u32 call; digests come back as (n, 8) words."""
        tensors, slot_of, slots, idx, sizes = [], {}, [], [], []
        def slot(t):
            key = (t.data_ptr(), t.numel())
            if key not in slot_of:
                slot_of[key] = len(tensors)
                tensors.append(t)
            return slot_of[key]

        for it in items:
            if it[0] == "cols":
                ix = np.asarray(it[2], dtype=np.int64)
                sl = np.array([slot(c.data) for c in it[1]], np.uint32)
                slots.append(np.repeat(sl, ix.size))
                idx.append(np.tile(ix, len(it[1])).astype(np.uint32))
                sizes.append(sl.size * ix.size)
                continue
            if it[0] == "col":
                t = it[1].data
                ix = np.asarray(it[2], dtype=np.int64)
            elif it[0] == "digs":
                # every layer of the tree in its one buffer: layer k starts at node 2^(L+1) - 2^(k+1)
                t = it[1].t.all
                top = 1 << (it[1].height + 1)
                nodes = (np.concatenate([top - (2 << k) + n for k, n in it[2]]) if it[2]
                         else np.zeros(0, np.int64))
                ix = (nodes[:, None] * 8 + np.arange(8)).reshape(-1)
            else:
                t = it[1].t.layer(it[2])
                nodes = np.asarray(it[3], dtype=np.int64)
                ix = (nodes[:, None] * 8 + np.arange(8)).reshape(-1)
            slots.append(np.full(ix.size, slot(t), np.uint32))
            idx.append(ix.astype(np.uint32))
            sizes.append(ix.size)
        if not items:
            return []
        words = self.B.gather_words(tensors, np.concatenate(slots), np.concatenate(idx))
        out, off = [], 0
        for it, n in zip(items, sizes):
            w = words[off:off + n]
            if it[0] == "cols":
                w = w.reshape(len(it[1]), -1)
            elif it[0] in ("dig", "digs"):
                w = w.reshape(-1, 8)
            out.append(w)
            off += n
        return out

    def gather_secure(self, col, idx):
        vals = [self.gather(c, idx) for c in col.columns]
        return [tuple(int(vals[k][i]) for k in range(4)) for i in range(len(idx))]

    def wide_fib_composition(self, evals, trace_log, rc, accum):
        self.B.wide_fib_composition(evals, trace_log, np.asarray(rc, np.uint32), accum)

    def interpolate_secure(self, accum, tw):
        self.B.interpolate_columns(accum.columns, tw)
        return accum.columns

    def split_at_mid(self, coeff_cols):
        be = self.be
        half = len(coeff_cols[0]) // 2
        left = [be.BaseColumn(c.data[:half]) for c in coeff_cols]
        right = [be.BaseColumn(c.data[half:]) for c in coeff_cols]
        return left, right

    def grind(self, digest, bits):
        return self.B.grind(digest, bits)

    def barycentric_weights(self, log_size, point):
        return self.B.barycentric_weights(log_size, point)

    def barycentric_eval(self, cols, weights):
        return self.fetch_evals([self.barycentric_eval_lazy(cols, weights)])[0]

    def barycentric_eval_lazy(self, cols, weights):
        """The values of cols at the weights' point, left on the device: (n, 4) words."""
        return self.B.barycentric_eval_at_point(cols, weights)

    def fetch_evals(self, handles):
        """Reads back the results of barycentric_eval_lazy calls in one copy."""
        import torch
        if not handles:
            return []
        flat = torch.cat(handles).cpu().numpy().view(np.uint32).tolist()
        out, k = [], 0
        for h in handles:
            out.append([tuple(r) for r in flat[k:k + h.shape[0]]])
            k += h.shape[0]
        return out

    def accumulate_numerators(self, cols, coeffs, log_blowup):
        return self.B.accumulate_numerators(cols, np.asarray(coeffs, np.uint32), log_blowup)

    def lift_and_accumulate(self, cols):
        return self.B.lift_and_accumulate(cols)

    def compute_quotients_and_combine(self, parts, points, fls, lifting, log_blowup, tw):
        pts = [(np.asarray(p_[0], np.uint32), np.asarray(p_[1], np.uint32)) for p_ in points]
        return self.B.compute_quotients_and_combine(parts, pts, [np.asarray(f, np.uint32) for f in fls], lifting,
                                                    log_blowup, tw)

    def fold_circle_into_line(self, col, alpha, tw):
        if isinstance(alpha, DeviceFelt):
            return self.B.fold_circle_into_line_device_alpha(col, alpha.data, tw)
        return self.B.fold_circle_into_line(col, np.asarray(alpha, np.uint32), tw)

    def fold_line(self, col, alpha, tw):
        if isinstance(alpha, DeviceFelt):
            return self.B.fold_line_device_alpha(col, alpha.data, tw)
        return self.B.fold_line(col, [np.asarray(alpha, np.uint32)], tw)

    def fold_line_steps(self, col, alphas, tw):
        """len(alphas) folds in one call (cs_fold_line_steps)."""
        return self.B.fold_line(col, [np.asarray(a, np.uint32) for a in alphas], tw)

    def pack_leaves(self, cols):
        return self.B.pack_leaves_input(cols)

    fri_graphs = True  # replay the FRI layer loop as a CUDA graph per (stream, size, parameters)

    def fri_layers(self, channel, fp, column, log_size, tw):
        """The FRI layer loop with the channel on the device. The loop has no host synchronisation,
        so after its first run for a (stream, log size, FRI parameters, twiddles) it is captured
        once as a CUDA graph over static buffers; later proofs copy their column and channel state
        in, replay it, and read the state and the roots back in one call."""
        if not self.fri_graphs:
            ch = DeviceFriChannel(self, channel)
            out = fri_layers(self, ch, fp, column, log_size, tw)
            ch.finish()
            return out
        import torch
        # the entry keeps `tw` alive, so its id cannot be reused while the graph refers to it
        key = (torch.cuda.current_stream().cuda_stream, log_size, fp, id(tw))
        g = self._fri_graphs.get(key)
        if g is None:
            ch = DeviceFriChannel(self, channel)
            out = fri_layers(self, ch, fp, column, log_size, tw)
            ch.finish()
            if len(self._fri_graphs) >= 8:  # oldest first out
                self._fri_graphs.pop(next(iter(self._fri_graphs)))
            self._fri_graphs[key] = self._capture_fri(channel, fp, column, log_size, tw) + (tw,)
            return out
        graph, static_in, ch, out, _ = g
        for dst, src in zip(static_in.columns, column.columns):
            dst.data.copy_(src.data)
        ch.reset(channel)
        graph.replay()
        ch.finish()
        return out

    def _capture_fri(self, channel, fp, column, log_size, tw):
        """Captures the layer loop. Python's collector is paused while the capture is open: a
        collection there could destroy an evicted graph caught in a reference cycle, and the
        release of its memory pool would end the capture (torch.cuda.graph collects once
        before the capture begins)."""
        import gc
        import torch
        static_in = self.be.SecureColumnByCoords.uninitialized(len(column))
        ch = DeviceFriChannel(self, channel)
        graph = torch.cuda.CUDAGraph()
        was_enabled = gc.isenabled()
        gc.disable()
        try:
            with torch.cuda.graph(graph):
                out = fri_layers(self, ch, fp, static_in, log_size, tw)
        finally:
            if was_enabled:
                gc.enable()
        return graph, static_in, ch, out


class DeviceFelt:
    """A QM31 drawn by the device channel, left in device memory (4 words)."""

    def __init__(self, data):
        self.data = data


class DeviceFriChannel:
    """The FRI commit loop's channel on the device (cs_channel_mix_root / cs_channel_draw_secure_felt):
    the state starts from the host channel's, every layer's root is mixed and its challenge drawn
    on the device, and `finish` reads the state and all the layer roots back in one call and
    brings the host channel to the same state."""

    def __init__(self, ops, channel):
        import torch
        self.ops, self.channel = ops, channel
        words = list(struct.unpack("<8I", channel.digest)) + [channel.n_draws]
        self.state = torch.tensor(np.array(words, np.uint32).view(np.int32), device="cuda")
        self.felts = torch.empty((64, 4), dtype=torch.int32, device="cuda")
        self.n_felts = 0
        self.trees = []

    def reset(self, channel):
        """Starts from the host channel's state again (for a replayed layer loop)."""
        import torch
        self.channel = channel
        words = list(struct.unpack("<8I", channel.digest)) + [channel.n_draws]
        self.state.copy_(torch.from_numpy(np.array(words, np.uint32).view(np.int32)))

    def mix_root(self, tree):
        from .backend import _stream
        from . import _lib
        self.trees.append(tree)
        root = tree.t.all[-1]
        _lib.call("cs_channel_mix_root", self.state.data_ptr(), root.data_ptr(), _stream())

    def draw(self):
        from .backend import _stream
        from . import _lib
        felt = self.felts[self.n_felts]
        self.n_felts += 1
        _lib.call("cs_channel_draw_secure_felt", self.state.data_ptr(), felt.data_ptr(), _stream())
        return DeviceFelt(felt)

    def finish(self):
        tensors = [self.state] + [t.t.all[-1] for t in self.trees]
        slots = np.concatenate([np.zeros(9, np.uint32)] + [np.full(8, i + 1, np.uint32)
                                                           for i in range(len(self.trees))])
        idx = np.concatenate([np.arange(9, dtype=np.uint32)] + [np.arange(8, dtype=np.uint32)] * len(self.trees))
        words = self.ops.B.gather_words(tensors, slots, idx)
        for i, tree in enumerate(self.trees):
            tree._root = words[9 + 8 * i:17 + 8 * i].astype("<u4").tobytes()
            self.channel.log.append(("mix_root", tree._root.hex()))
        self.channel.digest = words[:8].astype("<u4").tobytes()
        self.channel.n_draws = int(words[8])


class PlainGpuOps(GpuOps):
    """The plain CUDA form: the same kernels, one launch per column for every
    per-column stage (interpolate, evaluate), as a backend without batched
    overrides calls them (the default PolyOps::interpolate_columns /
    evaluate_polynomials loop, crates/stwo/src/prover/poly/circle/ops.rs:25-40,102-140), and
    the FRI layer loop launched eagerly every time (no graph)."""

    fri_graphs = False

    def interpolate(self, cols, tw):
        for c in cols:
            self.B.interpolate_columns([c], tw)

    def evaluate(self, coeffs, log_size, tw):
        return [self.B.evaluate_polynomials([c], log_size, tw)[0] for c in coeffs]

    def interpolate_secure(self, accum, tw):
        for c in accum.columns:
            self.B.interpolate_columns([c], tw)
        return accum.columns
