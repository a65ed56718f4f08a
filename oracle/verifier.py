"""ORACLE — test infrastructure only: the reference verifier restated for a
Wide-Fibonacci proof produced by proving_gb300.prover (acceptance check).

Follows verify_ex (crates/stwo/src/core/verifier.rs:30-119),
CommitmentSchemeVerifier (crates/stwo/src/core/pcs/verifier.rs:20-140),
fri_answers (crates/stwo/src/core/pcs/quotients.rs:115-184), FriVerifier
(crates/stwo/src/core/fri.rs:149-720) and MerkleVerifierLifted::verify
(crates/stwo/src/core/vcs_lifted/verifier.rs:107-200). The channel is the
C oracle's; field arithmetic here is written independently of the prover.
Raises VerificationError on the first failed check.
"""
from __future__ import annotations

import hashlib
import struct

import numpy as np

from . import oracle as O

P = O.P


class VerificationError(Exception):
    pass


# ---------------------------------------------------------------- field helpers

def _q(x):
    return np.asarray([int(v) % P for v in x], np.uint32)


def qmul(x, y):
    return tuple(int(v) for v in O.qm31_mul(_q(x), _q(y)))


def qinv(x):
    return tuple(int(v) for v in O.qm31_inv(_q(x)))


def qadd(x, y):
    return tuple((a + b) % P for a, b in zip(x, y))


def qsub(x, y):
    return tuple((a - b) % P for a, b in zip(x, y))


def qm(a):
    return (a % P, 0, 0, 0)


def qconj(x):
    return (x[0], x[1], (-x[2]) % P, (-x[3]) % P)


def qdouble_x(x):
    s = qmul(x, x)
    return qsub(qadd(s, s), qm(1))


def bitrev(i, n):
    return int(O.bit_reverse(np.arange(1 << n, dtype=np.uint32))[i]) if n else i


def point_of_index(idx):
    return O.circle_index_to_point(idx & ((1 << 31) - 1))


def circle_domain_index(log_size, j):
    half_init, half_step, hs = 1 << (31 - (log_size + 1)), 1 << (31 - (log_size - 1)), 1 << (log_size - 1)
    mask = (1 << 31) - 1
    if j < hs:
        return (half_init + j * half_step) & mask
    return (-(half_init + (j - hs) * half_step)) & mask


# ---------------------------------------------------------------- Merkle

def merkle_verify(root, height, column_log_sizes, query_positions, queried_values, witness):
    """MerkleVerifierLifted::verify (crates/stwo/src/core/vcs_lifted/verifier.rs:107-200)."""
    if height == 0:
        return
    order = sorted(range(len(column_log_sizes)), key=lambda i: column_log_sizes[i])
    by_pos = {}
    for k, pos in enumerate(query_positions):
        vals = [queried_values[i][k] for i in order]
        if pos in by_pos and by_pos[pos] != vals:
            raise VerificationError("inconsistent duplicate query values")
        by_pos[pos] = vals
    layer = [(pos, hashlib.blake2s(b"".join(struct.pack("<I", v) for v in by_pos[pos])).digest())
             for pos in sorted(by_pos)]
    wit = iter(witness)
    for _ in range(height):
        nxt, i = [], 0
        while i < len(layer):
            idx0, h0 = layer[i]
            if i + 1 < len(layer) and layer[i + 1][0] == idx0 ^ 1:
                children = (h0, layer[i + 1][1])
                i += 2
            else:
                try:
                    w = next(wit)
                except StopIteration:
                    raise VerificationError("Merkle witness too short")
                children = (h0, w) if idx0 & 1 == 0 else (w, h0)
                i += 1
            nxt.append((idx0 >> 1, hashlib.blake2s(children[0] + children[1]).digest()))
        layer = nxt
    if next(wit, None) is not None:
        raise VerificationError("Merkle witness too long")
    if len(layer) != 1 or layer[0][1] != root:
        raise VerificationError("Merkle root mismatch")


# ---------------------------------------------------------------- verify

def verify_wide_fib(proof, n_cols: int, log_n_rows: int):
    verify_wide_fib_components(proof, [n_cols], [log_n_rows])


def verify_wide_fib_components(proof, n_cols_list, log_sizes):
    """Wide-Fibonacci components in one proof, their columns in one lifted trace tree (the verifier
    side of test_e2e_lifted_fib_prove, crates/examples/src/wide_fibonacci/mod.rs:553-575)."""
    n_cols = sum(n_cols_list)
    cfg = proof.config
    fp = cfg.fri_params
    b = fp.log_blowup_factor
    ch = O.Blake2sChannel()
    # commitments of the preprocessed (empty) tree and the trace tree (test flow,
    # crates/examples/src/wide_fibonacci/mod.rs:228-231)
    ch.mix_root(proof.commitments[0])
    ch.mix_root(proof.commitments[1])
    lifting = cfg.trace_lifting_log_size
    max_log_degree_bound = lifting - b
    random_coeff = tuple(int(v) for v in ch.draw_secure_felt())
    ch.mix_root(proof.commitments[2])
    if not ch.verify_pow_nonce(16, proof.oods_proof_of_work):
        raise VerificationError("OODS proof of work")
    ch.mix_u64(proof.oods_proof_of_work)
    t = ch.draw_secure_felt()
    px, py = O.random_point_from_t(t)
    oods = (tuple(int(v) for v in px), tuple(int(v) for v in py))

    sv = proof.sampled_values
    if len(sv) != 3 or len(sv[0]) != 0 or len(sv[1]) != n_cols or len(sv[2]) != 8:
        raise VerificationError("unexpected sampled_values structure")
    # composition value from the split halves (crates/stwo/src/core/proof.rs:27-57)
    def partial(ev):
        r = ev[0]
        for k, e in ((1, (0, 1, 0, 0)), (2, (0, 0, 1, 0)), (3, (0, 0, 0, 1))):
            r = qadd(r, qmul(ev[k], e))
        return r
    left = partial([sv[2][k][0] for k in range(4)])
    right = partial([sv[2][k][0] for k in range(4, 8)])
    x = oods[0]
    for _ in range(max_log_degree_bound - 1):
        x = qdouble_x(x)
    comp = qadd(left, qmul(x, right))
    # the AIR at the OODS point (Horner accumulation, denominator V_trace(oods))
    xv = oods[0]
    for _ in range(max_log_degree_bound - 1):
        xv = qdouble_x(xv)
    dinv = qinv(xv)
    acc = qm(0)
    mask = [c[0] for c in sv[1]]
    start = 0
    for nc in n_cols_list:
        # each component's constraints in order (Components::eval_composition_polynomial_at_point)
        m = mask[start:start + nc]
        for k in range(nc - 2):
            cons = qsub(m[k + 2], qadd(qmul(m[k], m[k]), qmul(m[k + 1], m[k + 1])))
            acc = qadd(qmul(acc, random_coeff), qmul(cons, dinv))
        start += nc
    if comp != acc:
        raise VerificationError("OODS values do not match the AIR")

    # --- verify_values (pcs/verifier.rs:56-140)
    ch.mix_felts(np.asarray([list(v) for tree in sv for col in tree for v in col], np.uint32))
    quot_coeff = tuple(int(v) for v in ch.draw_secure_felt())
    # FRI commitment phase
    ch.mix_root(proof.fri_first_layer["commitment"])
    first_alpha = tuple(int(v) for v in ch.draw_secure_felt())
    column_log = lifting
    line_log = column_log - 1 - (fp.fold_step - 1)
    inner_alphas, layer_logs, steps = [], [], []
    bound = max_log_degree_bound - fp.fold_step
    n_inner = len(proof.fri_inner_layers)
    for li, layer in enumerate(proof.fri_inner_layers):
        ch.mix_root(layer["commitment"])
        step = fp.fold_step if li < n_inner - 1 else bound - fp.log_last_layer_degree_bound
        if not 1 <= step <= fp.fold_step:
            raise VerificationError("invalid number of FRI layers")
        inner_alphas.append(tuple(int(v) for v in ch.draw_secure_felt()))
        layer_logs.append(line_log)
        steps.append(step)
        bound -= step
        line_log -= step
    if bound != fp.log_last_layer_degree_bound:
        raise VerificationError("invalid number of FRI layers")
    if len(proof.fri_last_layer_poly) > (1 << fp.log_last_layer_degree_bound):
        raise VerificationError("last layer degree")
    ch.mix_felts(np.asarray([list(c) for c in proof.fri_last_layer_poly], np.uint32))
    if not ch.verify_pow_nonce(fp.pow_bits, proof.fri_proof_of_work):
        raise VerificationError("FRI proof of work")
    ch.mix_u64(proof.fri_proof_of_work)
    queries = sorted(set(int(q) for q in ch.draw_queries(column_log, fp.n_queries)))

    # tree decommitments
    sizes = [[], [log_n + b for nc, log_n in zip(n_cols_list, log_sizes) for _ in range(nc)],
             [max_log_degree_bound + b] * 8]
    heights = [0, lifting, lifting]
    for tree in range(3):
        merkle_verify(proof.commitments[tree], heights[tree], sizes[tree], queries, proof.queried_values[tree],
                      proof.decommitments[tree])

    # fri_answers: the DEEP quotient at every query (quotients.rs:115-184)
    samples = [(mask_col[0]) for mask_col in sv[1]] + [c[0] for c in sv[2]]
    queried = proof.queried_values[1] + proof.queried_values[2]
    pow_ = qm(1)
    coeffs = []
    for v in samples:
        a = qsub(qconj(v), v)
        c = qsub(qconj(oods[1]), oods[1])
        bb = qsub(qmul(v, c), qmul(a, oods[1]))
        coeffs.append((qmul(pow_, a), qmul(pow_, bb), qmul(pow_, c)))
        pow_ = qmul(pow_, quot_coeff)
    answers = []
    for k, pos in enumerate(queries):
        dx, dy = point_of_index(circle_domain_index(lifting, bitrev(pos, lifting)))
        # denominator (prx - x) * piy - (pry - y) * pix in CM31
        prx, pix = (oods[0][0], oods[0][1]), (oods[0][2], oods[0][3])
        pry, piy = (oods[1][0], oods[1][1]), (oods[1][2], oods[1][3])
        def cmul(u, w):
            return ((u[0] * w[0] - u[1] * w[1]) % P, (u[0] * w[1] + u[1] * w[0]) % P)
        d = tuple((s - t) % P for s, t in zip(cmul(((prx[0] - dx) % P, prx[1]), piy),
                                                cmul(((pry[0] - dy) % P, pry[1]), pix)))
        n = pow((d[0] * d[0] + d[1] * d[1]) % P, P - 2, P)
        dinv_c = ((d[0] * n) % P, (-d[1] * n) % P)
        num = qm(0)
        for (a, bb, c), col in zip(coeffs, queried):
            num = qadd(num, qsub(tuple((c_ * col[k]) % P for c_ in c), qadd(tuple((a_ * dy) % P for a_ in a), bb)))
        r0 = cmul((num[0], num[1]), dinv_c)
        r1 = cmul((num[2], num[3]), dinv_c)
        answers.append((r0[0], r0[1], r1[0], r1[1]))

    # FRI decommitment (fri.rs:306-399, 460-720), fold_step 1
    def rebuild(qs, evals, witness):
        wit = iter(witness)
        ev = iter(evals)
        positions, subsets, starts = [], [], []
        i = 0
        while i < len(qs):
            j = i
            while j + 1 < len(qs) and qs[j + 1] >> 1 == qs[i] >> 1:
                j += 1
            group = qs[i:j + 1]
            start = (group[0] >> 1) << 1
            vals = []
            for pos in (start, start + 1):
                positions.append(pos)
                if pos in group:
                    vals.append(next(ev))
                else:
                    try:
                        vals.append(next(wit))
                    except StopIteration:
                        raise VerificationError("insufficient FRI witness")
            subsets.append(vals)
            starts.append(start)
            i = j + 1
        if next(wit, None) is not None:
            raise VerificationError("FRI witness too long")
        return positions, subsets, starts

    def check_layer(layer, log_size, positions, subsets):
        vals = [v for s in subsets for v in s]
        cols = [[v[c] for v in vals] for c in range(4)]
        merkle_verify(layer["commitment"], log_size, [log_size] * 4, positions, cols, layer["decommitment"])

    def ibfly(v0, v1, t):
        return qadd(v0, v1), tuple((x * t) % P for x in qsub(v0, v1))

    pos, subsets, starts = rebuild(queries, answers, [tuple(w) for w in proof.fri_first_layer["fri_witness"]])
    check_layer(proof.fri_first_layer, column_log, pos, subsets)
    evals = []
    for s, start in zip(subsets, starts):
        _, py_ = point_of_index(circle_domain_index(column_log, bitrev(start, column_log)))
        f0, f1 = ibfly(s[0], s[1], pow(py_, P - 2, P))
        evals.append(qadd(qmul(first_alpha, f1), f0))
    qs = sorted(set(q >> 1 for q in queries))
    for layer, alpha, log_size in zip(proof.fri_inner_layers, inner_alphas, layer_logs):
        pos, subsets, starts = rebuild(qs, evals, [tuple(w) for w in layer["fri_witness"]])
        check_layer(layer, log_size, pos, subsets)
        evals = []
        init, step = 1 << (31 - (log_size + 2)), 1 << (31 - log_size)
        for s, start in zip(subsets, starts):
            x, _ = point_of_index(init + bitrev(start, log_size) * step)
            f0, f1 = ibfly(s[0], s[1], pow(x, P - 2, P))
            evals.append(qadd(f0, qmul(alpha, f1)))
        qs = sorted(set(q >> 1 for q in qs))
    # last layer: a constant polynomial
    if fp.log_last_layer_degree_bound != 0:
        raise NotImplementedError("last layer degree bound > 0")
    for e in evals:
        if e != tuple(proof.fri_last_layer_poly[0]):
            raise VerificationError("last layer evaluations invalid")
