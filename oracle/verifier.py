"""ORACLE — test infrastructure only: the reference verifier restated for the
proofs of proving_gb300.prover and proving_gb300.air_prover (acceptance check):
Wide-Fibonacci components, their LogUp neighbours, and any AIR recorded by the
constraint evaluator (verify_components).

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
    if len(queried_values) != len(column_log_sizes) or any(len(v) != len(query_positions) for v in queried_values):
        raise VerificationError("queried values do not match the columns and queries")
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


def _draw_oods(ch, proof):
    """The OODS proof of work and point (crates/stwo/src/core/verifier.rs:55-62)."""
    if not ch.verify_pow_nonce(16, proof.oods_proof_of_work):
        raise VerificationError("OODS proof of work")
    ch.mix_u64(proof.oods_proof_of_work)
    t = ch.draw_secure_felt()
    px, py = O.random_point_from_t(t)
    return (tuple(int(v) for v in px), tuple(int(v) for v in py))


def _partial(ev):
    """SecureField::from_partial_evals: sum of ev[k] times the k-th basis element."""
    r = ev[0]
    for k, e in ((1, (0, 1, 0, 0)), (2, (0, 0, 1, 0)), (3, (0, 0, 0, 1))):
        r = qadd(r, qmul(ev[k], e))
    return r


def _composition_at_oods(comp_samples, oods, max_log_degree_bound):
    """The composition value from its split halves (crates/stwo/src/core/proof.rs:27-57) and
    1 / V(CanonicCoset(max_log_degree_bound)) at the point."""
    left = _partial([comp_samples[k][0] for k in range(4)])
    right = _partial([comp_samples[k][0] for k in range(4, 8)])
    x = oods[0]
    for _ in range(max_log_degree_bound - 1):
        x = qdouble_x(x)
    return qadd(left, qmul(x, right)), qinv(x)


def _fib_constraints(mask, n_cols_list):
    """Each Wide-Fibonacci component's constraints in order: c - (a^2 + b^2)."""
    out, start = [], 0
    for nc in n_cols_list:
        m = mask[start:start + nc]
        out += [qsub(m[k + 2], qadd(qmul(m[k], m[k]), qmul(m[k + 1], m[k + 1]))) for k in range(nc - 2)]
        start += nc
    return out


def _qpoint_add(p, q):
    return (qsub(qmul(p[0], q[0]), qmul(p[1], q[1])), qadd(qmul(p[0], q[1]), qmul(p[1], q[0])))


def verify_wide_fib_components(proof, n_cols_list, log_sizes):
    """Wide-Fibonacci components in one proof, their columns in one lifted trace tree (the verifier
    side of test_e2e_lifted_fib_prove, crates/examples/src/wide_fibonacci/mod.rs:553-575)."""
    n_cols = sum(n_cols_list)
    cfg = proof.config
    b = cfg.fri_params.log_blowup_factor
    ch = O.Blake2sChannel()
    # commitments of the preprocessed (empty) tree and the trace tree (test flow,
    # crates/examples/src/wide_fibonacci/mod.rs:228-231)
    ch.mix_root(proof.commitments[0])
    ch.mix_root(proof.commitments[1])
    lifting = cfg.trace_lifting_log_size
    max_log_degree_bound = lifting - b
    random_coeff = tuple(int(v) for v in ch.draw_secure_felt())
    ch.mix_root(proof.commitments[2])
    oods = _draw_oods(ch, proof)

    sv = proof.sampled_values
    if len(sv) != 3 or len(sv[0]) != 0 or len(sv[1]) != n_cols or len(sv[2]) != 8:
        raise VerificationError("unexpected sampled_values structure")
    comp, dinv = _composition_at_oods(sv[2], oods, max_log_degree_bound)
    # the AIR at the OODS point (Components::eval_composition_polynomial_at_point: Horner accumulation)
    acc = qm(0)
    for cons in _fib_constraints([c[0] for c in sv[1]], n_cols_list):
        acc = qadd(qmul(acc, random_coeff), qmul(cons, dinv))
    if comp != acc:
        raise VerificationError("OODS values do not match the AIR")

    sample_points = [[], [[oods]] * n_cols, [[oods]] * 8]
    sizes = [[], [log_n + b for nc, log_n in zip(n_cols_list, log_sizes) for _ in range(nc)],
             [max_log_degree_bound + b] * 8]
    _verify_values(proof, ch, sample_points, sizes, [0, lifting, lifting])


def verify_fib_and_lookups(proof, n_cols_list, fib_logs, lookup_logs, claimed_sums):
    """Wide-Fibonacci components and single-column LogUp components in one proof (the proof of
    proving_gb300.prover.prove_fib_and_lookups). The claimed sums are the statement: mixed into the
    channel before the interaction commitment. Each LogUp component's constraint at the point is
    (cur - prev + claimed / 2^n) (v - z) + 1 (crates/constraint-framework/src/logup.rs:95-150),
    its interaction columns sampled at (point - G, point)."""
    cfg = proof.config
    b = cfg.fri_params.log_blowup_factor
    lifting = cfg.trace_lifting_log_size
    max_log_degree_bound = lifting - b
    n_fib = sum(n_cols_list)
    n_look = len(lookup_logs)
    ch = O.Blake2sChannel()
    ch.mix_root(proof.commitments[0])
    ch.mix_root(proof.commitments[1])
    z = tuple(int(v) for v in ch.draw_secure_felt())
    ch.draw_secure_felt()  # alpha
    ch.mix_felts(np.asarray([list(c) for c in claimed_sums], np.uint32).reshape(-1, 4))
    ch.mix_root(proof.commitments[2])
    random_coeff = tuple(int(v) for v in ch.draw_secure_felt())
    ch.mix_root(proof.commitments[3])
    oods = _draw_oods(ch, proof)

    sv = proof.sampled_values
    if (len(sv) != 4 or len(sv[0]) != 0 or len(sv[1]) != n_fib + n_look or len(sv[2]) != 4 * n_look
            or len(sv[3]) != 8 or any(len(c) != 2 for c in sv[2])):
        raise VerificationError("unexpected sampled_values structure")
    comp, dinv = _composition_at_oods(sv[3], oods, max_log_degree_bound)
    mask = [c[0] for c in sv[1]]
    constraints = _fib_constraints(mask[:n_fib], n_cols_list)
    for k, log_n in enumerate(lookup_logs):
        v = mask[n_fib + k]
        prev = _partial([sv[2][4 * k + j][0] for j in range(4)])
        cur = _partial([sv[2][4 * k + j][1] for j in range(4)])
        shift = qmul(tuple(int(c) for c in claimed_sums[k]), qm(pow(1 << log_n, P - 2, P)))
        constraints.append(qadd(qmul(qadd(qsub(cur, prev), shift), qsub(v, z)), qm(1)))
    acc = qm(0)
    for cons in constraints:
        acc = qadd(qmul(acc, random_coeff), qmul(cons, dinv))
    if comp != acc:
        raise VerificationError("OODS values do not match the AIR")

    # the previous row: the point minus the generator of CanonicCoset(max_log_degree_bound)
    g = point_of_index(1 << (31 - max_log_degree_bound))
    prev_pt = _qpoint_add(oods, (qm(int(g[0])), qm(-int(g[1]))))
    sample_points = [[], [[oods]] * (n_fib + n_look), [[prev_pt, oods]] * (4 * n_look), [[oods]] * 8]
    trace_sizes = [log_n + b for nc, log_n in zip(n_cols_list, fib_logs) for _ in range(nc)]
    trace_sizes += [log_n + b for log_n in lookup_logs]
    sizes = [[], trace_sizes, [log_n + b for log_n in lookup_logs for _ in range(4)],
             [max_log_degree_bound + b] * 8]
    _verify_values(proof, ch, sample_points, sizes, [0, lifting, lifting, lifting])


def _air_at_point(air, mask, params):
    """An AIR's constraints at a point (PointEvaluator, crates/constraint-framework/src/point.rs:
    12-64) from its expression DAG: mask values and parameters are QM31, four base values combine
    as from_partial_evals."""
    memo = {}

    def ev(x):
        if x.key in memo:
            return memo[x.key]
        if x.op == "mask":
            v = tuple(mask[x.args])
        elif x.op == "const":
            v = qm(x.args[0])
        elif x.op == "param":
            v = tuple(int(c) % P for c in params[x.args[0]])
        elif x.op == "secure":
            v = _partial([ev(c) for c in x.args])
        elif x.op == "neg":
            v = qsub(qm(0), ev(x.args[0]))
        else:
            u, w = ev(x.args[0]), ev(x.args[1])
            v = {"add": qadd, "sub": qsub, "mul": qmul}[x.op](u, w)
        memo[x.key] = v
        return v
    return [ev(c) for c in air.constraints]


def verify_components(proof, ch, components, column_log_sizes, preprocessed_columns=(),
                      include_all_preprocessed_columns=False):
    """verify (crates/stwo/src/core/verifier.rs:19-119) for components written against the
    constraint evaluator, after the caller has replayed the trees' commitments and its own draws on
    ch (as the reference's verifier-side example code does). components: (air, log_size, params)
    in proving order. column_log_sizes: per committed tree (the composition's aside), the log size
    of every column's trace domain (CommitmentSchemeVerifier::commit's log_sizes). The columns of
    each tree are taken by the components in order, the preprocessed tree's by id from
    preprocessed_columns. The last commitment is the composition tree's."""
    cfg = proof.config
    b = cfg.fri_params.log_blowup_factor
    lifting = cfg.trace_lifting_log_size
    mldb = lifting - b
    n_trees = len(proof.commitments) - 1
    if len(column_log_sizes) != n_trees:
        raise VerificationError("one list of column sizes per committed tree")
    random_coeff = tuple(int(v) for v in ch.draw_secure_felt())
    ch.mix_root(proof.commitments[-1])
    oods = _draw_oods(ch, proof)

    # every tree's sample points: the components' mask offsets in steps of CanonicCoset(mldb)
    points = [[[] for _ in sizes] for sizes in column_log_sizes]
    pre = list(preprocessed_columns)
    taken = [0] * n_trees
    places = []
    for air, log_size, _ in components:
        place = {}
        for tree, cols in air.mask_offsets.items():
            if tree >= n_trees or taken[tree] + len(cols) > len(column_log_sizes[tree]):
                raise VerificationError("a component reads columns that were not committed")
            place[tree] = taken[tree]
            for offsets in cols:
                if column_log_sizes[tree][taken[tree]] != log_size:
                    raise VerificationError("a component's column has another size")
                pts = []
                for o in offsets:
                    g = point_of_index((o * (1 << (31 - mldb))) % (1 << 31))
                    pts.append(_qpoint_add(oods, (qm(int(g[0])), qm(int(g[1])))))
                points[tree][taken[tree]] = pts
                taken[tree] += 1
        pidx = []
        for name in air.preprocessed:
            if name not in pre:
                raise VerificationError(f"preprocessed column {name} is not committed")
            pidx.append(pre.index(name))
            points[0][pidx[-1]] = [oods]
        places.append((place, pidx))
    if include_all_preprocessed_columns:
        points[0] = [[oods] for _ in column_log_sizes[0]]
    sv = proof.sampled_values
    if (len(sv) != n_trees + 1 or any(len(sv[t]) != len(points[t]) for t in range(n_trees)) or len(sv[-1]) != 8
            or any(len(sv[t][c]) != len(points[t][c]) for t in range(n_trees) for c in range(len(points[t])))):
        raise VerificationError("unexpected sampled_values structure")

    # the components' constraints at the point against the composition polynomial's value
    comp, dinv = _composition_at_oods(sv[-1], oods, mldb)
    acc = qm(0)
    for (air, _, params), (place, pidx) in zip(components, places):
        mask = {}
        for tree, cols in air.mask_offsets.items():
            for k, offsets in enumerate(cols):
                for j, o in enumerate(offsets):
                    mask[(tree, k, o)] = sv[tree][place[tree] + k][j]
        for k, idx in enumerate(pidx):
            mask[(0, k, 0)] = sv[0][idx][0]
        for cons in _air_at_point(air, mask, params):
            acc = qadd(qmul(acc, random_coeff), qmul(cons, dinv))
    if comp != acc:
        raise VerificationError("OODS values do not match the AIR")

    heights = [lifting if column_log_sizes[t] else 0 for t in range(n_trees)] + [lifting]
    sizes = [[ls + b for ls in tree] for tree in column_log_sizes] + [[mldb + b] * 8]
    _verify_values(proof, ch, points + [[[oods]] * 8], sizes, heights)


def _verify_values(proof, ch, sample_points, sizes, heights):
    """verify_values (crates/stwo/src/core/pcs/verifier.rs:56-140) with the FRI verifier: sample_points
    and sizes per tree and column (the column's evaluation log size), heights per tree."""
    cfg = proof.config
    fp = cfg.fri_params
    lifting = cfg.trace_lifting_log_size
    max_log_degree_bound = lifting - fp.log_blowup_factor
    sv = proof.sampled_values
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
    for tree in range(len(heights)):
        merkle_verify(proof.commitments[tree], heights[tree], sizes[tree], queries, proof.queried_values[tree],
                      proof.decommitments[tree])

    # fri_answers: the DEEP quotient at every query (quotients.rs:115-184). Samples in tree and column
    # order, each with the next power of the quotient coefficient; a column sampled at (previous row,
    # point) first opens the point shifted by the period G_(lifting - log size) with the point's
    # value (build_samples_with_randomness_and_periodicity, crates/stwo/src/core/pcs/quotients.rs:274-319).
    entries = []  # (point, value, queried values of the column)
    for tree, (pts_t, sv_t) in enumerate(zip(sample_points, sv)):
        for ci, (pts, vals) in enumerate(zip(pts_t, sv_t)):
            col = proof.queried_values[tree][ci]
            if len(pts) == 2:
                per = point_of_index(1 << (31 - (lifting - sizes[tree][ci])))
                entries.append((_qpoint_add(pts[1], (qm(int(per[0])), qm(int(per[1])))), tuple(vals[1]), col))
            for pt, v in zip(pts, vals):
                entries.append((pt, tuple(v), col))
    pow_ = qm(1)
    coeffs = []
    for pt, v, col in entries:
        a = qsub(qconj(v), v)
        c = qsub(qconj(pt[1]), pt[1])
        bb = qsub(qmul(v, c), qmul(a, pt[1]))
        coeffs.append((pt, qmul(pow_, a), qmul(pow_, bb), qmul(pow_, c), col))
        pow_ = qmul(pow_, quot_coeff)

    def cmul(u, w):
        return ((u[0] * w[0] - u[1] * w[1]) % P, (u[0] * w[1] + u[1] * w[0]) % P)

    answers = []
    for k, pos in enumerate(queries):
        dx, dy = point_of_index(circle_domain_index(lifting, bitrev(pos, lifting)))
        total = qm(0)
        for pt, a, bb, c, col in coeffs:
            # denominator (prx - x) * piy - (pry - y) * pix in CM31
            prx, pix = (pt[0][0], pt[0][1]), (pt[0][2], pt[0][3])
            pry, piy = (pt[1][0], pt[1][1]), (pt[1][2], pt[1][3])
            d = tuple((s - t) % P for s, t in zip(cmul(((prx[0] - dx) % P, prx[1]), piy),
                                                    cmul(((pry[0] - dy) % P, pry[1]), pix)))
            n = pow((d[0] * d[0] + d[1] * d[1]) % P, P - 2, P)
            dinv_c = ((d[0] * n) % P, (-d[1] * n) % P)
            num = qsub(tuple((c_ * col[k]) % P for c_ in c), qadd(tuple((a_ * dy) % P for a_ in a), bb))
            r0 = cmul((num[0], num[1]), dinv_c)
            r1 = cmul((num[2], num[3]), dinv_c)
            total = qadd(total, (r0[0], r0[1], r1[0], r1[1]))
        answers.append(total)

    # FRI decommitment (fri.rs:306-399, 460-800): each layer's queries grouped in cosets of
    # 2^step positions, rebuilt from the previous layer's values and the witness, checked against
    # the layer's tree (leaves of 4 positions when step > 1 and the layer has 4 or more values,
    # build_merkle_verification_inputs) and folded step times into the next layer's values
    def rebuild(qs, evals, witness, step):
        wit = iter(witness)
        ev = iter(evals)
        positions, subsets, starts = [], [], []
        i = 0
        while i < len(qs):
            j = i
            while j + 1 < len(qs) and qs[j + 1] >> step == qs[i] >> step:
                j += 1
            group = set(qs[i:j + 1])
            start = (qs[i] >> step) << step
            vals = []
            for pos in range(start, start + (1 << step)):
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

    def check_layer(layer, log_size, positions, subsets, step):
        vals = [v for s in subsets for v in s]
        if step > 1 and log_size >= 2:
            # leaf r holds positions 4r..4r+3, column coord + 4 offset (pack_leaves_input)
            leaves = sorted(set(p_ >> 2 for p_ in positions))
            by_pos = dict(zip(positions, vals))
            cols = [[by_pos[4 * r + off][coord] for r in leaves] for off in range(4) for coord in range(4)]
            merkle_verify(layer["commitment"], log_size - 2, [log_size - 2] * 16, leaves, cols, layer["decommitment"])
        else:
            cols = [[v[c] for v in vals] for c in range(4)]
            merkle_verify(layer["commitment"], log_size, [log_size] * 4, positions, cols, layer["decommitment"])

    def ibfly(v0, v1, t):
        return qadd(v0, v1), tuple((x * t) % P for x in qsub(v0, v1))

    def fold_coset(vals, init, log_n, alpha):
        """fold_coset (fri.rs:770-800): values on the x-coordinates of Coset(init, log_n) in
        bit-reversed order folded log_n times, alpha squared after each fold, the domain doubled."""
        cur = list(vals)
        step_idx = (1 << (31 - log_n)) if log_n else 0
        a = alpha
        for i in range(log_n):
            n = log_n - i
            nxt = []
            for j in range(0, 1 << n, 2):
                x, _ = point_of_index(init + bitrev(j, n) * step_idx)
                f0, f1 = ibfly(cur[j], cur[j + 1], pow(x, P - 2, P))
                nxt.append(qadd(f0, qmul(a, f1)))
            cur = nxt
            init, step_idx, a = 2 * init, 2 * step_idx, qmul(a, a)
        return cur[0]

    # first layer: the circle fold, then fold_step - 1 line folds with alpha^2 (fold_circle)
    k = fp.fold_step
    pos, subsets, starts = rebuild(queries, answers, [tuple(w) for w in proof.fri_first_layer["fri_witness"]], k)
    check_layer(proof.fri_first_layer, column_log, pos, subsets, k)
    evals = []
    half_init = 1 << (31 - (column_log + 1))
    half_step = 1 << (31 - (column_log - 1))
    for sv_, start in zip(subsets, starts):
        # the subset's circle domain: half coset at the start's point, 2^(k-1) points
        init = (half_init + bitrev(start, column_log) * half_step) % (1 << 31)
        sub_step = (1 << (31 - (k - 1))) if k > 1 else 0
        line = []
        for j in range(0, 1 << k, 2):
            _, py_ = point_of_index(init + bitrev(j, k) * sub_step)
            f0, f1 = ibfly(sv_[j], sv_[j + 1], pow(py_, P - 2, P))
            line.append(qadd(f0, qmul(first_alpha, f1)))
        evals.append(fold_coset(line, init, k - 1, qmul(first_alpha, first_alpha)))
    qs = sorted(set(q >> k for q in queries))
    for layer, alpha, log_size, step in zip(proof.fri_inner_layers, inner_alphas, layer_logs, steps):
        pos, subsets, starts = rebuild(qs, evals, [tuple(w) for w in layer["fri_witness"]], step)
        check_layer(layer, log_size, pos, subsets, step)
        init0, lstep = 1 << (31 - (log_size + 2)), 1 << (31 - log_size)
        evals = [fold_coset(sv_, (init0 + bitrev(start, log_size) * lstep) % (1 << 31), step, alpha)
                 for sv_, start in zip(subsets, starts)]
        qs = sorted(set(q >> step for q in qs))
    # last layer (fri.rs:540-560): the polynomial, its coefficients bit-reversed, at each query's
    # point of the last line domain, by folding with the doublings of x (LinePoly::eval_at_point)
    last_log = line_log
    coeffs = [tuple(int(v) for v in c) for c in proof.fri_last_layer_poly]
    n_log = len(coeffs).bit_length() - 1
    if len(coeffs) != 1 << n_log:
        raise VerificationError("last layer size")

    def line_eval(cs, xs_):
        if len(cs) == 1:
            return cs[0]
        h = len(cs) // 2
        return qadd(line_eval(cs[:h], xs_[1:]), qmul(line_eval(cs[h:], xs_[1:]), xs_[0]))
    init0, lstep = 1 << (31 - (last_log + 2)), 1 << (31 - last_log)
    for q, e in zip(qs, evals):
        x, _ = point_of_index(init0 + bitrev(q, last_log) * lstep)
        xs_ = []
        xq = qm(x)
        for _ in range(n_log):
            xs_.append(xq)
            xq = qsub(qadd(qmul(xq, xq), qmul(xq, xq)), qm(1))
        if e != line_eval(coeffs, xs_):
            raise VerificationError("last layer evaluations invalid")


# ---------------------------------------------------------------- proof bytes

class _FriParams:
    def __init__(self, pow_bits, log_blowup_factor, log_last_layer_degree_bound, n_queries, fold_step):
        self.pow_bits, self.log_blowup_factor = pow_bits, log_blowup_factor
        self.log_last_layer_degree_bound, self.n_queries, self.fold_step = (log_last_layer_degree_bound, n_queries,
                                                                           fold_step)


class _PcsConfig:
    def __init__(self, fri_params, trace_lifting_log_size):
        self.fri_params, self.trace_lifting_log_size = fri_params, trace_lifting_log_size


class ParsedProof:
    """A StarkProof read back from its CairoSerialize felt stream (crates/cairo-serialize/src/
    serialize.rs:99-210). Every vector carries its length, so the stream is self-describing; the
    lifting log size is not serialized and is given by the statement."""


def parse_proof(data: bytes, trace_lifting_log_size: int) -> ParsedProof:
    w = np.frombuffer(data, "<u8").astype(np.uint64)
    pos = [0]

    def take():
        if pos[0] >= len(w):
            raise VerificationError("truncated proof")
        v = int(w[pos[0]])
        pos[0] += 1
        return v

    def vec(f):
        n = take()
        if n > len(w) - pos[0]:
            raise VerificationError("vector length beyond the proof")
        return [f() for _ in range(n)]

    def hsh():
        return struct.pack("<8I", *[take() for _ in range(8)])

    def q():
        return tuple(take() for _ in range(4))

    p = ParsedProof()
    p.config = _PcsConfig(_FriParams(*[take() for _ in range(5)]), trace_lifting_log_size)
    p.commitments = vec(hsh)
    p.oods_proof_of_work = take()
    p.sampled_values = vec(lambda: vec(lambda: vec(q)))
    p.decommitments = vec(lambda: vec(hsh))
    p.queried_values = vec(lambda: vec(lambda: vec(take)))

    def layer():
        return {"fri_witness": vec(q), "decommitment": vec(hsh), "commitment": hsh()}

    p.fri_first_layer = layer()
    p.fri_inner_layers = vec(layer)
    p.fri_last_layer_poly = vec(q)
    if take() != len(p.fri_last_layer_poly).bit_length() - 1:
        raise VerificationError("last layer log size")
    p.fri_proof_of_work = take()
    if pos[0] != len(w):
        raise VerificationError("trailing words after the proof")
    return p
