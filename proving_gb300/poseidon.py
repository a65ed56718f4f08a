"""The Poseidon2 example prover (crates/examples/src/poseidon/mod.rs:305-379),
restated on the host over a backend, with the device doing the trace, the
LogUp interaction trace and the constraint quotients.

`prove_poseidon` follows `prove_poseidon` and then `prove_ex`
(crates/stwo/src/prover/mod.rs:39-138) call for call: the empty preprocessed
tree, the trace tree, the lookup elements, the interaction tree, the
composition polynomial (EvaluationMode::ExtendToEvalDomain: the trace
polynomials evaluated on CanonicCoset(log_n_rows + 2),
crates/stwo/src/prover/air/accumulation.rs:42-62), the OODS samples with the
LogUp column's previous-row mask and its periodicity sample, FRI and the
decommitments.

The reference cannot finish this proof: its own prove test for the AIR is
ignored upstream ("AIRs with constraint degree >= 2 are not supported yet in
the lifted protocol"). With pcs config `poseidon_pcs_config` the trace is
committed lifted by one level while the composition polynomial is not, so the
out-of-domain sanity check of prove_ex compares the composition at the OODS
point p with the constraints at 2p and fails (ProvingError::ConstraintsNotSatisfied).
`prove_poseidon` reproduces that: by default it raises the same error after
building the proof; with check=False it returns the proof words the reference
computes before its check, so two backends can be compared byte for byte.
"""
from __future__ import annotations

import hashlib

import numpy as np

from . import prover as pr
from .prover import P, qm, qm_add, qm_inv, qm_mul, qm_sub, qv_mul, qv_sub, qv_sum

N_STATE = 16
N_PARTIAL_ROUNDS = 14
N_HALF_FULL_ROUNDS = 4
N_INSTANCES = 8
N_COLUMNS_PER_REP = N_STATE * (1 + 2 * N_HALF_FULL_ROUNDS) + N_PARTIAL_ROUNDS  # 158
N_COLUMNS = N_INSTANCES * N_COLUMNS_PER_REP  # 1264
N_INTERACTION_COLUMNS = 4 * N_INSTANCES  # 32
N_CONSTRAINTS = N_INSTANCES * (2 * N_HALF_FULL_ROUNDS * N_STATE + N_PARTIAL_ROUNDS) + N_INSTANCES  # 1144
LOG_EXPAND = 2
ROUND_CONST = 1234
COMPOSITION_LOG_SPLIT = 1  # crates/stwo/src/core/verifier.rs:17


class ConstraintsNotSatisfied(RuntimeError):
    """ProvingError::ConstraintsNotSatisfied (crates/stwo/src/prover/mod.rs:137-145)."""


def poseidon_pcs_config(log_n_instances: int, fri_params: pr.FriParams) -> pr.PcsConfig:
    """poseidon_pcs_config (mod.rs:305-318)."""
    log_n_rows = log_n_instances - 3
    return pr.PcsConfig(fri_params, trace_lifting_log_size=log_n_rows + LOG_EXPAND - COMPOSITION_LOG_SPLIT
                        + fri_params.log_blowup_factor)


# ------------------------------------------------------------ the AIR at a point

_M4 = np.array([[5, 7, 1, 3], [4, 6, 1, 1], [1, 3, 5, 7], [1, 1, 4, 6]], np.int64)
# apply_external_round_matrix = circ(2 M4, M4, M4, M4) (mod.rs:91-113)
EXTERNAL = np.block([[2 * _M4 if i == j else _M4 for j in range(4)] for i in range(4)])
# apply_internal_round_matrix: all ones plus 2^(i+1) on the diagonal (mod.rs:115-129)
INTERNAL = np.ones((N_STATE, N_STATE), np.int64) + np.diag([1 << (i + 1) for i in range(N_STATE)])


def _mat(m, s):
    """m (16x16 small integers) applied to states s (..., 16, 4) coordinate-wise."""
    return np.einsum("ij,...jc->...ic", m, s) % P


def _pow5(x):
    x2 = qv_mul(x, x)
    return qv_mul(qv_mul(x2, x2), x)


def _from_partial_evals(v):
    """QM31::from_partial_evals (crates/stwo/src/core/fields/qm31.rs:48-54) on 4 QM31 values."""
    return pr.from_partial_evals([tuple(int(c) for c in x) for x in v])


def composition_at_point(point, trace_mask, inter_mask, lookup, claimed, random_coeff, max_log_degree_bound: int,
                         log_n_rows: int):
    """eval_composition_polynomial_at_point for the Poseidon component (PointEvaluator,
    crates/constraint-framework/src/point.rs; component.rs:220-243): the 1144 constraints on the
    sampled values, in evaluation order, Horner-combined with random_coeff and divided by
    V(CanonicCoset(max_log_degree_bound)) at the point. trace_mask: 1264 QM31; inter_mask: per
    interaction column its samples (the last four have [previous row, row])."""
    tm = np.asarray(trace_mask, np.int64).reshape(N_INSTANCES, N_COLUMNS_PER_REP, 4)
    s = tm[:, :N_STATE].copy()
    init = s.copy()
    rc_const = np.array([ROUND_CONST, 0, 0, 0], np.int64)
    round_cons = [[] for _ in range(N_INSTANCES)]
    c = N_STATE

    def full_round(s, c):
        s = _mat(EXTERNAL, (s + rc_const) % P)
        m = tm[:, c:c + N_STATE]
        cons = qv_sub(_pow5(s), m)
        for k in range(N_INSTANCES):
            round_cons[k].append(cons[k])
        return m.copy(), c + N_STATE

    for _ in range(N_HALF_FULL_ROUNDS):
        s, c = full_round(s, c)
    for _ in range(N_PARTIAL_ROUNDS):
        s[:, 0] = (s[:, 0] + rc_const) % P
        s = _mat(INTERNAL, s)
        m = tm[:, c]
        cons = qv_sub(_pow5(s[:, 0]), m)
        for k in range(N_INSTANCES):
            round_cons[k].append(cons[k][None])
        s[:, 0] = m
        c += 1
    for _ in range(N_HALF_FULL_ROUNDS):
        s, c = full_round(s, c)
    cons = [np.concatenate(rc_k, axis=0) for rc_k in round_cons]  # 8 x (142, 4)

    # LogUp batches (finalize_logup_in_pairs, crates/constraint-framework/src/lib.rs:185-232)
    z = np.asarray(lookup[:4], np.int64)
    alpha = tuple(int(x) for x in lookup[4:])
    ap = np.asarray(pr.secure_powers(alpha, N_STATE), np.int64)  # (16, 4)

    def combine(vals):  # (8, 16, 4) -> (8, 4)
        return qv_sub(qv_sum(qv_mul(vals, ap[None]).transpose(1, 0, 2)), z)

    d0, d1 = combine(init), combine(s)
    num, den = qv_sub(d1, d0), qv_mul(d0, d1)
    shift = qm_mul(tuple(int(x) for x in claimed), qm(pr.m_inv(1 << log_n_rows)))
    prev_col = qm(0)
    logup_cons = []
    for k in range(N_INSTANCES):
        samples = inter_mask[4 * k:4 * k + 4]
        cur = _from_partial_evals([col[-1] for col in samples])
        diff = qm_sub(cur, prev_col)
        if k == N_INSTANCES - 1:
            prev_row = _from_partial_evals([col[0] for col in samples])
            diff = qm_add(qm_sub(diff, prev_row), shift)
        prev_col = cur
        logup_cons.append(qm_sub(qm_mul(diff, tuple(int(x) for x in den[k])), tuple(int(x) for x in num[k])))
    all_cons = np.concatenate(cons + [np.asarray(logup_cons, np.int64)], axis=0)
    assert all_cons.shape[0] == N_CONSTRAINTS
    powers = np.asarray(list(reversed(pr.secure_powers(random_coeff, N_CONSTRAINTS))), np.int64)
    total = tuple(int(v) for v in qv_sum(qv_mul(all_cons, powers)))
    x = point[0]
    for _ in range(max_log_degree_bound - 1):
        x = pr.q_double_x(x)
    return qm_mul(total, qm_inv(x))


# ------------------------------------------------------------ the prover

def prove_poseidon(ops, log_n_rows: int, config: pr.PcsConfig, channel: pr.Blake2sChannel, twiddles,
                   check: bool = True, generic: bool = False):
    """prove_poseidon (mod.rs:320-379) + prove_ex (crates/stwo/src/prover/mod.rs:39-138).
    twiddles: for CanonicCoset(log_n_rows + LOG_EXPAND + log_blowup_factor). generic=True evaluates
    the constraints through the generic path (proving_gb300.framework.poseidon_air, a run-time
    compiled kernel) instead of the hand-written composition kernel."""
    fp = config.fri_params
    b = fp.log_blowup_factor
    L = config.trace_lifting_log_size
    n = log_n_rows

    # --- preprocessed tree: empty (mod.rs:342-348)
    pre_root = hashlib.blake2s(b"").digest()
    channel.mix_root(pre_root)

    # --- trace (mod.rs:350-356); the evaluations stay for the interaction trace
    trace = ops.poseidon_trace(n)
    trace_coeffs = ops.interpolate_into(trace, twiddles)
    trace_ext = ops.evaluate(trace_coeffs, n + b, twiddles)
    trace_tree = ops.merkle_commit(trace_ext, L)
    channel.mix_root(trace_tree.root)

    # --- lookup elements (PoseidonElements::draw, crates/constraint-framework/src/logup.rs:70-79)
    z = channel.draw_secure_felt()
    alpha = channel.draw_secure_felt()
    lookup = list(z) + list(alpha)

    # --- interaction trace (mod.rs:361-367)
    inter, claimed = ops.poseidon_interaction(trace, lookup)
    del trace
    claimed = tuple(int(x) for x in claimed)
    ops.interpolate(inter, twiddles)
    inter_coeffs = inter
    inter_ext = ops.evaluate(inter_coeffs, n + b, twiddles)
    inter_tree = ops.merkle_commit(inter_ext, L)
    channel.mix_root(inter_tree.root)

    # --- composition polynomial (air/component_prover.rs:95-116)
    random_coeff = channel.draw_secure_felt()
    eval_log = n + LOG_EXPAND
    # EvaluationMode::infer: constraint log degree LOG_EXPAND > log_blowup_factor -> ExtendToEvalDomain;
    # equal -> SubDomain{0}, whose evaluation domain is the committed one (the same values)
    if LOG_EXPAND > b:
        trace_eval = ops.evaluate(trace_coeffs, eval_log, twiddles)
        inter_eval = ops.evaluate(inter_coeffs, eval_log, twiddles)
    elif LOG_EXPAND == b:
        trace_eval, inter_eval = trace_ext, inter_ext
    else:
        raise NotImplementedError("log_blowup_factor above the constraint degree (SubDomain with expansion)")
    rc = np.asarray(list(reversed(pr.secure_powers(random_coeff, N_CONSTRAINTS))), np.uint32)
    accum = ops.secure_zeros(1 << eval_log)
    if generic:
        from . import framework as fw
        ops.air_composition(fw.poseidon_air_recorded(), {1: trace_eval, 2: inter_eval}, n,
                            fw.poseidon_params(lookup, claimed, n), rc, accum)
    else:
        ops.poseidon_composition(trace_eval, inter_eval, n, lookup, claimed, rc, accum)
    del trace_eval, inter_eval
    comp_coeffs = ops.interpolate_secure(accum, twiddles)
    left, right = ops.split_at_mid(comp_coeffs)
    comp_evals = ops.evaluate(left + right, (eval_log - 1) + b, twiddles)
    comp_tree = ops.merkle_commit(comp_evals, L)
    channel.mix_root(comp_tree.root)

    # --- OODS proof of work and point (mod.rs:75-83)
    oods_pow = ops.grind(channel.digest, pr.OODS_POW_BITS)
    channel.mix_u64(oods_pow)
    oods = pr.random_point(channel.draw_secure_felt())

    # --- mask points (crates/constraint-framework/src/component.rs:202-214): offsets in steps of
    # CanonicCoset(max_log_degree_bound); the last LogUp column is also read at offset -1
    lifting = L
    mldb = lifting - b
    g = pr.m31_subgroup_generator(mldb)
    prev_pt = pr.qpoint_add_m31(oods, (g[0], (-g[1]) % P))
    inter_points = [[oods]] * (N_INTERACTION_COLUMNS - 4) + [[prev_pt, oods]] * 4
    columns = [[], trace_ext, inter_ext, comp_evals]
    sample_points = [[], [[oods]] * N_COLUMNS, inter_points, [[oods]] * 8]
    sampled = pr.sample_values(ops, columns, sample_points, lifting)
    channel.mix_felts([v for tree in sampled for col in tree for v in col])

    quotient_coeff = channel.draw_secure_felt()
    quotients = pr.compute_fri_quotients(ops, columns, sample_points, sampled, quotient_coeff, lifting, b, twiddles)
    fri = pr.fri_commit(ops, channel, fp, quotients, lifting, twiddles)

    fri_pow = ops.grind(channel.digest, fp.pow_bits)
    channel.mix_u64(fri_pow)
    queries = sorted(set(channel.draw_queries(lifting, fp.n_queries)))
    reads = pr.Reads()
    first = pr.FriLayerDecommit(reads, quotients, fri["first"]["tree"], queries, fp.fold_step, ops)
    inner = []
    layer_queries = pr.fold_queries(queries, fp.fold_step)
    for layer in fri["inner"]:
        inner.append(pr.FriLayerDecommit(reads, layer["eval"], layer["tree"], layer_queries, layer["fold_step"], ops))
        layer_queries = pr.fold_queries(layer_queries, layer["fold_step"])
    trees = [pr.MerkleDecommit(reads, tree, queries, cols, ops)
             for tree, cols in ((trace_tree, trace_ext), (inter_tree, inter_ext), (comp_tree, comp_evals))]
    reads.run(ops)

    proof = pr.StarkProof(config=config)
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

    # --- sanity check (mod.rs:121-132)
    comp = sampled[3]
    left_v = pr.from_partial_evals([comp[k][0] for k in range(4)])
    right_v = pr.from_partial_evals([comp[k][0] for k in range(4, 8)])
    x = oods[0]
    for _ in range(mldb - 1):
        x = pr.q_double_x(x)
    composition_oods = qm_add(left_v, qm_mul(x, right_v))
    expected = composition_at_point(oods, [c[0] for c in sampled[1]], sampled[2], lookup, claimed, random_coeff,
                                    mldb, n)
    proof.constraints_satisfied = composition_oods == expected
    if check and not proof.constraints_satisfied:
        raise ConstraintsNotSatisfied("Constraints not satisfied.")
    return proof


__all__ = ["prove_poseidon", "poseidon_pcs_config", "composition_at_point", "ConstraintsNotSatisfied",
           "N_COLUMNS", "N_INTERACTION_COLUMNS", "N_CONSTRAINTS"]
