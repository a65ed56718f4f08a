"""ORACLE — test infrastructure only: the reference's GKR batch verifier and
sum-check verifier restated, to accept or reject proofs made by
proving_gb300.gkr.prove_batch.

Follows partially_verify_batch and Gate
(crates/stwo/src/prover/lookups/gkr_verifier.rs:17-230) and
sumcheck::partially_verify (crates/stwo/src/prover/lookups/sumcheck.rs:150-183).
The channel is the C oracle's; the field helpers are the oracle verifier's,
written independently of the prover. Raises GkrError on the first failed check.
"""
from __future__ import annotations

from . import oracle as O
from .verifier import P, qadd, qm, qmul, qsub

MAX_DEGREE = 3
LOGUP, GRAND_PRODUCT = "logup", "grand_product"


class GkrError(Exception):
    pass


def _t(x):
    return tuple(int(v) % P for v in x)


def _horner(coeffs, x):
    acc = qm(0)
    for c in reversed(coeffs):
        acc = qadd(qmul(acc, x), c)
    return acc


def _degree(coeffs):
    n = len(coeffs)
    while n and all(v == 0 for v in coeffs[n - 1]):
        n -= 1
    return max(n - 1, 0)


def _eq(x, y):
    r = qm(1)
    for xi, yi in zip(x, y):
        r = qmul(r, qadd(qmul(xi, yi), qmul(qsub(qm(1), xi), qsub(qm(1), yi))))
    return r


def _mix(channel, felts):
    if felts:
        channel.mix_felts([list(f) for f in felts])
    else:
        channel.mix_u32s([])


def sumcheck_partially_verify(claim, round_polys, channel):
    """Returns (assignment, claimed evaluation) or raises GkrError."""
    assignment = []
    for rnd, poly in enumerate(round_polys):
        if _degree(poly) > MAX_DEGREE:
            raise GkrError(f"sum-check degree too high in round {rnd}")
        s = qadd(_horner(poly, qm(0)), _horner(poly, qm(1)))
        if s != claim:
            raise GkrError(f"sum-check sum does not match the claim in round {rnd}")
        _mix(channel, poly)
        challenge = _t(channel.draw_secure_felt())
        claim = _horner(poly, challenge)
        assignment.append(challenge)
    return assignment, claim


def gate_eval(gate, mask):
    """Gate::eval (gkr_verifier.rs)."""
    if gate == LOGUP:
        if len(mask) != 2:
            raise GkrError("invalid mask")
        (na, nb), (da, db) = mask
        return [qadd(qmul(db, na), qmul(da, nb)), qmul(da, db)]
    if len(mask) != 1:
        raise GkrError("invalid mask")
    a, b = mask[0]
    return [qmul(a, b)]


def partially_verify_batch(gates, proof, channel: O.Blake2sChannel):
    """Returns (ood_point, claims_to_verify_by_instance, n_variables_by_instance)."""
    sumcheck_proofs = proof.sumcheck_proofs
    masks_by_instance = [[m.columns for m in ms] for ms in proof.layer_masks_by_instance]
    outputs = proof.output_claims_by_instance
    if len(masks_by_instance) != len(outputs):
        raise GkrError("malformed proof")
    n_instances = len(masks_by_instance)
    n_layers = max(len(m) for m in masks_by_instance)
    if n_layers != len(sumcheck_proofs):
        raise GkrError("malformed proof")
    if len(gates) != n_instances:
        raise GkrError("number of instances mismatch")
    ood_point = []
    claims_to_verify = [None] * n_instances
    for layer, round_polys in enumerate(sumcheck_proofs):
        remaining = n_layers - layer
        for inst in range(n_instances):
            if len(masks_by_instance[inst]) == remaining:
                claims_to_verify[inst] = [_t(c) for c in outputs[inst]]
        for claims in claims_to_verify:
            if claims is not None:
                _mix(channel, claims)
        sumcheck_alpha = _t(channel.draw_secure_felt())
        instance_lambda = _t(channel.draw_secure_felt())
        sc_claims, sc_instances = [], []
        for inst, claims in enumerate(claims_to_verify):
            if claims is not None:
                n_unused = n_layers - len(masks_by_instance[inst])
                sc_claims.append(qmul(_horner(claims, instance_lambda), qm(1 << n_unused)))
                sc_instances.append(inst)
        sc_claim = _horner(sc_claims, sumcheck_alpha)
        sc_ood, sc_eval = sumcheck_partially_verify(sc_claim, round_polys, channel)
        layer_evals = []
        for inst in sc_instances:
            n_unused = n_layers - len(masks_by_instance[inst])
            mask = masks_by_instance[inst][layer - n_unused]
            out = gate_eval(gates[inst], mask)
            e = _eq(ood_point[n_unused:], sc_ood[n_unused:])
            layer_evals.append(qmul(e, _horner(out, instance_lambda)))
        if sc_eval != _horner(layer_evals, sumcheck_alpha):
            raise GkrError(f"circuit check failed in layer {layer}")
        for inst in sc_instances:
            n_unused = n_layers - len(masks_by_instance[inst])
            mask = masks_by_instance[inst][layer - n_unused]
            _mix(channel, [v for col in mask for v in col])
        challenge = _t(channel.draw_secure_felt())
        ood_point = list(sc_ood) + [challenge]
        for inst in sc_instances:
            n_unused = n_layers - len(masks_by_instance[inst])
            mask = masks_by_instance[inst][layer - n_unused]
            claims_to_verify[inst] = [qadd(qmul(challenge, qsub(v1, v0)), v0) for v0, v1 in mask]
    return ood_point, claims_to_verify, [len(m) for m in masks_by_instance]

