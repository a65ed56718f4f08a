"""GKR batch prover (proving_gb300.gkr) over the CPU oracle's GkrOps, checked by
the restated verifier: the reference's tests of
crates/stwo/src/prover/lookups/{utils.rs, gkr_verifier.rs, backend/cpu/lookups/gkr.rs}
with the same assertions (output claims are the product / fraction sum; the
claims left to verify are the input columns' MLEs at the OOD point)."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import oracle as O
from gkr_cpu_backend import CpuGkrOps, mle_eval_at_point
from oracle.gkr_verifier import GRAND_PRODUCT, LOGUP, GkrError, partially_verify_batch
from proving_gb300 import gkr as G
from proving_gb300 import prover as pr

P = pr.P


def draw_felts(ch, n):
    return [ch.draw_secure_felt() for _ in range(n)]


def seeded_felts(seed, n):
    rng = np.random.default_rng(seed)
    return [tuple(int(v) for v in r) for r in rng.integers(0, P, size=(n, 4))]


def product(values):
    r = pr.qm(1)
    for v in values:
        r = pr.qm_mul(r, v)
    return r


def fraction_sum(nums, dens):
    n, d = pr.qm(0), pr.qm(1)
    for a, b in zip(nums, dens):  # Fraction<N, D>: n/d + a/b = (b n + d a) / (d b)
        n, d = pr.qm_add(pr.qm_mul(b, n), pr.qm_mul(d, a)), pr.qm_mul(d, b)
    return n, d


def prove_and_verify(layers, gates):
    ops = CpuGkrOps()
    proof, artifact = G.prove_batch(ops, pr.Blake2sChannel(), layers)
    ood, claims, n_vars = partially_verify_batch(gates, proof, O.Blake2sChannel())
    assert ood == artifact.ood_point
    assert claims == artifact.claims_to_verify_by_instance
    assert n_vars == artifact.n_variables_by_instance
    return proof, ood, claims, n_vars


def test_gen_eq_evals():
    ops = CpuGkrOps()
    zero, one, two = pr.qm(0), pr.qm(1), pr.qm(2)
    y = [pr.qm(7), pr.qm(3)]
    got = ops.values(ops.gen_eq_evals(y, two), 4)
    want = [pr.qm_mul(G.eq(x, y), two) for x in ([zero, zero], [zero, one], [one, zero], [one, one])]
    assert got == want


def test_lagrange_interpolation_and_horner():
    xs = [pr.qm(v) for v in (5, 1, 3, 9)]
    ys = [pr.qm(v) for v in (1, 2, 3, 4)]
    poly = G.interpolate_lagrange(xs, ys)
    for x, y in zip(xs, ys):
        assert G.poly_eval(poly, x) == y
    coeffs = [pr.qm(9), pr.qm(2), pr.qm(3)]
    assert G.poly_eval(coeffs, pr.qm(7)) == pr.qm(9 + 2 * 7 + 3 * 49)


def test_eq_on_hypercube_points():
    zero, one = pr.qm(0), pr.qm(1)
    a = [one, zero, one]
    assert G.eq(a, a) == one
    assert G.eq(a, [one, zero, zero]) == zero
    with pytest.raises(AssertionError):
        G.eq([zero, one], [zero])


def test_polynomial_trimming_matches_reference_semantics():
    # UnivariatePoly::new trims; a linear combination keeps the longest length
    assert G.poly_new([pr.qm(1), pr.qm(0)]) == [pr.qm(1)]
    assert G.poly_new([pr.qm(0)]) == []
    comb = G.poly_linear_combination([[pr.qm(1), pr.qm(1)], [pr.qm(0), pr.qm(P - 1)]], pr.qm(1))
    assert comb == [pr.qm(1), pr.qm(0)]


def test_grand_product_works():
    values = draw_felts(pr.Blake2sChannel(), 1 << 5)
    ops = CpuGkrOps()
    proof, r, claims, _ = prove_and_verify([G.Layer(G.GRAND_PRODUCT, [ops.mle_from_host(values)])], [GRAND_PRODUCT])
    assert proof.output_claims_by_instance == [[product(values)]]
    assert claims == [[mle_eval_at_point(values, r)]]


def test_logup_with_generic_trace_works():
    nums, dens = seeded_felts(1, 32), seeded_felts(2, 32)
    ops = CpuGkrOps()
    layer = G.Layer(G.LOGUP_GENERIC, [ops.mle_from_host(nums), ops.mle_from_host(dens)])
    proof, r, claims, _ = prove_and_verify([layer], [LOGUP])
    assert proof.output_claims_by_instance == [list(fraction_sum(nums, dens))]
    assert claims == [[mle_eval_at_point(nums, r), mle_eval_at_point(dens, r)]]


def test_logup_with_singles_trace_works():
    dens = seeded_felts(3, 32)
    ops = CpuGkrOps()
    proof, r, claims, _ = prove_and_verify([G.Layer(G.LOGUP_SINGLES, [ops.mle_from_host(dens)])], [LOGUP])
    assert proof.output_claims_by_instance == [list(fraction_sum([pr.qm(1)] * 32, dens))]
    assert claims == [[pr.qm(1), mle_eval_at_point(dens, r)]]


def test_logup_with_multiplicities_trace_works():
    rng = np.random.default_rng(4)
    nums = [int(v) for v in rng.integers(0, P, 32)]
    dens = seeded_felts(5, 32)
    ops = CpuGkrOps()
    layer = G.Layer(G.LOGUP_MULTIPLICITIES, [ops.mle_from_host(nums, base=True), ops.mle_from_host(dens)])
    proof, r, claims, _ = prove_and_verify([layer], [LOGUP])
    assert proof.output_claims_by_instance == [list(fraction_sum([pr.qm(v) for v in nums], dens))]
    assert claims == [[mle_eval_at_point(np.asarray(nums), r), mle_eval_at_point(dens, r)]]


@pytest.mark.parametrize("logs", [(5, 5), (5, 7)])
def test_prove_batch_works(logs):
    ch = pr.Blake2sChannel()
    cols = [draw_felts(ch, 1 << n) for n in logs]
    ops = CpuGkrOps()
    layers = [G.Layer(G.GRAND_PRODUCT, [ops.mle_from_host(c)]) for c in cols]
    proof, r, claims, n_vars = prove_and_verify(layers, [GRAND_PRODUCT] * 2)
    assert n_vars == list(logs)
    assert proof.output_claims_by_instance == [[product(c)] for c in cols]
    for c, n, cl in zip(cols, logs, claims):
        assert cl == [mle_eval_at_point(c, r[len(r) - n:])]


def test_mixed_kinds_batch():
    ops = CpuGkrOps()
    gp = seeded_felts(6, 1 << 6)
    nums, dens = seeded_felts(7, 1 << 4), seeded_felts(8, 1 << 4)
    sdens = seeded_felts(9, 1 << 5)
    layers = [G.Layer(G.GRAND_PRODUCT, [ops.mle_from_host(gp)]),
              G.Layer(G.LOGUP_GENERIC, [ops.mle_from_host(nums), ops.mle_from_host(dens)]),
              G.Layer(G.LOGUP_SINGLES, [ops.mle_from_host(sdens)])]
    proof, r, claims, n_vars = prove_and_verify(layers, [GRAND_PRODUCT, LOGUP, LOGUP])
    assert n_vars == [6, 4, 5]
    assert claims[1] == [mle_eval_at_point(nums, r[-4:]), mle_eval_at_point(dens, r[-4:])]


def test_tampered_proof_is_rejected():
    values = seeded_felts(10, 1 << 4)
    ops = CpuGkrOps()
    proof, _ = G.prove_batch(ops, pr.Blake2sChannel(), [G.Layer(G.GRAND_PRODUCT, [ops.mle_from_host(values)])])
    poly = proof.sumcheck_proofs[2][0]
    poly[0] = pr.qm_add(poly[0], pr.qm(1))
    with pytest.raises(GkrError):
        partially_verify_batch([GRAND_PRODUCT], proof, O.Blake2sChannel())
    proof2, _ = G.prove_batch(ops, pr.Blake2sChannel(), [G.Layer(G.GRAND_PRODUCT, [ops.mle_from_host(values)])])
    proof2.output_claims_by_instance[0][0] = pr.qm_add(proof2.output_claims_by_instance[0][0], pr.qm(1))
    with pytest.raises(GkrError):
        partially_verify_batch([GRAND_PRODUCT], proof2, O.Blake2sChannel())


def test_round_constants_match_lagrange_correction():
    """The precomputed form of correct_sum_as_poly_in_first_variable gives the coefficients of
    the reference's interpolate_lagrange form for every k."""
    rng = np.random.default_rng(12)
    for n in (1, 2, 5, 9):
        y = [tuple(int(v) for v in r) for r in rng.integers(0, P, size=(n, 4))]
        consts = G.RoundConstants(y)
        for k in range(1, n + 1):
            f0, f2, claim = [tuple(int(v) for v in r) for r in rng.integers(0, P, size=(3, 4))]
            assert consts.correct_sum(f0, f2, claim, k) == G.correct_sum_as_poly_in_first_variable(f0, f2, claim, y, k)
