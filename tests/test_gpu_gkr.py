"""GKR lookups on the device (cs_gkr_*, cs_mle_fix_first_variable) against the
CPU oracle's GkrOps: every operation bit-exact at small and large sizes, whole
batch proofs equal value for value and accepted by the restated verifier."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import oracle as O
from gkr_cpu_backend import CpuGkrOps, mle_eval_at_point
from oracle.gkr_verifier import GRAND_PRODUCT, LOGUP, partially_verify_batch
from proving_gb300 import gkr as G
from proving_gb300 import prover as pr

pytestmark = pytest.mark.gpu
P = pr.P


@pytest.fixture(scope="module")
def dev():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from proving_gb300 import _lib
    _lib.load()
    return G.DeviceGkrOps()


def felts(seed, n):
    return np.random.default_rng(seed).integers(0, P, size=(n, 4), dtype=np.int64)


def base(seed, n):
    return np.random.default_rng(seed).integers(0, P, size=n, dtype=np.int64)


def as_tuples(a):
    return [tuple(int(x) for x in r) for r in np.asarray(a)]


def dev_values(dev, mle):
    return dev.values(mle, 1 << mle.n_variables)


@pytest.mark.parametrize("n", [0, 1, 2, 5, 10, 11, 14, 15, 18])
def test_gen_eq_evals_matches_oracle(dev, n):
    y, v = as_tuples(felts(n, n)), as_tuples(felts(100 + n, 1))[0]
    cpu = CpuGkrOps()
    assert dev_values(dev, dev.gen_eq_evals(y, v)) == cpu.values(cpu.gen_eq_evals(y, v), 1 << n)


@pytest.mark.parametrize("log_n", [1, 2, 5, 17])
@pytest.mark.parametrize("is_base", [False, True])
def test_fix_first_variable_matches_oracle(dev, log_n, is_base):
    vals = base(log_n, 1 << log_n) if is_base else felts(log_n, 1 << log_n)
    x = as_tuples(felts(7, 1))[0]
    cpu = CpuGkrOps()
    want = cpu.fix_first_variable(cpu.mle_from_host(vals, is_base), x)
    got = dev.fix_first_variable(dev.mle_from_host(vals, is_base), x)
    assert dev_values(dev, got) == cpu.values(want, 1 << (log_n - 1))


def make_layer(ops, kind, log_n, seed):
    d = ops.mle_from_host(felts(seed, 1 << log_n))
    if kind == G.GRAND_PRODUCT:
        return G.Layer(kind, [d])
    if kind == G.LOGUP_SINGLES:
        return G.Layer(kind, [d])
    if kind == G.LOGUP_MULTIPLICITIES:
        return G.Layer(kind, [ops.mle_from_host(base(seed + 1, 1 << log_n), True), d])
    return G.Layer(kind, [ops.mle_from_host(felts(seed + 1, 1 << log_n)), d])


KINDS = [G.GRAND_PRODUCT, G.LOGUP_GENERIC, G.LOGUP_MULTIPLICITIES, G.LOGUP_SINGLES]


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("log_n", [1, 2, 7, 18])
def test_next_layer_matches_oracle(dev, kind, log_n):
    cpu = CpuGkrOps()
    want = cpu.next_layer(make_layer(cpu, kind, log_n, 11))
    got = dev.next_layer(make_layer(dev, kind, log_n, 11))
    assert got.kind == want.kind
    for g, w in zip(got.mles, want.mles):
        assert dev_values(dev, g) == cpu.values(w, 1 << (log_n - 1))


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("log_n", [2, 3, 9, 19])
def test_sum_as_poly_matches_oracle(dev, kind, log_n):
    cpu = CpuGkrOps()
    lam = as_tuples(felts(5, 1))[0]
    eq_vals = felts(6, 1 << (log_n - 1))  # longer than the 2^(log_n - 2) terms used
    items_cpu = [(make_layer(cpu, kind, log_n, 21), cpu.mle_from_host(eq_vals), lam)]
    items_dev = [(make_layer(dev, kind, log_n, 21), dev.mle_from_host(eq_vals), lam)]
    assert dev.sum_as_poly_evals(items_dev) == cpu.sum_as_poly_evals(items_cpu)


def batch(ops, spec):
    layers, gates = [], []
    for i, (kind, log_n) in enumerate(spec):
        layers.append(make_layer(ops, kind, log_n, 31 + 7 * i))
        gates.append(GRAND_PRODUCT if kind == G.GRAND_PRODUCT else LOGUP)
    return layers, gates


def proof_words(proof):
    return (proof.sumcheck_proofs, [[m.columns for m in ms] for ms in proof.layer_masks_by_instance],
            proof.output_claims_by_instance)


@pytest.mark.parametrize("spec", [
    [(G.GRAND_PRODUCT, 6)],
    [(G.GRAND_PRODUCT, 10), (G.LOGUP_GENERIC, 8), (G.LOGUP_SINGLES, 6), (G.LOGUP_MULTIPLICITIES, 9)],
    [(G.LOGUP_MULTIPLICITIES, 2), (G.LOGUP_GENERIC, 12)],
])
def test_prove_batch_matches_oracle_and_verifies(dev, spec):
    cpu = CpuGkrOps()
    lc, gates = batch(cpu, spec)
    ld, _ = batch(dev, spec)
    pc, ac = G.prove_batch(cpu, pr.Blake2sChannel(), lc)
    pd, ad = G.prove_batch(dev, pr.Blake2sChannel(), ld)
    assert proof_words(pd) == proof_words(pc)
    assert ad.ood_point == ac.ood_point and ad.claims_to_verify_by_instance == ac.claims_to_verify_by_instance
    ood, claims, n_vars = partially_verify_batch(gates, pd, O.Blake2sChannel())
    assert n_vars == [n for _, n in spec] and claims == ad.claims_to_verify_by_instance


def test_large_logup_batch_verifies(dev):
    """2^20-value LogUp (generic) and 2^18 grand product: the verifier accepts, the outputs are
    the fraction sum / product and the final claims are the inputs' MLEs at the OOD point."""
    nums, dens, gp = felts(41, 1 << 20), felts(42, 1 << 20), felts(43, 1 << 18)
    layers = [G.Layer(G.LOGUP_GENERIC, [dev.mle_from_host(nums), dev.mle_from_host(dens)]),
              G.Layer(G.GRAND_PRODUCT, [dev.mle_from_host(gp)])]
    proof, art = G.prove_batch(dev, pr.Blake2sChannel(), layers)
    ood, claims, _ = partially_verify_batch([LOGUP, GRAND_PRODUCT], proof, O.Blake2sChannel())
    assert claims == art.claims_to_verify_by_instance
    assert claims[0] == [mle_eval_at_point(nums, ood), mle_eval_at_point(dens, ood)]
    assert claims[1] == [mle_eval_at_point(gp, ood[2:])]
    # the output layer of a binary tree of products / fraction sums (any order gives the same values)
    cpu = CpuGkrOps()
    lay = G.Layer(G.GRAND_PRODUCT, [cpu.mle_from_host(gp)])
    while lay.n_variables:
        lay = cpu.next_layer(lay)
    assert proof.output_claims_by_instance[1] == cpu.values(lay.mles[0], 1)


@pytest.mark.parametrize("spec", [
    [(G.GRAND_PRODUCT, 1)],
    [(G.GRAND_PRODUCT, 7)],
    [(G.GRAND_PRODUCT, 10), (G.LOGUP_GENERIC, 8), (G.LOGUP_SINGLES, 6), (G.LOGUP_MULTIPLICITIES, 9)],
    [(G.LOGUP_MULTIPLICITIES, 2), (G.LOGUP_GENERIC, 12)],
    [(G.LOGUP_SINGLES, 14), (G.LOGUP_SINGLES, 14)],
])
def test_native_prove_batch_equals_driver(dev, spec):
    """cs_gkr_prove_batch (the protocol in native code) gives the Python driver's proof, artifact
    and final channel state; the verifier accepts it."""
    layers, gates = batch(dev, spec)
    ch_py, ch_nat = pr.Blake2sChannel(), pr.Blake2sChannel()
    ch_py.mix_u32s([7, 8, 9])
    ch_nat.mix_u32s([7, 8, 9])
    p_py, a_py = G.prove_batch(dev, ch_py, layers)
    p_nat, a_nat = G.prove_batch_native(ch_nat, layers)
    assert proof_words(p_nat) == proof_words(p_py)
    assert (a_nat.ood_point, a_nat.claims_to_verify_by_instance, a_nat.n_variables_by_instance) == \
        (a_py.ood_point, a_py.claims_to_verify_by_instance, a_py.n_variables_by_instance)
    assert (ch_nat.digest, ch_nat.n_draws) == (ch_py.digest, ch_py.n_draws)
    vch = O.Blake2sChannel(ch_py_start_digest(spec))
    ood, claims, _ = partially_verify_batch(gates, p_nat, vch)
    assert ood == a_nat.ood_point and claims == a_nat.claims_to_verify_by_instance


def ch_py_start_digest(spec):
    ch = pr.Blake2sChannel()
    ch.mix_u32s([7, 8, 9])
    return ch.digest


def test_native_prove_batch_large_logup(dev):
    """2^20-fraction LogUp through the native driver: verifies and ends at the inputs' MLEs."""
    nums, dens = felts(51, 1 << 20), felts(52, 1 << 20)
    layers = [G.Layer(G.LOGUP_GENERIC, [dev.mle_from_host(nums), dev.mle_from_host(dens)])]
    proof, art = G.prove_batch_native(pr.Blake2sChannel(), layers)
    ood, claims, _ = partially_verify_batch([LOGUP], proof, O.Blake2sChannel())
    assert claims == [[mle_eval_at_point(nums, ood), mle_eval_at_point(dens, ood)]] == art.claims_to_verify_by_instance
