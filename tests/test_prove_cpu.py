"""Whole-proof host logic on the CPU: the restated prover driven by the oracle
backend produces Wide-Fibonacci proofs that the restated verifier accepts
(crates/examples/src/wide_fibonacci/mod.rs:182-241) and rejects when tampered
with (a bad OODS nonce, :245-309; a changed queried value; a changed FRI value)."""
import copy

import pytest

from oracle import oracle as O
from cpu_backend import CpuOps
from oracle.verifier import VerificationError, verify_wide_fib
from proving_gb300 import prover as pr
from proving_gb300.synthetic import m31_column

N_COLS = 100


def make_proof(log_n, n_queries=70):
    ops = CpuOps()
    trace = O.wide_fib_trace(m31_column(1, log_n), m31_column(2, log_n), N_COLS)
    fp = pr.FriParams(pow_bits=10, log_blowup_factor=1, log_last_layer_degree_bound=0, n_queries=n_queries,
                      fold_step=1)
    cfg = pr.PcsConfig(fp, trace_lifting_log_size=log_n + 1)
    return pr.prove_wide_fib(ops, ops.columns_from_host(trace), log_n, cfg, pr.Blake2sChannel(),
                             ops.twiddles(log_n + 2))


@pytest.mark.parametrize("log_n", [4, 5, 8])
def test_prove_then_verify(log_n):
    verify_wide_fib(make_proof(log_n), N_COLS, log_n)


def test_tampering_is_rejected():
    proof = make_proof(5)
    bad = copy.deepcopy(proof)
    bad.oods_proof_of_work += 1
    with pytest.raises(VerificationError):
        verify_wide_fib(bad, N_COLS, 5)
    bad = copy.deepcopy(proof)
    bad.queried_values[1][7][3] = (bad.queried_values[1][7][3] + 1) % O.P
    with pytest.raises(VerificationError):
        verify_wide_fib(bad, N_COLS, 5)
    bad = copy.deepcopy(proof)
    w = list(bad.fri_first_layer["fri_witness"][0])
    w[0] = (w[0] + 1) % O.P
    bad.fri_first_layer["fri_witness"][0] = tuple(w)
    with pytest.raises(VerificationError):
        verify_wide_fib(bad, N_COLS, 5)


def test_invalid_trace_is_refused():
    # a trace that violates a constraint fails the prover's own OODS check
    ops = CpuOps()
    log_n = 4
    trace = O.wide_fib_trace(m31_column(1, log_n), m31_column(2, log_n), N_COLS)
    trace[50][3] = (int(trace[50][3]) + 1) % O.P
    fp = pr.FriParams(n_queries=20)
    cfg = pr.PcsConfig(fp, trace_lifting_log_size=log_n + 1)
    with pytest.raises(RuntimeError, match="constraints not satisfied"):
        pr.prove_wide_fib(ops, ops.columns_from_host(trace), log_n, cfg, pr.Blake2sChannel(), ops.twiddles(log_n + 2))


def test_proof_bytes_are_deterministic():
    assert make_proof(4).to_bytes() == make_proof(4).to_bytes()


def test_felt_stream_follows_cairo_serialize():
    # CairoSerialize for StarkProof (crates/cairo-serialize/src/serialize.rs:99-210): the pcs config
    # is the 5 FRI parameters only, then commitments, the OODS nonce, sampled values,
    # decommitments, queried values and the FRI proof, whose LinePoly ends with log2 of its size
    proof = make_proof(4, n_queries=3)
    w = proof.to_words()
    fp = proof.config.fri_params
    assert w[:5] == [fp.pow_bits, fp.log_blowup_factor, fp.log_last_layer_degree_bound, fp.n_queries, fp.fold_step]
    k = 5
    assert w[k] == 3  # preprocessed, trace and composition roots
    k += 1 + 3 * 8
    assert w[k] == proof.oods_proof_of_work
    k += 1
    assert w[k] == 3 and w[k + 1] == 0 and w[k + 2] == N_COLS  # sampled values: trees, then the trace's columns
    # the stream ends with the last-layer poly (length, coefficients, log length) and the FRI nonce
    poly = proof.fri_last_layer_poly
    tail = [len(poly)] + [c for q in poly for c in q] + [len(poly).bit_length() - 1, proof.fri_proof_of_work]
    assert w[-len(tail):] == tail
    assert len(proof.to_bytes()) == 8 * len(w)


def lifted_components_inputs():
    # test_e2e_lifted_fib_prove (crates/examples/src/wide_fibonacci/mod.rs:495-577): components of
    # 4 columns x 2^9 and 5 columns x 2^3, inputs a = 1, b = row (generate_test_inputs, :130-134),
    # FriParams::test_params() = (pow 10, last layer 0, blowup 1, 3 queries, fold step 1), tree
    # height 9 + 1. Returns (host traces, log sizes, FRI parameters).
    import numpy as np
    traces = []
    for n_cols, log_n in ((4, 9), (5, 3)):
        a = np.ones(1 << log_n, np.uint32)
        b = np.arange(1 << log_n, dtype=np.uint32)
        traces.append(O.wide_fib_trace(a, b, n_cols))
    return traces, [9, 3], (10, 1, 0, 3, 1)


def lifted_components_proof(ops):
    traces, logs, _ = lifted_components_inputs()
    fp = pr.FriParams(pow_bits=10, log_blowup_factor=1, log_last_layer_degree_bound=0, n_queries=3, fold_step=1)
    cfg = pr.PcsConfig(fp, trace_lifting_log_size=9 + 1)
    return pr.prove_wide_fib_components(ops, [ops.columns_from_host(t) for t in traces], logs, cfg,
                                        pr.Blake2sChannel(), ops.twiddles(10))


def test_lifted_components_prove_then_verify():
    from oracle.verifier import verify_wide_fib_components
    proof = lifted_components_proof(CpuOps())
    verify_wide_fib_components(proof, [4, 5], [9, 3])
    # the short component's columns are lifted from 2^4 to the tree height 10
    assert len(proof.sampled_values[1]) == 9
    bad = copy.deepcopy(proof)
    bad.sampled_values[1][6][0] = tuple((v + 1) % O.P for v in bad.sampled_values[1][6][0])
    with pytest.raises(VerificationError):
        verify_wide_fib_components(bad, [4, 5], [9, 3])


def fib_and_lookups_inputs():
    # the mixed-size batched trace in one proof: Wide-Fibonacci components of 4 columns x 2^9 and
    # 5 columns x 2^3, and single-column LogUp components of 2^8 and 2^4 rows (seeded values).
    # Returns (host traces, log sizes, lookup values, lookup log sizes, FRI parameters).
    import numpy as np
    traces, logs, _ = lifted_components_inputs()
    rng = np.random.default_rng(7)
    values = [rng.integers(0, O.P, 1 << n, dtype=np.uint32) for n in (8, 4)]
    return traces, logs, values, [8, 4], (10, 1, 0, 3, 1)


def fib_and_lookups_proof(ops):
    traces, logs, values, lookup_logs, _ = fib_and_lookups_inputs()
    fp = pr.FriParams(pow_bits=10, log_blowup_factor=1, log_last_layer_degree_bound=0, n_queries=3, fold_step=1)
    cfg = pr.PcsConfig(fp, trace_lifting_log_size=9 + 1)
    return pr.prove_fib_and_lookups(ops, [ops.columns_from_host(t) for t in traces], logs,
                                    [ops.columns_from_host([v])[0] for v in values], lookup_logs, cfg,
                                    pr.Blake2sChannel(), ops.twiddles(10))


def test_fib_and_lookups_prove_then_verify():
    from oracle.verifier import verify_fib_and_lookups
    proof = fib_and_lookups_proof(CpuOps())
    claimed = proof.claimed_sums
    verify_fib_and_lookups(proof, [4, 5], [9, 3], [8, 4], claimed)
    assert [len(t) for t in proof.sampled_values] == [0, 11, 8, 8]
    assert all(len(c) == 2 for c in proof.sampled_values[2])
    # a wrong claimed sum (the statement) is rejected
    wrong = [tuple((v + 1) % O.P for v in claimed[0])] + claimed[1:]
    with pytest.raises(VerificationError):
        verify_fib_and_lookups(proof, [4, 5], [9, 3], [8, 4], wrong)
    # a tampered previous-row sample of the short LogUp component is rejected
    bad = copy.deepcopy(proof)
    bad.sampled_values[2][5][0] = tuple((v + 1) % O.P for v in bad.sampled_values[2][5][0])
    with pytest.raises(VerificationError):
        verify_fib_and_lookups(bad, [4, 5], [9, 3], [8, 4], claimed)
