"""The oracle's own prover (oracle/oracle_prover.c): the reference's prove_ex, commitment scheme,
FRI prover, lifted Merkle decommitment and CairoSerialize felt stream restated in C over the
oracle's CPU ops, written from the reference and sharing no code with the product. Checked here,
on the CPU, against the restated verifier (oracle/verifier.py, which reads the raw proof words)
and against the product's restated host prover run over the oracle's ops (tests/cpu_backend.py):
two independent statements of the transcript order that must give the same bytes."""
import numpy as np
import pytest

from cpu_backend import CpuOps
from oracle import oracle as O
from oracle.verifier import VerificationError, parse_proof, verify_fib_and_lookups, verify_wide_fib_components
from proving_gb300 import prover as pr
from proving_gb300.synthetic import m31_column


def _traces(shape, seed):
    return [O.wide_fib_trace(m31_column(seed + 2 * k, l), m31_column(seed + 2 * k + 1, l), n)
            for k, (n, l) in enumerate(shape)]


def _cfg(lifting, n_queries):
    fp = pr.FriParams(pow_bits=10, log_blowup_factor=1, log_last_layer_degree_bound=0, n_queries=n_queries,
                      fold_step=1)
    return pr.PcsConfig(fp, trace_lifting_log_size=lifting)


@pytest.mark.parametrize("shape,n_queries", [([(100, 4)], 70), ([(4, 9), (5, 3)], 3), ([(10, 6), (3, 6), (7, 11)], 20),
                                             ([(3, 2)], 5), ([(6, 2), (3, 1)], 7)])
def test_oracle_prover_equals_host_prover_and_verifies(shape, n_queries):
    traces = _traces(shape, 50)
    logs = [l for _, l in shape]
    L = max(logs) + 1
    words, _ = O.prove_fib_and_lookups((10, 1, 0, n_queries, 1), traces, logs)
    verify_wide_fib_components(parse_proof(words, L), [n for n, _ in shape], logs)
    cpu = CpuOps()
    host = pr.prove_wide_fib_components(cpu, [cpu.columns_from_host(t) for t in traces], logs, _cfg(L, n_queries),
                                        pr.Blake2sChannel(), cpu.twiddles(L + 1))
    assert host.to_bytes() == words


@pytest.mark.parametrize("shape,lookup_logs,n_queries", [([(4, 9), (5, 3)], [8, 4], 3),
                                                         ([(10, 5), (3, 8)], [8, 2, 5, 8], 70),
                                                         ([(3, 4)], [10], 11)])
def test_oracle_prover_with_lookups(shape, lookup_logs, n_queries):
    traces = _traces(shape, 7)
    rng = np.random.default_rng(7)
    values = [rng.integers(0, O.P, 1 << l, dtype=np.uint32) for l in lookup_logs]
    logs = [l for _, l in shape]
    L = max(logs + lookup_logs) + 1
    words, claimed = O.prove_fib_and_lookups((10, 1, 0, n_queries, 1), traces, logs, values, lookup_logs)
    verify_fib_and_lookups(parse_proof(words, L), [n for n, _ in shape], logs, lookup_logs, claimed)
    # the claimed sums are sums of the fractions 1 / (z - v); a wrong one is rejected
    wrong = [tuple((v + 1) % O.P for v in claimed[0])] + claimed[1:]
    with pytest.raises(VerificationError):
        verify_fib_and_lookups(parse_proof(words, L), [n for n, _ in shape], logs, lookup_logs, wrong)
    cpu = CpuOps()
    host = pr.prove_fib_and_lookups(cpu, [cpu.columns_from_host(t) for t in traces], logs,
                                    [cpu.columns_from_host([v])[0] for v in values], lookup_logs,
                                    _cfg(L, n_queries), pr.Blake2sChannel(), cpu.twiddles(L + 1))
    assert host.claimed_sums == claimed
    assert host.to_bytes() == words


def test_config1_shape_proves_and_verifies():
    # 100 columns x 2^14 rows, 70 queries, pow 10 (the benchmark's Wide-Fibonacci statement)
    traces = _traces([(100, 14)], 11)
    words, _ = O.prove_fib_and_lookups((10, 1, 0, 70, 1), traces, [14])
    verify_wide_fib_components(parse_proof(words, 15), [100], [14])


def test_tampered_proof_words_are_rejected():
    traces = _traces([(10, 5), (3, 8)], 7)
    rng = np.random.default_rng(7)
    values = [rng.integers(0, O.P, 1 << l, dtype=np.uint32) for l in (8, 4)]
    words, claimed = O.prove_fib_and_lookups((10, 1, 0, 70, 1), traces, [5, 8], values, [8, 4])
    n = len(words) // 8
    for k in (3, 40, n // 3, n // 2, n - 30, n - 1):
        bad = bytearray(words)
        bad[8 * k] ^= 1
        with pytest.raises(VerificationError):
            verify_fib_and_lookups(parse_proof(bytes(bad), 9), [10, 3], [5, 8], [8, 4], claimed)


def test_unsatisfied_constraints_are_not_proved():
    trace = _traces([(10, 6)], 5)
    trace[0][4] = trace[0][4].copy()
    trace[0][4][9] = (int(trace[0][4][9]) + 1) % O.P
    with pytest.raises(O.ProofError):
        O.prove_fib_and_lookups((10, 1, 0, 20, 1), trace, [6])


@pytest.mark.parametrize("log_n,generic", [(3, False), (5, False), (3, True)])
def test_oracle_poseidon_equals_host_prover(log_n, generic):
    # the Poseidon2 AIR (the words the reference computes before its sanity check); generic: its
    # constraints through the framework's evaluator (poseidon_air, relation entries in pairs)
    from proving_gb300 import poseidon as ps
    cpu = CpuOps()
    fp = pr.FriParams(pow_bits=10, log_blowup_factor=1, log_last_layer_degree_bound=0, n_queries=70, fold_step=1)
    host = ps.prove_poseidon(cpu, log_n, ps.poseidon_pcs_config(log_n + 3, fp), pr.Blake2sChannel(),
                             cpu.twiddles(log_n + 3), check=False, generic=generic)
    assert host.to_bytes() == O.prove_poseidon((10, 1, 0, 70, 1), log_n)


@pytest.mark.parametrize("fold_step,last_layer", [(2, 0), (3, 1)])
def test_oracle_poseidon_fold_steps_equal_host_prover(fold_step, last_layer):
    # the Poseidon2 proof with several folds per FRI layer: the oracle's prover and the host prover
    from proving_gb300 import poseidon as ps
    cpu = CpuOps()
    fp = pr.FriParams(pow_bits=10, log_blowup_factor=1, log_last_layer_degree_bound=last_layer, n_queries=70,
                      fold_step=fold_step)
    host = ps.prove_poseidon(cpu, 4, ps.poseidon_pcs_config(7, fp), pr.Blake2sChannel(), cpu.twiddles(7), check=False)
    assert host.to_bytes() == O.prove_poseidon((10, 1, last_layer, 70, fold_step), 4)


def test_unsupported_arguments_are_refused():
    with pytest.raises(O.ProofError):
        O.prove_fib_and_lookups((10, 2, 0, 5, 1), _traces([(3, 4)], 1), [4])  # log blowup 2
    with pytest.raises(O.ProofError):
        O.prove_fib_and_lookups((10, 1, 0, 5, 0), _traces([(3, 4)], 1), [4])  # fold step 0


@pytest.mark.parametrize("fold_step,last_layer", [(2, 0), (3, 0), (2, 2), (4, 1)])
def test_oracle_prover_fold_steps_equal_the_host_prover(fold_step, last_layer):
    # FRI with several folds per layer and packed leaves, and last layers of higher degree: the
    # oracle's own prover and the host prover on the oracle's operations give the same words, and
    # the restated verifier accepts them
    from test_prove_cpu import fib_and_lookups_inputs
    from oracle.verifier import parse_proof, verify_fib_and_lookups
    traces, logs, values, lookup_logs, _ = fib_and_lookups_inputs()
    fri = (10, 1, last_layer, 3, fold_step)
    want, claimed = O.prove_fib_and_lookups(fri, traces, logs, values, lookup_logs)
    ops = CpuOps()
    fp = pr.FriParams(pow_bits=10, log_blowup_factor=1, log_last_layer_degree_bound=last_layer, n_queries=3,
                      fold_step=fold_step)
    cfg = pr.PcsConfig(fp, trace_lifting_log_size=10)
    got = pr.prove_fib_and_lookups(ops, [ops.columns_from_host(t) for t in traces], logs,
                                   [ops.columns_from_host([v])[0] for v in values], lookup_logs, cfg,
                                   pr.Blake2sChannel(), ops.twiddles(10))
    assert got.to_bytes() == want
    verify_fib_and_lookups(parse_proof(want, 10), [4, 5], logs, lookup_logs, claimed)
