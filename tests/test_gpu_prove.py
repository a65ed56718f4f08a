"""Whole Wide-Fibonacci proofs of the restated host prover (proving_gb300.prover) on the CUDA
backend against the oracle's own prover (oracle/oracle_prover.c: prove_ex, the commitment scheme,
FRI and the felt stream restated in C from the reference, sharing no code with the product):
byte-identical proofs, and the restated verifier accepts them. Sizes include the benchmark's shape
(100 columns, 2^14 rows, log blowup 1, 70 queries, pow 10)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import oracle as O  # noqa: E402
from oracle.verifier import parse_proof, verify_fib_and_lookups, verify_wide_fib_components  # noqa: E402
from proving_gb300 import prover as pr  # noqa: E402
from proving_gb300.synthetic import m31_column  # noqa: E402

N_COLS = 100
FRI = (10, 1, 0, 70, 1)


@pytest.fixture(scope="module")
def gpu():
    from proving_gb300 import build
    build.build()
    return pr.GpuOps()


def _config(lifting, n_queries=70):
    fp = pr.FriParams(pow_bits=10, log_blowup_factor=1, log_last_layer_degree_bound=0, n_queries=n_queries,
                      fold_step=1)
    return pr.PcsConfig(fp, trace_lifting_log_size=lifting)


def _prove(ops, trace_host, log_n):
    ch = pr.Blake2sChannel()
    proof = pr.prove_wide_fib(ops, ops.columns_from_host(trace_host), log_n, _config(log_n + 1), ch,
                              ops.twiddles(log_n + 2))
    return proof, ch


@pytest.mark.parametrize("log_n", [4, 7, 10, 14])
def test_gpu_proof_bytes_equal_oracle_prover(gpu, log_n):
    trace = O.wide_fib_trace(m31_column(11, log_n), m31_column(12, log_n), N_COLS)
    g, _ = _prove(gpu, trace, log_n)
    want, _ = O.prove_fib_and_lookups(FRI, [trace], [log_n])
    assert g.to_bytes() == want
    verify_wide_fib_components(parse_proof(want, log_n + 1), [N_COLS], [log_n])


def test_device_trace_generation_proof(gpu):
    # trace generated on the device (cs_wide_fib_trace) proves the same statement
    log_n = 10
    a, b = m31_column(21, log_n), m31_column(22, log_n)
    from proving_gb300.backend import BaseColumn, CudaBackend
    dev_trace = CudaBackend.wide_fib_trace(BaseColumn.from_cpu(a), BaseColumn.from_cpu(b), N_COLS)
    proof = pr.prove_wide_fib(gpu, dev_trace, log_n, _config(log_n + 1), pr.Blake2sChannel(),
                              gpu.twiddles(log_n + 2))
    want, _ = O.prove_fib_and_lookups(FRI, [O.wide_fib_trace(a, b, N_COLS)], [log_n])
    assert proof.to_bytes() == want


def test_lifted_components_match_oracle_prover(gpu):
    # two Wide-Fibonacci components of 2^9 and 2^3 rows in one lifted tree (test_e2e_lifted_fib_prove,
    # crates/examples/src/wide_fibonacci/mod.rs:495-577)
    from test_prove_cpu import lifted_components_inputs, lifted_components_proof
    traces, logs, fri = lifted_components_inputs()
    want, _ = O.prove_fib_and_lookups(fri, traces, logs)
    assert lifted_components_proof(gpu).to_bytes() == want
    verify_wide_fib_components(parse_proof(want, max(logs) + 1), [len(t) for t in traces], logs)


def test_fib_and_lookups_match_oracle_prover(gpu):
    # Wide-Fibonacci and LogUp components of four sizes in one proof: the same bytes and claimed
    # sums, and the restated verifier accepts
    from test_prove_cpu import fib_and_lookups_inputs, fib_and_lookups_proof
    traces, logs, values, lookup_logs, fri = fib_and_lookups_inputs()
    want, claimed = O.prove_fib_and_lookups(fri, traces, logs, values, lookup_logs)
    g = fib_and_lookups_proof(gpu)
    assert g.claimed_sums == claimed
    assert g.to_bytes() == want
    verify_fib_and_lookups(parse_proof(want, max(logs + lookup_logs) + 1), [len(t) for t in traces], logs,
                           lookup_logs, claimed)


@pytest.mark.parametrize("fold_step,last_layer", [(2, 0), (3, 1), (4, 2)])
def test_fold_steps_match_oracle_prover(gpu, fold_step, last_layer):
    # FRI with several folds per layer (packed leaves) and last layers of higher degree on the
    # device: the oracle prover's bytes
    from test_prove_cpu import fib_and_lookups_inputs
    traces, logs, values, lookup_logs, _ = fib_and_lookups_inputs()
    want, _ = O.prove_fib_and_lookups((10, 1, last_layer, 3, fold_step), traces, logs, values, lookup_logs)
    fp = pr.FriParams(pow_bits=10, log_blowup_factor=1, log_last_layer_degree_bound=last_layer, n_queries=3,
                      fold_step=fold_step)
    cfg = pr.PcsConfig(fp, trace_lifting_log_size=10)
    got = pr.prove_fib_and_lookups(gpu, [gpu.columns_from_host(t) for t in traces], logs,
                                   [gpu.columns_from_host([v])[0] for v in values], lookup_logs, cfg,
                                   pr.Blake2sChannel(), gpu.twiddles(10))
    assert got.to_bytes() == want


def test_mixed_shape_proof_matches_oracle_prover(gpu):
    # the batched mixed-size trace at a reduced scale (60 base columns, 12 LogUp components, log sizes
    # 4..11): Wide-Fibonacci components per size plus LogUp components
    from proving_gb300.synthetic import mixed_trace_shape
    comps, lookup_logs = mixed_trace_shape(seed=3, n_base=60, n_interaction=12, lo=4, hi=11, mean=7.0)
    max_log = max([l for _, l in comps] + lookup_logs)
    host = [O.wide_fib_trace(m31_column(10 + i, l), m31_column(50 + i, l), n) for i, (n, l) in enumerate(comps)]
    vals = [m31_column(90 + k, l) for k, l in enumerate(lookup_logs)]
    g = pr.prove_fib_and_lookups(gpu, [gpu.columns_from_host(t) for t in host], [l for _, l in comps],
                                 [gpu.columns_from_host([v])[0] for v in vals], lookup_logs, _config(max_log + 1),
                                 pr.Blake2sChannel(), gpu.twiddles(max_log + 2))
    want, claimed = O.prove_fib_and_lookups(FRI, host, [l for _, l in comps], vals, lookup_logs)
    assert g.to_bytes() == want
    assert g.claimed_sums == claimed
    verify_fib_and_lookups(parse_proof(want, max_log + 1), [n for n, _ in comps], [l for _, l in comps],
                           lookup_logs, claimed)


def test_fri_graph_replay_matches_oracle_prover():
    # the second and third proofs of one size replay the captured FRI layer loop: each equals the
    # oracle's proof of its own trace
    from proving_gb300 import build
    build.build()
    ops = pr.GpuOps()
    log_n = 8
    tw = ops.twiddles(log_n + 2)
    seen = set()
    for seed in (31, 33, 35):
        trace = O.wide_fib_trace(m31_column(seed, log_n), m31_column(seed + 1, log_n), N_COLS)
        g = pr.prove_wide_fib(ops, ops.columns_from_host(trace), log_n, _config(log_n + 1), pr.Blake2sChannel(), tw)
        want, _ = O.prove_fib_and_lookups(FRI, [trace], [log_n])
        assert g.to_bytes() == want
        seen.add(g.to_bytes())
    assert len(seen) == 3 and len(ops._fri_graphs) == 1


def test_tampered_trace_is_not_proved_by_the_oracle():
    # a trace that breaks one constraint: the oracle's prover reports ConstraintsNotSatisfied (its
    # sanity check, crates/stwo/src/prover/mod.rs:121-132) or a last layer of too high degree
    trace = O.wide_fib_trace(m31_column(5, 6), m31_column(6, 6), 10)
    trace[4] = trace[4].copy()
    trace[4][9] = (int(trace[4][9]) + 1) % O.P
    with pytest.raises(O.ProofError):
        O.prove_fib_and_lookups((10, 1, 0, 20, 1), [trace], [6])
    assert np.any(trace[4] != O.wide_fib_trace(m31_column(5, 6), m31_column(6, 6), 10)[4])
