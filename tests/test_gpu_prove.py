"""Whole Wide-Fibonacci proofs with the CUDA backend: the same restated prover
driven by the GPU backend and by the CPU oracle gives byte-identical proofs
(and transcripts), and the restated verifier accepts them. Sizes include the
config-1 shape (100 columns, 2^14 rows, blowup 2, 70 queries, pow 10)."""
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import oracle as O  # noqa: E402
from oracle.cpu_ops import CpuOps  # noqa: E402
from oracle.verifier import verify_wide_fib  # noqa: E402
from proving_gb300 import prover as pr  # noqa: E402
from proving_gb300.synthetic import m31_column  # noqa: E402

N_COLS = 100


@pytest.fixture(scope="module")
def gpu():
    from proving_gb300 import build
    build.build()
    return pr.GpuOps()


def _prove(ops, trace_host, log_n):
    fp = pr.FriParams(pow_bits=10, log_blowup_factor=1, log_last_layer_degree_bound=0, n_queries=70, fold_step=1)
    cfg = pr.PcsConfig(fp, trace_lifting_log_size=log_n + 1)
    ch = pr.Blake2sChannel()
    proof = pr.prove_wide_fib(ops, ops.columns_from_host(trace_host), log_n, cfg, ch, ops.twiddles(log_n + 2))
    return proof, ch


@pytest.mark.parametrize("log_n", [4, 7, 10, 14])
def test_gpu_proof_bytes_equal_oracle(gpu, log_n):
    trace = O.wide_fib_trace(m31_column(11, log_n), m31_column(12, log_n), N_COLS)
    g, gch = _prove(gpu, trace, log_n)
    c, cch = _prove(CpuOps(), trace, log_n)
    assert gch.digest == cch.digest
    assert g.to_bytes() == c.to_bytes()
    verify_wide_fib(g, N_COLS, log_n)


def test_device_trace_generation_proof(gpu):
    # trace generated on the device (cs_wide_fib_trace) proves the same statement
    log_n = 10
    a, b = m31_column(21, log_n), m31_column(22, log_n)
    from proving_gb300.backend import BaseColumn, CudaBackend
    dev_trace = CudaBackend.wide_fib_trace(BaseColumn.from_cpu(a), BaseColumn.from_cpu(b), N_COLS)
    fp = pr.FriParams()
    cfg = pr.PcsConfig(fp, trace_lifting_log_size=log_n + 1)
    proof = pr.prove_wide_fib(gpu, dev_trace, log_n, cfg, pr.Blake2sChannel(), gpu.twiddles(log_n + 2))
    host, _ = _prove(CpuOps(), O.wide_fib_trace(a, b, N_COLS), log_n)
    assert proof.to_bytes() == host.to_bytes()


def test_lifted_components_match_oracle(gpu):
    # two Wide-Fibonacci components of 2^9 and 2^3 rows in one lifted tree (test_e2e_lifted_fib_prove,
    # crates/examples/src/wide_fibonacci/mod.rs:495-577): the same proof bytes on both backends
    from oracle.verifier import verify_wide_fib_components
    from test_prove_cpu import lifted_components_proof
    g, c = lifted_components_proof(gpu), lifted_components_proof(CpuOps())
    assert g.to_bytes() == c.to_bytes()
    verify_wide_fib_components(g, [4, 5], [9, 3])


def test_fib_and_lookups_match_oracle(gpu):
    # Wide-Fibonacci and LogUp components of four sizes in one proof: the same bytes and claimed sums
    # on both backends, and the restated verifier accepts
    from oracle.verifier import verify_fib_and_lookups
    from test_prove_cpu import fib_and_lookups_proof
    g, c = fib_and_lookups_proof(gpu), fib_and_lookups_proof(CpuOps())
    assert g.claimed_sums == c.claimed_sums
    assert g.to_bytes() == c.to_bytes()
    verify_fib_and_lookups(g, [4, 5], [9, 3], [8, 4], g.claimed_sums)


def test_mixed_shape_proof_matches_oracle(gpu):
    # the batched mixed-size trace at a reduced scale (60 base columns, 12 LogUp components, log sizes
    # 4..11): Wide-Fibonacci components per size plus LogUp components, same proof bytes on both backends
    from oracle.verifier import verify_fib_and_lookups
    from proving_gb300.synthetic import mixed_trace_shape
    comps, lookup_logs = mixed_trace_shape(seed=3, n_base=60, n_interaction=12, lo=4, hi=11, mean=7.0)
    max_log = max([l for _, l in comps] + lookup_logs)
    fp = pr.FriParams(pow_bits=10, log_blowup_factor=1, log_last_layer_degree_bound=0, n_queries=70, fold_step=1)
    cfg = pr.PcsConfig(fp, trace_lifting_log_size=max_log + 1)

    def prove(ops):
        traces = [ops.columns_from_host(O.wide_fib_trace(m31_column(10 + i, l), m31_column(50 + i, l), n))
                  for i, (n, l) in enumerate(comps)]
        values = [ops.columns_from_host([m31_column(90 + k, l)])[0] for k, l in enumerate(lookup_logs)]
        return pr.prove_fib_and_lookups(ops, traces, [l for _, l in comps], values, lookup_logs, cfg,
                                        pr.Blake2sChannel(), ops.twiddles(max_log + 2))

    g, c = prove(gpu), prove(CpuOps())
    assert g.to_bytes() == c.to_bytes()
    assert g.claimed_sums == c.claimed_sums
    verify_fib_and_lookups(g, [n for n, _ in comps], [l for _, l in comps], lookup_logs, g.claimed_sums)


def test_fri_graph_replay_matches_oracle():
    # the second and third proofs of one size replay the captured FRI layer loop: each equals the
    # oracle's proof of its own trace
    from proving_gb300 import build
    build.build()
    ops = pr.GpuOps()
    log_n = 8
    tw = ops.twiddles(log_n + 2)
    fp = pr.FriParams(pow_bits=10, log_blowup_factor=1, log_last_layer_degree_bound=0, n_queries=70, fold_step=1)
    cfg = pr.PcsConfig(fp, trace_lifting_log_size=log_n + 1)
    seen = set()
    for seed in (31, 33, 35):
        trace = O.wide_fib_trace(m31_column(seed, log_n), m31_column(seed + 1, log_n), N_COLS)
        g = pr.prove_wide_fib(ops, ops.columns_from_host(trace), log_n, cfg, pr.Blake2sChannel(), tw)
        c, _ = _prove(CpuOps(), trace, log_n)
        assert g.to_bytes() == c.to_bytes()
        seen.add(g.to_bytes())
    assert len(seen) == 3 and len(ops._fri_graphs) == 1
