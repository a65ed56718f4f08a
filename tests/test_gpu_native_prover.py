"""The native prover (cs_prove_wide_fib: the generic prover's loop in C++ over the library's kernels)
gives the proof bytes of the restated prover on the same backend and of the oracle backend."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import oracle as O  # noqa: E402
from oracle.cpu_ops import CpuOps  # noqa: E402
from oracle.verifier import verify_wide_fib_components  # noqa: E402
from proving_gb300 import prover as pr  # noqa: E402
from proving_gb300.synthetic import m31_column  # noqa: E402


@pytest.fixture(scope="module")
def B():
    from proving_gb300 import build
    build.build()
    from proving_gb300.backend import CudaBackend
    return CudaBackend


def _traces(shape, seed):
    return [O.wide_fib_trace(m31_column(seed + 2 * k, l), m31_column(seed + 2 * k + 1, l), n)
            for k, (n, l) in enumerate(shape)]


@pytest.mark.parametrize("shape,n_queries", [([(100, 4)], 70), ([(100, 7)], 70), ([(100, 14)], 70),
                                             ([(4, 9), (5, 3)], 3), ([(10, 6), (3, 6), (7, 11)], 20)])
def test_native_proof_bytes_equal_restated_prover(B, shape, n_queries):
    from proving_gb300.backend import BaseColumn
    host = _traces(shape, 50)
    logs = [l for _, l in shape]
    L = max(logs) + 1
    fp = pr.FriParams(pow_bits=10, log_blowup_factor=1, log_last_layer_degree_bound=0, n_queries=n_queries, fold_step=1)
    cfg = pr.PcsConfig(fp, trace_lifting_log_size=L)
    ops = pr.GpuOps()
    tw = ops.twiddles(L + 1)
    native = B.prove_wide_fib_native([[BaseColumn.from_cpu(c) for c in t] for t in host], logs,
                                     (fp.pow_bits, fp.log_blowup_factor, fp.log_last_layer_degree_bound,
                                      fp.n_queries), tw)
    restated = pr.prove_wide_fib_components(ops, [ops.columns_from_host(t) for t in host], logs, cfg,
                                            pr.Blake2sChannel(), tw)
    assert native == restated.to_bytes()
    if max(logs) <= 10:
        cpu = CpuOps()
        oracle = pr.prove_wide_fib_components(cpu, [cpu.columns_from_host(t) for t in host], logs, cfg,
                                              pr.Blake2sChannel(), cpu.twiddles(L + 1))
        assert native == oracle.to_bytes()
        verify_wide_fib_components(restated, [n for n, _ in shape], logs)


def _fib_lookup_inputs(shape, lookup_logs, seed):
    traces = _traces(shape, seed)
    rng = np.random.default_rng(seed)
    values = [rng.integers(0, O.P, 1 << l, dtype=np.uint32) for l in lookup_logs]
    return traces, values


@pytest.mark.parametrize("shape,lookup_logs,n_queries", [([(4, 9), (5, 3)], [8, 4], 3),
                                                         ([(10, 5), (3, 8)], [8, 2, 5, 8], 70)])
def test_native_fib_and_lookups_equal_restated_prover(B, shape, lookup_logs, n_queries):
    from proving_gb300.backend import BaseColumn
    host, values = _fib_lookup_inputs(shape, lookup_logs, 7)
    logs = [l for _, l in shape]
    L = max(logs + lookup_logs) + 1
    fp = pr.FriParams(pow_bits=10, log_blowup_factor=1, log_last_layer_degree_bound=0, n_queries=n_queries, fold_step=1)
    cfg = pr.PcsConfig(fp, trace_lifting_log_size=L)
    ops = pr.GpuOps()
    tw = ops.twiddles(L + 1)
    native, claimed = B.prove_fib_and_lookups_native(
        [[BaseColumn.from_cpu(c) for c in t] for t in host], logs, [BaseColumn.from_cpu(v) for v in values],
        lookup_logs, (fp.pow_bits, fp.log_blowup_factor, fp.log_last_layer_degree_bound, fp.n_queries), tw)
    restated = pr.prove_fib_and_lookups(ops, [ops.columns_from_host(t) for t in host], logs,
                                        [ops.columns_from_host([v])[0] for v in values], lookup_logs, cfg,
                                        pr.Blake2sChannel(), tw)
    assert claimed == restated.claimed_sums
    assert native == restated.to_bytes()


@pytest.mark.parametrize("log_n", [4, 7])
def test_native_poseidon_equals_restated_prover(B, log_n):
    from proving_gb300 import poseidon as ps
    fp = pr.FriParams(pow_bits=10, log_blowup_factor=1, log_last_layer_degree_bound=0, n_queries=70, fold_step=1)
    cfg = ps.poseidon_pcs_config(log_n + 3, fp)
    ops = pr.GpuOps()
    tw = ops.twiddles(log_n + 3)
    native = B.prove_poseidon_native(log_n, (fp.pow_bits, fp.log_blowup_factor, fp.log_last_layer_degree_bound,
                                             fp.n_queries), tw)
    restated = ps.prove_poseidon(ops, log_n, cfg, pr.Blake2sChannel(), tw, check=False)
    assert native == restated.to_bytes()
