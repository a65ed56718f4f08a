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
