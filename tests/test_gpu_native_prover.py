"""The native provers (cs_prove_wide_fib, cs_prove_fib_and_lookups, cs_prove_poseidon: the generic
prover's loop in C++ over the library's kernels) against the oracle's own prover
(oracle/oracle_prover.c, the reference's prove_ex restated in C, sharing no code with the product):
byte-identical proofs, which the restated verifier accepts. Small shapes here, including edge
sizes; the BASELINE-size proofs are in test_gpu_proof_parity_full.py."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import oracle as O  # noqa: E402
from oracle.verifier import parse_proof, verify_fib_and_lookups, verify_wide_fib_components  # noqa: E402
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
                                             ([(4, 9), (5, 3)], 3), ([(10, 6), (3, 6), (7, 11)], 20),
                                             ([(3, 2)], 5), ([(5, 2), (3, 1)], 9)])
def test_native_proof_bytes_equal_oracle_prover(B, shape, n_queries):
    from proving_gb300.backend import BaseColumn
    host = _traces(shape, 50)
    logs = [l for _, l in shape]
    L = max(logs) + 1
    tw = pr.GpuOps().twiddles(L + 1)
    native = B.prove_wide_fib_native([[BaseColumn.from_cpu(c) for c in t] for t in host], logs,
                                     (10, 1, 0, n_queries), tw)
    want, _ = O.prove_fib_and_lookups((10, 1, 0, n_queries, 1), host, logs)
    assert native == want
    verify_wide_fib_components(parse_proof(native, L), [n for n, _ in shape], logs)


def _fib_lookup_inputs(shape, lookup_logs, seed):
    traces = _traces(shape, seed)
    rng = np.random.default_rng(seed)
    values = [rng.integers(0, O.P, 1 << l, dtype=np.uint32) for l in lookup_logs]
    return traces, values


@pytest.mark.parametrize("shape,lookup_logs,n_queries", [([(4, 9), (5, 3)], [8, 4], 3),
                                                         ([(10, 5), (3, 8)], [8, 2, 5, 8], 70),
                                                         ([(3, 3)], [11, 1], 17)])
def test_native_fib_and_lookups_equal_oracle_prover(B, shape, lookup_logs, n_queries):
    from proving_gb300.backend import BaseColumn
    host, values = _fib_lookup_inputs(shape, lookup_logs, 7)
    logs = [l for _, l in shape]
    L = max(logs + lookup_logs) + 1
    tw = pr.GpuOps().twiddles(L + 1)
    native, claimed = B.prove_fib_and_lookups_native(
        [[BaseColumn.from_cpu(c) for c in t] for t in host], logs, [BaseColumn.from_cpu(v) for v in values],
        lookup_logs, (10, 1, 0, n_queries), tw)
    want, want_claimed = O.prove_fib_and_lookups((10, 1, 0, n_queries, 1), host, logs, values, lookup_logs)
    assert claimed == want_claimed
    assert native == want
    verify_fib_and_lookups(parse_proof(native, L), [n for n, _ in shape], logs, lookup_logs, claimed)


@pytest.mark.parametrize("fold_step,last_layer,n_queries", [(2, 0, 3), (3, 1, 20), (4, 2, 70), (2, 3, 5)])
def test_native_fold_steps_equal_oracle_prover(B, fold_step, last_layer, n_queries):
    # FRI with several folds per layer in the native loop (packed leaves, the channel on the host
    # for the layer loop) and last layers of higher degree: the oracle prover's words
    from proving_gb300.backend import BaseColumn
    shape, lookup_logs = [(4, 9), (5, 3)], [8, 4]
    host, values = _fib_lookup_inputs(shape, lookup_logs, 7)
    logs = [l for _, l in shape]
    L = max(logs + lookup_logs) + 1
    tw = pr.GpuOps().twiddles(L + 1)
    fri = (10, 1, last_layer, n_queries, fold_step)
    native, claimed = B.prove_fib_and_lookups_native(
        [[BaseColumn.from_cpu(c) for c in t] for t in host], logs, [BaseColumn.from_cpu(v) for v in values],
        lookup_logs, fri, tw)
    want, want_claimed = O.prove_fib_and_lookups(fri, host, logs, values, lookup_logs)
    assert claimed == want_claimed
    assert native == want


@pytest.mark.parametrize("fold_step,last_layer", [(2, 0), (3, 1)])
def test_native_poseidon_fold_steps_equal_oracle_prover(B, fold_step, last_layer):
    tw = pr.GpuOps().twiddles(7)
    assert B.prove_poseidon_native(4, (10, 1, last_layer, 70, fold_step), tw) == \
        O.prove_poseidon((10, 1, last_layer, 70, fold_step), 4)


@pytest.mark.parametrize("log_n", [4, 7])
def test_native_poseidon_equals_oracle_prover(B, log_n):
    tw = pr.GpuOps().twiddles(log_n + 3)
    native = B.prove_poseidon_native(log_n, (10, 1, 0, 70), tw)
    assert native == O.prove_poseidon((10, 1, 0, 70, 1), log_n)


@pytest.mark.parametrize("log_n", [4, 9])
def test_restated_host_prover_equals_native(B, log_n):
    # the restated (Python) host prover on the same kernels gives the native prover's bytes
    from proving_gb300.backend import BaseColumn
    host = _traces([(20, log_n)], 3)
    fp = pr.FriParams(pow_bits=10, log_blowup_factor=1, log_last_layer_degree_bound=0, n_queries=30, fold_step=1)
    ops = pr.GpuOps()
    tw = ops.twiddles(log_n + 2)
    native = B.prove_wide_fib_native([[BaseColumn.from_cpu(c) for c in t] for t in host], [log_n], (10, 1, 0, 30), tw)
    restated = pr.prove_wide_fib_components(ops, [ops.columns_from_host(t) for t in host], [log_n],
                                            pr.PcsConfig(fp, trace_lifting_log_size=log_n + 1), pr.Blake2sChannel(),
                                            tw)
    assert native == restated.to_bytes()


def test_plain_form_gives_the_same_proofs(B):
    # CS_PROVE_PLAIN (one launch per column for every per-column stage) proves the same bytes as the
    # batched form, for Wide-Fibonacci with LogUp components of several sizes and for Poseidon2
    from proving_gb300 import _lib
    from proving_gb300.backend import BaseColumn
    shape, lookup_logs = [(10, 5), (3, 8), (4, 2)], [8, 2, 5, 8, 11]
    host, values = _fib_lookup_inputs(shape, lookup_logs, 9)
    logs = [l for _, l in shape]
    L = max(logs + lookup_logs) + 1
    tw = pr.GpuOps().twiddles(L + 1)
    proofs, launches = [], []
    for plain in (False, True):
        n0 = _lib.load().cs_kernel_launch_count()
        w, cl = B.prove_fib_and_lookups_native([[BaseColumn.from_cpu(c) for c in t] for t in host], logs,
                                               [BaseColumn.from_cpu(v) for v in values], lookup_logs, (10, 1, 0, 20),
                                               tw, plain=plain)
        torch.cuda.synchronize()
        launches.append(_lib.load().cs_kernel_launch_count() - n0)
        proofs.append((w, cl))
    assert proofs[0] == proofs[1]
    assert launches[1] > launches[0]
    want, _ = O.prove_fib_and_lookups((10, 1, 0, 20, 1), host, logs, values, lookup_logs)
    assert proofs[0][0] == want
    tw = pr.GpuOps().twiddles(7)
    assert B.prove_poseidon_native(4, (10, 1, 0, 70), tw, plain=True) == B.prove_poseidon_native(4, (10, 1, 0, 70), tw)
