"""Whole proofs at the benchmark sizes: the native provers on the GPU against the oracle's own
prover (oracle/oracle_prover.c: prove_ex, the commitment scheme, FRI and the CairoSerialize felt
stream restated in C from the reference, sharing no code with the product), byte for byte, and the
restated verifier (oracle/verifier.py) accepts the bytes.

- Wide-Fibonacci, 100 columns x 2^14 rows (log blowup 1, 70 queries, pow 10);
- the batched mixed-size trace: 480 Wide-Fibonacci columns in 13 components and 120 single-column
  LogUp components, log sizes 10..22 (mean ~16), lifting log size 23;
- Poseidon2, 8 instances per row, 2^18 rows (2^21 permutations): the words the reference computes
  before its sanity check, which this AIR fails in the lifted protocol.

The oracle runs on every host core; the mixed-size proof takes it about a minute."""
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import oracle as O  # noqa: E402
from oracle.verifier import parse_proof, verify_fib_and_lookups, verify_wide_fib_components  # noqa: E402
from proving_gb300.synthetic import m31_column, mixed_trace_shape  # noqa: E402

FRI = (10, 1, 0, 70)


@pytest.fixture(scope="module")
def B():
    from proving_gb300 import build
    build.build()
    from proving_gb300.backend import CudaBackend
    return CudaBackend


def _twiddles(domain_log):
    from proving_gb300 import prover as pr
    return pr.GpuOps().twiddles(domain_log)


def test_wide_fibonacci_100x2e14(B):
    from proving_gb300.backend import BaseColumn
    a, b = m31_column(101, 14), m31_column(102, 14)
    trace = B.wide_fib_trace(BaseColumn.from_cpu(a), BaseColumn.from_cpu(b), 100)
    native = B.prove_wide_fib_native([trace], [14], FRI, _twiddles(16))
    want, _ = O.prove_fib_and_lookups(FRI + (1,), [O.wide_fib_trace(a, b, 100)], [14])
    assert native == want
    verify_wide_fib_components(parse_proof(native, 15), [100], [14])


def test_mixed_size_600_plus_120_columns(B):
    from proving_gb300.backend import BaseColumn
    comps, lookup_logs = mixed_trace_shape()
    assert sum(n for n, _ in comps) + len(lookup_logs) == 600 and len(lookup_logs) == 120
    logs = [l for _, l in comps]
    max_log = max(logs + lookup_logs)
    seeds = [(m31_column(300 + i, l), m31_column(400 + i, l)) for i, (_, l) in enumerate(comps)]
    values = [m31_column(500 + k, l) for k, l in enumerate(lookup_logs)]
    traces = [B.wide_fib_trace(BaseColumn.from_cpu(a), BaseColumn.from_cpu(b), n) for (a, b), (n, _) in zip(seeds, comps)]
    native, claimed = B.prove_fib_and_lookups_native(traces, logs, [BaseColumn.from_cpu(v) for v in values],
                                                     lookup_logs, FRI, _twiddles(max_log + 2))
    del traces
    torch.cuda.empty_cache()
    host = [O.wide_fib_trace(a, b, n) for (a, b), (n, _) in zip(seeds, comps)]
    want, want_claimed = O.prove_fib_and_lookups(FRI + (1,), host, logs, values, lookup_logs)
    assert claimed == want_claimed
    assert native == want
    verify_fib_and_lookups(parse_proof(native, max_log + 1), [n for n, _ in comps], logs, lookup_logs, claimed)


def test_poseidon_2e18_rows(B):
    native = B.prove_poseidon_native(18, FRI, _twiddles(21))
    assert native == O.prove_poseidon(FRI + (1,), 18)
