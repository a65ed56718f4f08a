"""GPU parity of the Wide-Fibonacci AIR kernels (trace generation and
constraint quotients on the evaluation domain) against the oracle."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import oracle as O  # noqa: E402
from proving_gb300.synthetic import m31_column, seeded_qm31  # noqa: E402


@pytest.fixture(scope="module")
def B():
    from proving_gb300 import build
    build.build()
    from proving_gb300.backend import CudaBackend
    return CudaBackend


@pytest.mark.parametrize("n_cols,log_n", [(3, 4), (100, 10), (100, 14)])
def test_trace_and_composition(B, n_cols, log_n):
    from proving_gb300.backend import BaseColumn, SecureColumnByCoords, canonic_half_coset
    a, b = m31_column(1, log_n), m31_column(2, log_n)
    cols = B.wide_fib_trace(BaseColumn.from_cpu(a), BaseColumn.from_cpu(b), n_cols)
    want_cols = O.wide_fib_trace(a, b, n_cols)
    for c, w in zip(cols, want_cols):
        assert np.array_equal(c.to_cpu(), w)
    # extend to the evaluation domain (log + 1) and evaluate the constraints there
    tree = B.precompute_twiddles(canonic_half_coset(log_n + 2))
    tw, itw = O.canonic_twiddles(log_n + 2)
    B.interpolate_columns(cols, tree)
    ev = B.evaluate_polynomials(cols, log_n + 1, tree)
    ev_o = O.evaluate_batch(O.interpolate_batch(want_cols, itw), [log_n + 1] * n_cols, tw)
    rc = np.stack([seeded_qm31(k) for k in range(n_cols - 2)])
    acc = SecureColumnByCoords.zeros(1 << (log_n + 1))
    B.wide_fib_composition(ev, log_n, rc, acc)
    want = O.wide_fib_composition(ev_o, log_n + 1, log_n, rc)
    assert all(np.array_equal(g, w) for g, w in zip(acc.to_cpu(), want))


@pytest.mark.parametrize("log_n", [1, 3, 9, 10, 13, 16])
def test_logup_running_sum(B, log_n):
    from proving_gb300.backend import BaseColumn
    v = m31_column(log_n + 40, log_n)
    z = seeded_qm31(log_n)
    got, claimed = B.logup_running_sum(BaseColumn.from_cpu(v), z)
    want, wclaimed = O.logup_running_sum(v, z)
    assert list(claimed) == list(wclaimed)
    assert all(np.array_equal(g, w) for g, w in zip(got.to_cpu(), want))


def test_logup_running_sums_batched(B):
    # 60 columns of sizes 2^1 .. 2^16 in one batch of launches (two kernel batches of 48 columns)
    from proving_gb300.backend import BaseColumn
    logs = [1 + (k * 7) % 16 for k in range(60)]
    z = seeded_qm31(99)
    vals = [m31_column(1000 + k, l) for k, l in enumerate(logs)]
    outs, claimed = B.logup_running_sums([BaseColumn.from_cpu(v) for v in vals], z)
    claimed = claimed.cpu().numpy().view(np.uint32)
    for k, (v, out) in enumerate(zip(vals, outs)):
        want, wclaimed = O.logup_running_sum(v, z)
        assert list(claimed[k]) == list(wclaimed)
        assert all(np.array_equal(g, w) for g, w in zip(out.to_cpu(), want))


@pytest.mark.parametrize("trace_log,eval_log", [(1, 2), (4, 5), (10, 11), (13, 15)])
def test_logup_composition(B, trace_log, eval_log):
    # a single-column LogUp component's constraint quotients, (cur - prev + claimed / 2^n) (v - z) + 1
    # over the vanishing polynomial, added to an accumulator that already holds values
    from proving_gb300.backend import BaseColumn, SecureColumnByCoords
    n = 1 << eval_log
    v = m31_column(eval_log + 7, eval_log)
    inter = [m31_column(eval_log + 8 + k, eval_log) for k in range(4)]
    z, claimed, rc = seeded_qm31(1), seeded_qm31(2), seeded_qm31(3)
    base = [m31_column(eval_log + 20 + k, eval_log) for k in range(4)]
    acc = SecureColumnByCoords([BaseColumn.from_cpu(c) for c in base])
    B.logup_composition(BaseColumn.from_cpu(v), SecureColumnByCoords([BaseColumn.from_cpu(c) for c in inter]),
                        trace_log, z, claimed, rc, acc)
    want = O.logup_composition(v, inter, trace_log, z, claimed, rc, out=[c.copy() for c in base])
    assert len(acc) == n
    assert all(np.array_equal(g, w) for g, w in zip(acc.to_cpu(), want))


def test_logup_compositions_batched(B):
    # 30 LogUp components of one size in two launches: the same accumulator as one call each
    from proving_gb300.backend import BaseColumn, SecureColumnByCoords
    trace_log, eval_log = 9, 10
    comps = []
    for k in range(30):
        v = m31_column(300 + k, eval_log)
        inter = [m31_column(400 + 4 * k + c, eval_log) for c in range(4)]
        comps.append((v, inter, seeded_qm31(500 + k), seeded_qm31(600 + k)))
    z = seeded_qm31(7)
    base = [m31_column(700 + c, eval_log) for c in range(4)]
    acc = SecureColumnByCoords([BaseColumn.from_cpu(c) for c in base])
    B.logup_compositions([BaseColumn.from_cpu(v) for v, _, _, _ in comps],
                         [SecureColumnByCoords([BaseColumn.from_cpu(c) for c in it]) for _, it, _, _ in comps],
                         trace_log, z, [c for _, _, c, _ in comps], [r for _, _, _, r in comps], acc)
    want = [c.copy() for c in base]
    for v, it, c, r in comps:
        want = O.logup_composition(v, it, trace_log, z, c, r, out=want)
    assert all(np.array_equal(g, w) for g, w in zip(acc.to_cpu(), want))
