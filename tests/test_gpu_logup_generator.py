"""GPU parity of the LogupTraceGenerator entry points (cs_logup_combine, cs_logup_gen_col,
cs_logup_finalize_last; crates/constraint-framework/src/prover/logup.rs:22-196) with the oracle's
restatement, bit-exact: a relation of several values with multiplicities batched in pairs (whose
oracle trace satisfies the relation's constraints, test_logup_generator_cpu.py), QM31 numerators,
and combinations of more values than one launch takes."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import oracle as O  # noqa: E402
from proving_gb300 import framework as fw  # noqa: E402
from proving_gb300.synthetic import m31_column, qm31_column, seeded_qm31  # noqa: E402
from test_logup_generator_cpu import pairs_interaction_oracle, pairs_trace  # noqa: E402

P = O.P


@pytest.fixture(scope="module")
def B():
    from proving_gb300 import build
    build.build()
    from proving_gb300 import backend
    return backend


@pytest.mark.parametrize("log_n", [1, 5, 10, 14])
def test_pair_batched_relation_equals_oracle(B, log_n):
    trace = pairs_trace(60 + log_n, log_n)
    z, alpha = seeded_qm31(61), seeded_qm31(62)
    want, want_claimed = pairs_interaction_oracle(trace, z, alpha)
    cols = [B.BaseColumn.from_cpu(t) for t in trace]
    pw = fw.alpha_powers(alpha, 2)
    d0 = B.logup_combine([cols[0], cols[1]], pw, z)
    d1 = B.logup_combine([cols[2], cols[0]], pw, z)
    d2 = B.logup_combine([cols[1]], pw[:1], z)
    n = 1 << log_n
    minus_one = B.BaseColumn.from_cpu(np.full(n, P - 1, np.uint32))
    one = B.BaseColumn.from_cpu(np.ones(n, np.uint32))
    gen = B.LogupTraceGenerator(log_n)
    gen.col_from_fractions([(cols[3], d0), (minus_one, d1)])
    gen.col_from_fractions([(one, d2)])
    inter, claimed = gen.finalize_last()
    assert claimed == tuple(int(x) for x in want_claimed)
    assert len(inter) == 8
    for k, (g, w) in enumerate(zip(inter, want)):
        assert np.array_equal(g.to_cpu(), w), k


def test_qm31_numerators_and_wide_combine_equal_oracle(B):
    log_n = 9
    vals = [m31_column(100 + i, log_n) for i in range(40)]  # two launches of combine (32 + 8 values)
    pw = fw.alpha_powers(seeded_qm31(101), 40)
    z = seeded_qm31(102)
    den = B.logup_combine([B.BaseColumn.from_cpu(v) for v in vals], pw, z)
    want_den = O.logup_combine(vals, pw, z)
    assert all(np.array_equal(a, b) for a, b in zip(den.to_cpu(), want_den))
    num = qm31_column(103, log_n)
    gen = B.LogupTraceGenerator(log_n)
    gen.col_from_fractions([(B.SecureColumnByCoords.from_cpu(num), den)])
    gen.col_from_fractions([(B.SecureColumnByCoords.from_cpu(qm31_column(104, log_n)), den)])
    inter, claimed = gen.finalize_last()
    c0 = O.logup_gen_col(num, want_den)
    c1 = O.logup_gen_col(qm31_column(104, log_n), want_den, c0)
    c1, want_claimed = O.logup_finalize_last(c1)
    assert claimed == tuple(int(x) for x in want_claimed)
    assert all(np.array_equal(g.to_cpu(), w) for g, w in zip(inter, c0 + c1))
