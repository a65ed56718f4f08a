"""LogupTraceGenerator (crates/constraint-framework/src/prover/logup.rs:22-130) restated in the
oracle: LookupElements::combine, write_frac + finalize_col, finalize_last. It reproduces the
single-column running sum, and the interaction trace it builds for a relation of several values
with multiplicities, batched in pairs, satisfies that relation's constraints written against the
framework's evaluator (add_to_relation, finalize_logup_in_pairs) on every row of the trace domain."""
import numpy as np
import pytest

from oracle import oracle as O
from oracle.air_eval import air_composition
from proving_gb300 import framework as fw
from proving_gb300.synthetic import m31_column, seeded_qm31

P = O.P


def pairs_air(e):
    """Three entries of relation `rel`: (m, [a, b]), (-1, [c, a]), (1, [b]); batched in pairs, so one
    cumulative column for the first two and the running-sum column for the third."""
    a, b, c, m = (e.next_trace_mask() for _ in range(4))
    e.add_to_relation("rel", m, [a, b])
    e.add_to_relation("rel", -1, [c, a])
    e.add_to_relation("rel", 1, [b])
    e.finalize_logup_in_pairs()


def pairs_trace(seed, log_n):
    rng = np.random.default_rng(seed)
    return [m31_column(seed + k, log_n) for k in range(3)] + [rng.integers(0, 5, 1 << log_n).astype(np.uint32)]


def pairs_interaction_oracle(trace, z, alpha):
    a, b, c, m = trace
    n = a.size
    pw = fw.alpha_powers(alpha, 2)
    d0, d1, d2 = O.logup_combine([a, b], pw, z), O.logup_combine([c, a], pw, z), O.logup_combine([b], pw[:1], z)
    col0 = O.logup_gen_col(m, d0)
    col0 = O.logup_gen_col(np.full(n, P - 1, np.uint32), d1, col0)  # the pair's sum in one column
    last = O.logup_gen_col(np.ones(n, np.uint32), d2, col0)
    last, claimed = O.logup_finalize_last(last)
    return col0 + last, claimed


@pytest.mark.parametrize("log_n", [1, 4, 9])
def test_generator_reproduces_the_single_column_running_sum(log_n):
    # fraction -1 / (v - z) = 1 / (z - v) for every row, finalized: the running-sum column
    v, z = m31_column(30 + log_n, log_n), seeded_qm31(31)
    den = O.logup_combine([v], [(1, 0, 0, 0)], z)
    col = O.logup_gen_col(np.full(1 << log_n, P - 1, np.uint32), den)
    got, claimed = O.logup_finalize_last(col)
    want, want_claimed = O.logup_running_sum(v, z)
    assert list(claimed) == list(want_claimed)
    assert all(np.array_equal(g, w) for g, w in zip(got, want))


def test_combine_is_the_alpha_weighted_sum_minus_z():
    # test_lookup_elements_combine (crates/constraint-framework/src/logup.rs:101-121) per row
    vals = [np.full(4, 123, np.uint32), np.full(4, 456, np.uint32), np.full(4, 789, np.uint32)]
    z, alpha = seeded_qm31(1), seeded_qm31(2)
    pw = fw.alpha_powers(alpha, 3)
    got = O.logup_combine(vals, pw, z)
    want = [0, 0, 0, 0]
    for v, p in zip((123, 456, 789), pw):
        want = [(w + v * int(x)) % P for w, x in zip(want, p)]
    want = [(w - int(x)) % P for w, x in zip(want, z)]
    assert [int(c[0]) for c in got] == want and all(len(set(c.tolist())) == 1 for c in got)


@pytest.mark.parametrize("log_n", [3, 6])
def test_generated_interaction_satisfies_the_relation_constraints(log_n):
    trace = pairs_trace(40 + log_n, log_n)
    z, alpha = seeded_qm31(41), seeded_qm31(42)
    inter, claimed = pairs_interaction_oracle(trace, z, alpha)
    air = fw.compile_air("pairs", pairs_air)
    assert air.n_constraints == 2
    params = fw.lookup_params("rel", z, alpha, 2)
    params["shift"] = fw.logup_shift(claimed, log_n)
    rc = np.stack([seeded_qm31(50), seeded_qm31(51)])
    got = air_composition(air, {1: trace, 2: inter}, log_n, log_n, params, rc, divide=False)
    assert all(not g.any() for g in got)
    # one changed multiplicity breaks the first (pair) constraint at its row (and only there)
    bad = [t.copy() for t in trace]
    bad[3][2] = (int(bad[3][2]) + 1) % P
    got = air_composition(air, {1: bad, 2: inter}, log_n, log_n, params, rc, divide=False)
    assert sorted({int(i) for g in got for i in np.nonzero(g)[0]}) == [2]
    # a changed running-sum word breaks the last constraint
    inter_bad = [c.copy() for c in inter]
    inter_bad[5][1] = (int(inter_bad[5][1]) + 1) % P
    got = air_composition(air, {1: trace, 2: inter_bad}, log_n, log_n, params, rc, divide=False)
    assert any(g.any() for g in got)
