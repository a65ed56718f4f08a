"""The generic constraint path on the CPU: AIRs written against the framework's evaluator give
the same quotients, evaluated by the oracle's CPU constraint evaluator, as the oracle's own
Wide-Fibonacci and LogUp composition functions; and the generated kernel source has the shape the
C ABI launches (no GPU needed)."""
import numpy as np
import pytest

from oracle import oracle as O
from oracle.air_eval import air_composition
from proving_gb300 import framework as fw
from proving_gb300.synthetic import m31_column, seeded_qm31


@pytest.mark.parametrize("n_cols,trace_log,eval_log", [(3, 3, 4), (10, 5, 6), (20, 6, 8)])
def test_wide_fib_air_matches_oracle(n_cols, trace_log, eval_log):
    air = fw.compile_air("wide_fib", fw.wide_fib_air, n_cols)
    assert air.n_constraints == n_cols - 2 and len(air.masks) == n_cols
    cols = [m31_column(40 + k, eval_log) for k in range(n_cols)]
    rc = np.stack([seeded_qm31(90 + k) for k in range(n_cols - 2)])
    base = [m31_column(70 + k, eval_log) for k in range(4)]
    got = air_composition(air, {1: cols}, eval_log, trace_log, {}, rc, out=base)
    want = O.wide_fib_composition(cols, eval_log, trace_log, rc, out=[b.copy() for b in base])
    assert all(np.array_equal(g, w) for g, w in zip(got, want))


@pytest.mark.parametrize("trace_log,eval_log", [(1, 2), (4, 5), (6, 8)])
def test_single_lookup_air_matches_oracle(trace_log, eval_log):
    air = fw.compile_air("lookup", fw.single_lookup_air)
    assert air.n_constraints == 1 and air.params == ["z", "shift"]
    assert sorted((m.interaction, m.column, m.offset) for m in air.masks) == \
        [(1, 0, 0)] + [(2, k, off) for k in range(4) for off in (-1, 0)]
    v = m31_column(5, eval_log)
    inter = [m31_column(6 + k, eval_log) for k in range(4)]
    z, claimed, rc = seeded_qm31(1), seeded_qm31(2), seeded_qm31(3)
    shift = (np.asarray(claimed, np.int64) * pow(1 << trace_log, O.P - 2, O.P) % O.P).astype(np.uint32)
    got = air_composition(air, {1: [v], 2: inter}, eval_log, trace_log, {"z": z, "shift": shift}, [rc])
    want = O.logup_composition(v, inter, trace_log, z, claimed, rc)
    assert all(np.array_equal(g, w) for g, w in zip(got, want))


def test_generated_source_shape():
    air = fw.compile_air("lookup", fw.single_lookup_air)
    src = air.source
    assert 'extern "C" __global__ void __launch_bounds__(256) cs_air_composition(' in src
    assert src.count("__ldg(cols[") == 9          # 1 value mask + 4 coordinates x 2 rows
    assert "prev_row(r, trace_log, eval_log)" in src
    # shared subexpressions are emitted once
    air2 = fw.compile_air("fib", fw.wide_fib_air, 5)
    assert air2.source.count("__ldg(cols[") == 5
    # 3 constraints use the squares of columns 0..3; each square is computed once
    assert air2.source.count("m31_mul(") == 4


def _relation_lookup_air(e):
    # single_lookup_air through add_to_relation + finalize_logup (crates/constraint-framework/src/
    # lib.rs:145-151, 185-226): multiplicity -1, values [v], relation "lookup"
    e.add_to_relation("lookup", -1, [e.next_trace_mask()])
    e.finalize_logup()


@pytest.mark.parametrize("trace_log,eval_log", [(2, 3), (5, 6)])
def test_relation_entries_finalized_like_the_hand_written_logup(trace_log, eval_log):
    # one entry, no batching: the constraint of single_lookup_air, with z = lookup_z and alpha^0 = 1
    air = fw.compile_air("lookup_rel", _relation_lookup_air)
    assert air.n_constraints == 1 and air.params == ["lookup_alpha0", "lookup_z", "shift"]
    v = m31_column(15, eval_log)
    inter = [m31_column(16 + k, eval_log) for k in range(4)]
    z, claimed, rc = seeded_qm31(21), seeded_qm31(22), seeded_qm31(23)
    shift = (np.asarray(claimed, np.int64) * pow(1 << trace_log, O.P - 2, O.P) % O.P).astype(np.uint32)
    params = {"lookup_alpha0": (1, 0, 0, 0), "lookup_z": z, "shift": shift}
    got = air_composition(air, {1: [v], 2: inter}, eval_log, trace_log, params, [rc])
    want = O.logup_composition(v, inter, trace_log, z, claimed, rc)
    assert all(np.array_equal(g, w) for g, w in zip(got, want))


def test_finalize_batches_need_fractions():
    e = fw.Evaluator()
    with pytest.raises(AssertionError):
        e.finalize_logup_in_pairs()


@pytest.mark.parametrize("trace_log,eval_log", [(3, 5), (4, 6)])
def test_poseidon_air_matches_oracle(trace_log, eval_log):
    # eval_poseidon_constraints (crates/examples/src/poseidon/mod.rs:137-187) written against the
    # evaluator, relation entries finalized in pairs: the oracle's Poseidon2 composition
    from proving_gb300.synthetic import m31_columns
    air = fw.poseidon_air_recorded()
    assert air.n_constraints == O.POSEIDON_CONSTRAINTS
    assert len(air.params) == 18
    # 1264 trace columns at the row; 28 interaction columns at the row, the last 4 at both rows
    assert sum(m.interaction == 1 for m in air.masks) == O.POSEIDON_COLS
    assert sorted((m.column, m.offset) for m in air.masks if m.offset == -1) == [(k, -1) for k in range(28, 32)]
    trace = m31_columns(500 + eval_log, O.POSEIDON_COLS, eval_log)
    inter = m31_columns(600 + eval_log, O.POSEIDON_INTERACTION_COLS, eval_log)
    lookup = list(seeded_qm31(31)) + list(seeded_qm31(32))
    claimed = list(seeded_qm31(33))
    rc = np.random.default_rng(eval_log).integers(0, O.P, (O.POSEIDON_CONSTRAINTS, 4)).astype(np.uint32)
    start = m31_columns(700, 4, eval_log)
    want = O.poseidon_composition(trace, inter, trace_log, lookup, claimed, rc, out=[s.copy() for s in start])
    got = air_composition(air, {1: trace, 2: inter}, eval_log, trace_log, fw.poseidon_params(lookup, claimed, trace_log),
                          rc, out=[s.copy() for s in start])
    assert all(np.array_equal(np.asarray(g, np.uint32), np.asarray(w, np.uint32)) for g, w in zip(got, want))


def test_large_bodies_are_split_into_functions():
    # a body over the single-function limit becomes non-inlined functions in constraint order, values
    # passed through xs; small AIRs keep one inlined body
    import re
    small = fw.compile_air("fib", fw.wide_fib_air, 100).source
    assert "__noinline__" not in small and "uint32_t xs[" not in small
    src = fw.poseidon_air_recorded().source
    groups = re.findall(r"cs_air_group(\d+)\(const uint32_t\* const\* __restrict__ cols", src)
    assert len(groups) > 8 and groups == [str(g) for g in range(len(groups))]
    n_xs = int(re.search(r"uint32_t xs\[(\d+)\];", src).group(1))
    assert 0 < n_xs < 4096
    # every xs slot a function reads was written by an earlier function
    written, bodies = set(), src.split("__device__ __noinline__ qm31 cs_air_group")[1:]
    for body in bodies:
        reads = {int(x) for x in re.findall(r"= xs\[(\d+)\]", body)} | \
                {int(x) for x in re.findall(r"qm31_make\(xs\[(\d+)\]", body)}
        assert reads <= written
        written |= {int(x) for x in re.findall(r"xs\[(\d+)\] =", body)}
    assert src.count(" qm31_add(acc, cs_air_group") == len(groups)
