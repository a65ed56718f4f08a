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
