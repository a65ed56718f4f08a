"""Mask offsets of the constraint framework on the CPU: the oracle's row arithmetic against the
reference's own known-answer case and against the circle points the rows stand for, and an AIR
with masks at several offsets satisfied row by row on its trace domain."""
import numpy as np
import pytest

from oracle import oracle as O
from oracle.air_eval import air_composition
from proving_gb300 import framework as fw
from proving_gb300.synthetic import m31_column, seeded_qm31

ORDER = 1 << 31  # the circle group's order; a point is its index


def _brev(i: int, log_n: int) -> int:
    return int(format(i, f"0{log_n}b")[::-1], 2) if log_n else 0


def _row_point(r: int, log_n: int) -> int:
    """The point of row r of CanonicCoset(log_n)'s circle domain in bit-reversed order, as a
    circle-group index: the half coset G_{2^(log_n+1)} + <G_{2^(log_n-1)}> in the first half of
    the natural order, its conjugates in the second (CircleDomain::at)."""
    i = _brev(r, log_n)
    half = 1 << (log_n - 1)
    init, step = 1 << (30 - log_n), 1 << (32 - log_n)
    return (init + i * step) % ORDER if i < half else (-(init + (i - half) * step)) % ORDER


def test_offset_two_back_is_previous_of_previous():
    # the reference's known answer (crates/stwo/src/core/utils.rs:256-276): domain 3, evaluation 6,
    # index 5, offset -2
    prev = O.prev_rows(3, 6)
    assert O.offset_rows(-2, 3, 6)[5] == prev[prev[5]]


@pytest.mark.parametrize("trace_log,eval_log", [(1, 1), (3, 3), (5, 5), (1, 2), (3, 6), (4, 5), (6, 9)])
@pytest.mark.parametrize("offset", [-5, -2, -1, 1, 3, 17])
def test_offset_row_is_a_trace_step_on_the_circle(trace_log, eval_log, offset):
    # row offset_row(r, k) holds the point of row r plus k generators of the trace's subgroup, on the
    # trace domain (coset order) and on every larger evaluation domain alike
    rows = O.offset_rows(offset, trace_log, eval_log)
    g = 1 << (31 - trace_log)
    for r in range(1 << eval_log):
        assert _row_point(int(rows[r]), eval_log) == (_row_point(r, eval_log) + offset * g) % ORDER


@pytest.mark.parametrize("trace_log,eval_log", [(2, 2), (4, 6)])
def test_offsets_compose_and_minus_one_is_the_previous_row(trace_log, eval_log):
    a, b = O.offset_rows(3, trace_log, eval_log), O.offset_rows(-5, trace_log, eval_log)
    assert np.array_equal(b[a], O.offset_rows(-2, trace_log, eval_log))
    assert np.array_equal(O.offset_rows(-1, trace_log, eval_log), O.prev_rows(trace_log, eval_log))
    assert np.array_equal(O.offset_rows(1 << trace_log, trace_log, eval_log), np.arange(1 << eval_log))


def window_air(e):
    """y is x two rows on, z is x three rows back, and w = x[-1] x[1] + x[0]."""
    x = e.next_interaction_mask(1, (-3, -1, 0, 1, 2))
    y, z, w = e.next_trace_mask(), e.next_trace_mask(), e.next_trace_mask()
    e.add_constraint(y - x[4])
    e.add_constraint(z - x[0])
    e.add_constraint(w - x[1] * x[3] - x[2])


def window_trace(log_n: int, seed: int, bad: bool = False):
    """x random; y, z, w from x's neighbours in coset order (the trace's row order along the
    subgroup), laid out in bit-reversed circle-domain order."""
    n = 1 << log_n
    xs = np.random.default_rng(seed).integers(0, O.P, n, dtype=np.int64)   # by coset index
    k = np.arange(n)
    y, z, w = xs[(k + 2) % n], xs[(k - 3) % n], (xs[(k - 1) % n] * xs[(k + 1) % n] + xs) % O.P
    if bad:
        y = xs[(k + 1) % n]
    # coset index -> natural circle-domain index -> bit-reversed row
    half = n // 2
    nat = np.where(k % 2 == 0, k // 2, n - 1 - (k - 1) // 2) if n > 1 else k
    rows = np.array([_brev(int(v), log_n) for v in nat], np.int64)
    cols = []
    for c in (xs, y, z, w):
        out = np.zeros(n, np.uint32)
        out[rows] = c
        cols.append(out)
    return cols


def test_window_air_masks_and_source():
    air = fw.compile_air("window", window_air)
    assert sorted({m.offset for m in air.masks}) == [-3, -1, 0, 1, 2]
    for name, call in (("ro_m3", "offset_row(r, -3, trace_log, eval_log)"), ("pr", "prev_row(r, trace_log, eval_log)"),
                       ("ro_p1", "offset_row(r, 1, trace_log, eval_log)"),
                       ("ro_p2", "offset_row(r, 2, trace_log, eval_log)")):
        assert f"const uint32_t {name} = {call};" in air.source
    with pytest.raises(ValueError):
        fw.compile_air("bad", lambda e: e.next_interaction_mask(1, (0.5,)))


@pytest.mark.parametrize("log_n", [1, 3, 6])
def test_window_air_holds_on_its_trace_domain(log_n):
    air = fw.compile_air("window", window_air)
    rc = np.stack([seeded_qm31(30 + k) for k in range(air.n_constraints)])
    zero = [np.zeros(1 << log_n, np.uint32) for _ in range(4)]
    got = air_composition(air, {1: window_trace(log_n, 5)}, log_n, log_n, {}, rc, out=zero, divide=False)
    assert all(not g.any() for g in got)
    bad = air_composition(air, {1: window_trace(log_n, 5, bad=True)}, log_n, log_n, {}, rc, out=zero,
                          divide=False)
    assert any(b.any() for b in bad)


def test_window_air_on_an_evaluation_domain_reads_the_offset_rows():
    # on a larger domain each mask reads its column at orc_offset_row: the quotient sum of the oracle's
    # evaluator equals one written out from those rows
    trace_log, eval_log = 3, 5
    air = fw.compile_air("window", window_air)
    cols = [m31_column(60 + k, eval_log).astype(np.int64) for k in range(4)]
    rc = np.stack([seeded_qm31(70 + k) for k in range(air.n_constraints)])
    got = air_composition(air, {1: cols}, eval_log, trace_log, {}, rc)
    x = {o: cols[0][O.offset_rows(o, trace_log, eval_log)] for o in (-3, -1, 1, 2)}
    cs = [(cols[1] - x[2]) % O.P, (cols[2] - x[-3]) % O.P, (cols[3] - x[-1] * x[1] - cols[0]) % O.P]
    acc = np.zeros((1 << eval_log, 4), np.int64)
    for k, c in enumerate(cs):
        acc = (acc + np.asarray(rc[k], np.int64)[None, :] * c[:, None]) % O.P
    den = O.vanishing_inverses(eval_log, trace_log).astype(np.int64)
    want = acc * den[:, None] % O.P
    assert all(np.array_equal(np.asarray(got[i], np.int64), want[:, i]) for i in range(4))
