"""ORACLE — test infrastructure only: the constraint DAG of proving_gb300.framework evaluated on
the CPU with numpy, row by row over an evaluation domain, as the reference's CPU constraint
evaluation does (crates/constraint-framework/src/prover/component_prover.rs:195-268 with
cpu_domain.rs): masks at the row and at rows a trace step offset away (orc_offset_row), each constraint times
its weight, summed, over V_trace(row), added to the accumulator. Field arithmetic is written
here on int64 arrays, independently of the prover's."""
from __future__ import annotations

import numpy as np

from . import oracle as O

P = O.P


def _m(x):
    return np.asarray(x, np.int64) % P


def _qmul(x, y):
    """QM31 product of (n, 4) arrays: (a + b u)(c + d u) = ac + (2 + i) bd + (ad + bc) u."""
    def cm(p0, p1, q0, q1):
        return (p0 * q0 - p1 * q1) % P, (p0 * q1 + p1 * q0) % P
    ac = cm(x[:, 0], x[:, 1], y[:, 0], y[:, 1])
    bd = cm(x[:, 2], x[:, 3], y[:, 2], y[:, 3])
    ad = cm(x[:, 0], x[:, 1], y[:, 2], y[:, 3])
    bc = cm(x[:, 2], x[:, 3], y[:, 0], y[:, 1])
    rbd = ((2 * bd[0] - bd[1]) % P, (bd[0] + 2 * bd[1]) % P)
    return np.stack([(ac[0] + rbd[0]) % P, (ac[1] + rbd[1]) % P, (ad[0] + bc[0]) % P, (ad[1] + bc[1]) % P], 1)


def _as_q(v, n):
    if v.ndim == 2:
        return v
    q = np.zeros((n, 4), np.int64)
    q[:, 0] = v
    return q


def _evaluator(columns_by_interaction, rows, params, n):
    """Row-wise evaluation of expression nodes over n rows: masks read their column at the rows of
    their offset (rows[offset]), values are int64 arrays, QM31 as (n, 4)."""
    memo = {}

    def ev(x):
        if x.key in memo:
            return memo[x.key]
        if x.op == "mask":
            inter, col, off = x.args
            v = np.asarray(columns_by_interaction[inter][col], np.int64)[rows[off]]
        elif x.op == "const":
            v = np.full(n, x.args[0], np.int64)
        elif x.op == "param":
            v = np.tile(np.asarray(params[x.args[0]], np.int64) % P, (n, 1))
        elif x.op == "secure":
            v = np.stack([ev(a) for a in x.args], 1)
        elif x.op == "neg":
            v = (-ev(x.args[0])) % P
        else:
            a, b = ev(x.args[0]), ev(x.args[1])
            if x.ext:
                if x.op == "mul" and not x.args[0].ext:    # M31 times QM31
                    v = b * a[:, None] % P
                elif x.op == "mul" and not x.args[1].ext:  # QM31 times M31
                    v = a * b[:, None] % P
                else:
                    a, b = _as_q(a, n), _as_q(b, n)
                    v = {"add": (a + b) % P, "sub": (a - b) % P, "mul": None}[x.op]
                    if v is None:
                        v = _qmul(a, b)
            else:
                v = {"add": (a + b) % P, "sub": (a - b) % P, "mul": (a * b) % P}[x.op]
        memo[x.key] = v
        return v

    return ev


def air_composition(air, columns_by_interaction, eval_log: int, trace_log: int, params, rc, out=None,
                    divide: bool = True, log_expansion: int = 0):
    """The accumulator (4 coordinate arrays, created when None) plus the AIR's quotients. With
    divide=False the weighted constraint sums are not divided by V_trace (on the trace domain itself,
    where V_trace is zero, they show whether every row satisfies the constraints). With
    log_expansion e the columns are committed on CanonicCoset(eval_log + e) and the rows are their
    first 2^eval_log, that domain's subdomain (component_prover.rs:36-48, 234-238)."""
    n = 1 << eval_log
    rows = {0: np.arange(n)}
    for m in air.masks:
        if m.offset not in rows:
            rows[m.offset] = O.offset_rows(m.offset, trace_log, eval_log)
    ev = _evaluator(columns_by_interaction, rows, params, n)
    acc = np.zeros((n, 4), np.int64)
    for c, w in zip(air.constraints, np.asarray(rc, np.int64).reshape(-1, 4)):
        v = _as_q(ev(c), n)
        acc = (acc + _qmul(v, np.tile(w % P, (n, 1)))) % P
    if divide:
        den = O.vanishing_inverses(eval_log, trace_log, log_expansion)
        acc = acc * den[:, None] % P
    if out is None:
        out = [np.zeros(n, np.uint32) for _ in range(4)]
    return [((np.asarray(o, np.int64) + acc[:, k]) % P).astype(np.uint32) for k, o in enumerate(out)]


def air_fractions(air, columns_by_interaction, log_n: int, params):
    """Each LogUp batch's combined (numerator, denominator) at every row of the trace domain, as
    4 coordinate arrays each: the values the interaction columns are generated from (the trace
    domain's coset-order neighbours for offset masks)."""
    n = 1 << log_n
    rows = {0: np.arange(n)}
    for num, den in air.logup:
        for root in (num, den):
            stack = [root]
            while stack:
                x = stack.pop()
                if x.op == "mask" and x.args[2] not in rows:
                    rows[x.args[2]] = O.offset_rows(x.args[2], log_n, log_n)
                stack.extend(a for a in x.args if hasattr(a, "key"))
    ev = _evaluator(columns_by_interaction, rows, params, n)
    out = []
    for num, den in air.logup:
        out.append(tuple([_as_q(ev(x), n)[:, k].astype(np.uint32) for k in range(4)] for x in (num, den)))
    return out
