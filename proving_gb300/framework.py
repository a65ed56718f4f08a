"""The generic constraint path: AIR constraints written against an evaluator
like the reference's ExprEvaluator (crates/constraint-framework/src/expr/
evaluator.rs:58-123, expressions in crates/constraint-framework/src/expr/mod.rs),
turned into the source of one CUDA kernel and compiled at run time with NVRTC
(libstwo_cuda.so: cs_rtc_compile_air / cs_rtc_air_composition).

An AIR is a function `evaluate(e)` that reads masks and adds constraints:

    def wide_fib(e, n_cols):
        a, b = e.next_trace_mask(), e.next_trace_mask()
        for _ in range(n_cols - 2):
            c = e.next_trace_mask()
            e.add_constraint(c - (a * a + b * b))
            a, b = b, c

Masks are M31 values of a trace or interaction column at a row offset (0: the
row, -1: the previous row of the trace domain). `e.secure(m0, m1, m2, m3)` is
SecureField::from_partial_evals of four base values (a QM31 interaction column
by its coordinates), `e.param(name)` a QM31 parameter fixed per launch (lookup
elements, claimed sums). Constraints may be M31 or QM31; the kernel adds
sum_k rc[k] C_k(row) / V_trace(row) to the accumulator, like
evaluate_constraint_quotients_on_domain (crates/constraint-framework/src/
prover/component_prover.rs:111-193).
"""
from __future__ import annotations

import ctypes
import hashlib
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

P = (1 << 31) - 1
CSRC = Path(__file__).resolve().parent / "csrc"


# ------------------------------------------------------------------ expressions

class Expr:
    """A node of the constraint DAG; `ext` marks QM31 values (else M31)."""
    __slots__ = ("op", "args", "ext", "key")

    def __init__(self, op: str, args: tuple, ext: bool):
        self.op, self.args, self.ext = op, args, ext
        self.key = (op,) + tuple(a.key if isinstance(a, Expr) else a for a in args)

    def _bin(self, op, other, swap=False):
        other = _lift(other)
        a, b = (other, self) if swap else (self, other)
        return Expr(op, (a, b), a.ext or b.ext)

    def __add__(self, o):
        return self._bin("add", o)

    def __radd__(self, o):
        return self._bin("add", o, True)

    def __sub__(self, o):
        return self._bin("sub", o)

    def __rsub__(self, o):
        return self._bin("sub", o, True)

    def __mul__(self, o):
        return self._bin("mul", o)

    def __rmul__(self, o):
        return self._bin("mul", o, True)

    def __neg__(self):
        return Expr("neg", (self,), self.ext)

    def __pow__(self, k: int):
        """x^k by squaring (k >= 1)."""
        assert isinstance(k, int) and k >= 1
        result, base = None, self
        while k:
            if k & 1:
                result = base if result is None else result * base
            k >>= 1
            if k:
                base = base * base
        return result


def _lift(x) -> Expr:
    if isinstance(x, Expr):
        return x
    if isinstance(x, int):
        return Expr("const", (x % P,), False)
    raise TypeError(f"not an expression: {x!r}")


@dataclass
class Mask:
    interaction: int
    column: int
    offset: int


class Evaluator:
    """Records an AIR's masks and constraints (the ExprEvaluator role). Columns are numbered per
    interaction (tree) in the order their masks are first taken, as next_trace_mask /
    next_interaction_mask number them (crates/constraint-framework/src/lib.rs:61-90)."""

    def __init__(self):
        self.columns: dict[int, int] = {}    # interaction -> columns taken so far
        self.params: list[str] = []
        self.constraints: list[Expr] = []

    def _mask(self, interaction: int, column: int, offset: int) -> Expr:
        if offset not in (0, -1):
            raise NotImplementedError("mask offsets 0 and -1 (the previous row)")
        return Expr("mask", (interaction, column, offset), False)

    def next_interaction_mask(self, interaction: int, offsets=(0,)):
        col = self.columns.get(interaction, 0)
        self.columns[interaction] = col + 1
        return [self._mask(interaction, col, off) for off in offsets]

    def next_trace_mask(self) -> Expr:
        return self.next_interaction_mask(1)[0]

    def secure(self, b0, b1, b2, b3) -> Expr:
        """SecureField::from_partial_evals of four M31 values."""
        parts = tuple(_lift(b) for b in (b0, b1, b2, b3))
        assert not any(p.ext for p in parts)
        return Expr("secure", parts, True)

    def param(self, name: str) -> Expr:
        if name not in self.params:
            self.params.append(name)
        return Expr("param", (name,), True)

    def add_constraint(self, c) -> None:
        self.constraints.append(_lift(c))


# ------------------------------------------------------------------ code generation

_PRELUDE = """typedef unsigned int uint32_t;
typedef unsigned long long uint64_t;
#include "field.cuh"
#include "rows.cuh"
using namespace cs;
"""


def _header(name: str) -> str:
    """A library header for NVRTC: its own fixed-width types come from the prelude."""
    return (CSRC / name).read_text().replace("#include <cstdint>\n", "")


@dataclass
class Air:
    """An AIR recorded by an Evaluator: its masks, parameters, constraints and kernel source."""
    name: str
    masks: list
    params: list
    constraints: list
    source: str = field(repr=False)

    @property
    def n_constraints(self) -> int:
        return len(self.constraints)

    def mask_columns(self, columns_by_interaction) -> list:
        """The device columns of the kernel's column table, in mask order: columns_by_interaction
        maps an interaction to its list of columns (evaluation-domain BaseColumns)."""
        return [columns_by_interaction[m.interaction][m.column] for m in self.masks]


def compile_air(name: str, evaluate, *args) -> Air:
    """Records `evaluate(e, *args)` and generates the kernel source."""
    e = Evaluator()
    evaluate(e, *args)
    # distinct masks in first-use order over the constraints
    order, slot = [], {}
    temps, lines = {}, []

    def visit(x: Expr) -> str:
        if x.key in temps:
            return temps[x.key]
        if x.op == "mask":
            k = x.args
            if k not in slot:
                slot[k] = len(order)
                order.append(Mask(*k))
            i = slot[k]
            row = "r" if k[2] == 0 else "pr"
            name = f"m{len(temps)}"
            lines.append(f"  const uint32_t {name} = __ldg(cols[{i}] + {row});")
        elif x.op == "const":
            name = f"k{len(temps)}"
            lines.append(f"  const uint32_t {name} = {x.args[0]}u;")
        elif x.op == "param":
            j = e.params.index(x.args[0])
            name = f"q{len(temps)}"
            lines.append(f"  const qm31 {name} = qm31_make(params[{4 * j}], params[{4 * j + 1}], "
                         f"params[{4 * j + 2}], params[{4 * j + 3}]);")
        elif x.op == "secure":
            parts = [visit(a) for a in x.args]
            name = f"s{len(temps)}"
            lines.append(f"  const qm31 {name} = qm31_make({', '.join(parts)});")
        else:
            ops = [visit(a) for a in x.args]
            name = f"t{len(temps)}"
            ty = "qm31" if x.ext else "uint32_t"
            if x.op == "neg":
                rhs = f"qm31_neg({ops[0]})" if x.ext else f"m31_neg({ops[0]})"
            else:
                a, b = x.args
                fn = {"add": "add", "sub": "sub", "mul": "mul"}[x.op]
                if not x.ext:
                    rhs = f"m31_{fn}({ops[0]}, {ops[1]})"
                elif a.ext and b.ext:
                    rhs = f"qm31_{fn}({ops[0]}, {ops[1]})"
                elif fn == "mul":  # one side M31
                    q, m = (ops[0], ops[1]) if a.ext else (ops[1], ops[0])
                    rhs = f"qm31_mul_m31({q}, {m})"
                else:
                    qa = ops[0] if a.ext else f"qm31_make({ops[0]}, 0, 0, 0)"
                    qb = ops[1] if b.ext else f"qm31_make({ops[1]}, 0, 0, 0)"
                    rhs = f"qm31_{fn}({qa}, {qb})"
            lines.append(f"  const {ty} {name} = {rhs};")
        temps[x.key] = name
        return name

    body = []
    for k, c in enumerate(e.constraints):
        v = visit(c)
        body.extend(lines)
        lines.clear()
        w = f"qm31_make(rc[{4 * k}], rc[{4 * k + 1}], rc[{4 * k + 2}], rc[{4 * k + 3}])"
        body.append(f"  acc = qm31_add(acc, {'qm31_mul' if c.ext else 'qm31_mul_m31'}({w}, {v}));")
    src = _PRELUDE + f"""
// AIR {name}: {len(order)} masks, {len(e.constraints)} constraints, {len(e.params)} parameters
extern "C" __global__ void __launch_bounds__(256) cs_air_composition(
    const uint32_t* const* __restrict__ cols, const uint32_t* __restrict__ rc, const uint32_t* __restrict__ params,
    const uint32_t* __restrict__ den, uint32_t eval_log, uint32_t trace_log,
    uint32_t* a0, uint32_t* a1, uint32_t* a2, uint32_t* a3) {{
  const uint32_t n = 1u << eval_log;
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {{
    const uint32_t pr = prev_row(r, trace_log, eval_log);
    (void)pr;
    qm31 acc = qm31_make(0, 0, 0, 0);
{chr(10).join('  ' + l for l in body)}
    const qm31 v = qm31_mul_m31(acc, den[r >> trace_log]);
    a0[r] = m31_add(a0[r], v.a.a);
    a1[r] = m31_add(a1[r], v.a.b);
    a2[r] = m31_add(a2[r], v.b.a);
    a3[r] = m31_add(a3[r], v.b.b);
  }}
}}
"""
    return Air(name, order, list(e.params), list(e.constraints), src)


# ------------------------------------------------------------------ device side

class CompiledAir:
    """An Air compiled for the device (cs_rtc_compile_air); compositions run through
    cs_rtc_air_composition."""

    _cache: dict = {}

    def __init__(self, air: Air):
        from . import _lib
        self.air = air
        names = ["field.cuh", "rows.cuh"]
        srcs = [_header(n).encode() for n in names]
        hs = (ctypes.c_char_p * len(srcs))(*srcs)
        hn = (ctypes.c_char_p * len(names))(*[n.encode() for n in names])
        handle = ctypes.c_void_p()
        log = ctypes.create_string_buffer(4096)
        _lib.call("cs_rtc_compile_air", air.source.encode(), len(names), hs, hn, len(air.masks),
                  air.n_constraints, len(air.params), ctypes.byref(handle), log, len(log))
        self.handle = handle

    @classmethod
    def get(cls, air: Air) -> "CompiledAir":
        """One compiled kernel per distinct source (kept for the process's lifetime)."""
        key = hashlib.sha256(air.source.encode()).hexdigest()
        if key not in cls._cache:
            cls._cache[key] = cls(air)
        return cls._cache[key]

    def composition(self, columns_by_interaction, trace_log: int, params, rc, accum) -> None:
        """Adds the AIR's constraint quotients over accum's domain (the evaluation domain of the
        columns). params: {name: QM31}; rc: one QM31 weight per constraint."""
        from . import _lib
        from .backend import _ptr_table, _stream
        cols = self.air.mask_columns(columns_by_interaction)
        # the kernel reads every mask column at rows below len(accum): the columns must be that long
        if any(len(c) != len(accum) for c in cols):
            raise ValueError("mask columns must be evaluations on the accumulator's domain")
        rcw = np.ascontiguousarray(np.asarray(rc, np.uint32).reshape(-1))
        assert rcw.size == 4 * self.air.n_constraints
        pw = np.ascontiguousarray(np.asarray([params[p] for p in self.air.params], np.uint32).reshape(-1))
        _lib.call("cs_rtc_air_composition", self.handle, _ptr_table([c.data for c in cols]),
                  rcw.ctypes.data, pw.ctypes.data if pw.size else None, len(accum).bit_length() - 1, trace_log,
                  _ptr_table([c.data for c in accum.columns]), _stream())


# ------------------------------------------------------------------ AIRs

def wide_fib_air(e: Evaluator, n_cols: int) -> None:
    """WideFibonacciEval::evaluate (crates/examples/src/wide_fibonacci/mod.rs:87-97)."""
    a, b = e.next_trace_mask(), e.next_trace_mask()
    for _ in range(n_cols - 2):
        c = e.next_trace_mask()
        e.add_constraint(c - (a * a + b * b))
        a, b = b, c


def single_lookup_air(e: Evaluator) -> None:
    """A single-column LogUp component: relation entry (multiplicity -1, values [v]) finalized
    with finalize_logup (crates/constraint-framework/src/logup.rs:95-150): with the interaction
    column's running sum at the row (cur) and at the previous row (prev) and shift = claimed sum /
    2^n, (cur - prev + shift) (v - z) + 1 = 0."""
    v = e.next_trace_mask()
    coords = [e.next_interaction_mask(2, (-1, 0)) for _ in range(4)]
    prev = e.secure(*[c[0] for c in coords])
    cur = e.secure(*[c[1] for c in coords])
    z, shift = e.param("z"), e.param("shift")
    e.add_constraint((cur - prev + shift) * (v - z) + 1)
