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
row, -1: the previous row of the trace domain, any other integer that many
trace steps away). `e.secure(m0, m1, m2, m3)` is
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

_NODE_IDS: dict = {}  # (op, child keys / literal args) -> key: equal expressions share one key


class Expr:
    """A node of the constraint DAG; `ext` marks QM31 values (else M31). `key` is an integer shared
    by structurally equal expressions (hash-consing over the children's keys), so keys hash in
    constant time however large the expression tree under a node grows (Poseidon2's partial rounds
    fold every state word into every other, round after round)."""
    __slots__ = ("op", "args", "ext", "key")

    def __init__(self, op: str, args: tuple, ext: bool):
        self.op, self.args, self.ext = op, args, ext
        k = (op,) + tuple(a.key if isinstance(a, Expr) else a for a in args)
        self.key = _NODE_IDS.setdefault(k, len(_NODE_IDS))

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
        self.mask_offsets: dict[int, list] = {}  # interaction -> the offsets of each column taken
        self.preprocessed: list[str] = []        # the preprocessed columns read, by name
        self.params: list[str] = []
        self.constraints: list[Expr] = []
        self.fracs: list[tuple[Expr, Expr]] = []  # LogUp fractions (numerator, denominator) of the row
        self.logup: list = []  # every finalized batch's combined (numerator, denominator), in column order
        self.relations: list[str] = []  # the relations add_to_relation names, in first-use order

    def _mask(self, interaction: int, column: int, offset: int) -> Expr:
        """A column at the row `offset` trace steps away (0 the row itself, -1 the previous row)."""
        if not isinstance(offset, int) or not -(1 << 30) <= offset < (1 << 30):
            raise ValueError(f"a mask offset is an integer of 31 bits or fewer: {offset!r}")
        return Expr("mask", (interaction, column, offset), False)

    def next_interaction_mask(self, interaction: int, offsets=(0,)):
        if interaction < 1:
            raise ValueError("the preprocessed tree is read with get_preprocessed_column")
        col = self.columns.get(interaction, 0)
        self.columns[interaction] = col + 1
        masks = [self._mask(interaction, col, off) for off in offsets]
        self.mask_offsets.setdefault(interaction, []).append(tuple(offsets))
        return masks

    def get_preprocessed_column(self, name: str) -> Expr:
        """EvalAtRow::get_preprocessed_column: a column of the preprocessed tree (interaction 0)
        at the row, named by its id; the component maps the name to its column in that tree."""
        if name not in self.preprocessed:
            self.preprocessed.append(name)
        return self._mask(0, self.preprocessed.index(name), 0)

    def next_trace_mask(self) -> Expr:
        return self.next_interaction_mask(1)[0]

    def next_extension_interaction_mask(self, interaction: int, offsets=(0,)) -> list:
        """EvalAtRow::next_extension_interaction_mask: the next four columns of `interaction` (a QM31
        column by its coordinates) at each offset, combined per offset (combine_ef)."""
        cols = [self.next_interaction_mask(interaction, offsets) for _ in range(4)]
        return [self.secure(*[c[k] for c in cols]) for k in range(len(offsets))]

    def add_to_relation(self, relation: str, multiplicity, values) -> None:
        """EvalAtRow::add_to_relation (crates/constraint-framework/src/lib.rs:145-151): the fraction
        multiplicity / combine(values) joins the row's LogUp sum, with LookupElements::combine
        (crates/constraint-framework/src/logup.rs:80-94) = sum_i alpha^i values[i] - z; z and the
        alpha powers are the parameters `{relation}_z` and `{relation}_alpha{i}`."""
        den = None
        for i, v in enumerate(values):
            term = self.param(f"{relation}_alpha{i}") * _lift(v)
            den = term if den is None else den + term
        den = den - self.param(f"{relation}_z")
        self.fracs.append((_lift(multiplicity), den))
        if relation not in self.relations:
            self.relations.append(relation)

    def finalize_logup_batched(self, batch_size: int, interaction: int = 2, shift: str = "shift") -> None:
        """finalize_logup_batched (the logup_proxy macro, crates/constraint-framework/src/lib.rs:
        185-221): the row's fractions summed in consecutive batches of batch_size (a/b + c/d =
        (ad + cb)/(bd)); every batch but the last has a cumulative-sum column of `interaction`
        (the constraint (cur - previous column) den - num = 0), and the last one the running sum's
        column read at the previous row too: (cur - prev_row - previous column + shift) den - num
        = 0, with shift = claimed sum / 2^log_size (the parameter `shift`)."""
        assert self.fracs and batch_size > 0, "no LogUp fractions to finalize"
        batches = []
        for i in range(0, len(self.fracs), batch_size):
            num, den = self.fracs[i]
            for n2, d2 in self.fracs[i + 1:i + batch_size]:
                num, den = num * d2 + n2 * den, den * d2
            batches.append((num, den))
        self.fracs = []
        self.logup.extend(batches)
        last_num, last_den = batches.pop()
        prev_col = None
        for num, den in batches:
            [cur] = self.next_extension_interaction_mask(interaction, (0,))
            diff = cur if prev_col is None else cur - prev_col
            prev_col = cur
            self.add_constraint(diff * den - num)
        prev_row, cur = self.next_extension_interaction_mask(interaction, (-1, 0))
        diff = cur - prev_row if prev_col is None else cur - prev_row - prev_col
        self.add_constraint((diff + self.param(shift)) * last_den - last_num)

    def finalize_logup(self, **kw) -> None:
        """finalize_logup: no batching (lib.rs:224-226)."""
        self.finalize_logup_batched(1, **kw)

    def finalize_logup_in_pairs(self, **kw) -> None:
        """finalize_logup_in_pairs: batches of two (lib.rs:230-232)."""
        self.finalize_logup_batched(2, **kw)

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
typedef int int32_t;
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
    # interaction -> the offsets of every column the AIR takes, in order, whether or not a
    # constraint reads it (InfoEvaluator's mask_offsets, crates/constraint-framework/src/info.rs)
    mask_offsets: dict = field(default_factory=dict, repr=False)
    preprocessed: list = field(default_factory=list)  # preprocessed column ids, interaction 0 order
    # the LogUp batches' combined fractions (numerator, denominator), one per interaction column
    # of finalize_logup_batched, and the trace masks their kernel (cs_air_fractions) reads
    logup: list = field(default_factory=list, repr=False)
    fraction_masks: list = field(default_factory=list, repr=False)
    relations: list = field(default_factory=list)

    @property
    def n_constraints(self) -> int:
        return len(self.constraints)

    def point_program(self):
        """The constraints at a point as the node program of cs_prove_air, for an AIR that reads
        trace columns (interaction 1) and the interaction columns of its relations (interaction 2,
        each at the row, or at the previous row and the row): nodes of 5 words (op, a0..a3) in
        topological order; op 0 is the sampled value of column a0 of tree a2 at its a1-th sample, 1
        the constant a0, 2 parameter a0, 3 from_partial_evals of nodes a0..a3, 4 -a0, 5 a0 + a1,
        6 a0 - a1, 7 a0 * a1. Returns (nodes (n, 5) uint32, each constraint's node, each trace
        column's offsets, each mask's (column, tree), each interaction column's "also at the
        previous row" flag); computed once per Air."""
        cached = self.__dict__.get("_point_program")
        if cached is not None:
            return cached
        if set(self.mask_offsets) - {1, 2} or self.preprocessed:
            raise NotImplementedError("a node program for AIRs that read trace and interaction columns")
        offs = [list(o) for o in self.mask_offsets.get(1, [])]
        inter = [list(o) for o in self.mask_offsets.get(2, [])]
        if any(o not in ([0], [-1, 0]) for o in inter):
            raise NotImplementedError("interaction columns read at the row, or at the previous row and the row")
        tree_offs = {1: offs, 2: inter}
        ids, prog = {}, []
        codes = {"neg": 4, "add": 5, "sub": 6, "mul": 7}
        for root in self.constraints:
            stack = [root]
            while stack:
                x = stack[-1]
                if x.key in ids:
                    stack.pop()
                    continue
                todo = [a for a in x.args if isinstance(a, Expr) and a.key not in ids]
                if todo:
                    stack.extend(todo)
                    continue
                stack.pop()
                if x.op == "mask":
                    tree, col, off = x.args
                    row = [0, col, tree_offs[tree][col].index(off), tree, 0]
                elif x.op == "const":
                    row = [1, x.args[0] % P, 0, 0, 0]
                elif x.op == "param":
                    row = [2, self.params.index(x.args[0]), 0, 0, 0]
                elif x.op == "secure":
                    row = [3] + [ids[a.key] for a in x.args]
                else:
                    kids = [ids[a.key] for a in x.args]
                    row = [codes[x.op]] + kids + [0] * (4 - len(kids))
                ids[x.key] = len(prog)
                prog.append(row)
        nodes = np.asarray(prog, np.uint32).reshape(-1, 5)
        out = (nodes, [ids[c.key] for c in self.constraints], offs, [(m.column, m.interaction) for m in self.masks],
               [len(o) == 2 for o in inter])
        self.__dict__["_point_program"] = out
        return out

    def mask_columns(self, columns_by_interaction) -> list:
        """The device columns of the kernel's column table, in mask order: columns_by_interaction
        maps an interaction to its list of columns (evaluation-domain BaseColumns)."""
        return [columns_by_interaction[m.interaction][m.column] for m in self.masks]


# Operations a split body calls through non-inlined wrappers, name -> (result type, parameters),
# e.g. {"qm31_mul": ("qm31", "qm31 a, qm31 b")}: the device compiler then has less code to
# optimize, at a cost in run time. Empty: everything is inlined. For the 1,144 constraints of
# Poseidon2 at 2^18 rows the proof takes 28.9 ms inlined (30 s to compile on the Grace host)
# against 34.1 ms with M31 products and QM31 operations wrapped (22 s).
_SPLIT_OPS: dict = {}
_SINGLE_LINES = 1500  # bodies up to this many lines stay one function
_CHUNK_NODES = 300    # computed nodes per function of a split body
_LEAVES = ("mask", "const", "param")


def _chunks(constraints, budget: int):
    """Splits the constraints, in order, into chunks of about `budget` computed nodes (any node but
    a mask, constant or parameter). A node belongs to the first chunk that reaches it; a later
    chunk that needs it reads it back instead of recomputing it. Returns (chunks of constraint
    indices, owner chunk of each computed node's key, keys of the nodes read by a later chunk)."""
    owner, exported, chunks, size = {}, set(), [[]], 0
    for k, c in enumerate(constraints):
        if size >= budget and chunks[-1]:
            chunks.append([])
            size = 0
        ch = len(chunks) - 1
        stack, seen = [c], set()
        while stack:
            x = stack.pop()
            if x.key in seen or x.op in _LEAVES:
                continue
            seen.add(x.key)
            o = owner.get(x.key)
            if o is not None:
                if o != ch:
                    exported.add(x.key)
                continue
            owner[x.key] = ch
            size += 1
            stack.extend(a for a in x.args if isinstance(a, Expr))
        chunks[-1].append(k)
    return chunks, owner, exported


def compile_air(name: str, evaluate, *args) -> Air:
    """Records `evaluate(e, *args)` and generates the kernel source."""
    e = Evaluator()
    evaluate(e, *args)
    # distinct masks in first-use order over the constraints
    order, slot = [], {}
    temps, lines = {}, []
    offsets = set()  # the mask offsets other than 0

    def row_name(o: int) -> str:
        return "r" if o == 0 else "pr" if o == -1 else f"ro_{'m' if o < 0 else 'p'}{abs(o)}"

    split = {"chunk": None, "owner": {}, "slot": {}}  # set while emitting a split body

    def op_name(fn: str) -> str:
        """The name a split body calls an operation by: its non-inlined wrapper when _SPLIT_OPS
        lists it (the kernel's sum of the functions too), else the operation itself."""
        return f"air_{fn}" if split["chunk"] is not None and fn in _SPLIT_OPS else fn

    def visit(x: Expr) -> str:
        if x.key in temps:
            return temps[x.key]
        ch = split["chunk"]
        if ch is not None and x.op not in _LEAVES and split["owner"][x.key] < ch:
            # computed by an earlier function of a split body: read back from xs
            o = split["slot"][x.key]
            name = f"x{len(temps)}"
            if x.ext:
                lines.append(f"  const qm31 {name} = qm31_make(xs[{o}], xs[{o + 1}], xs[{o + 2}], xs[{o + 3}]);")
            else:
                lines.append(f"  const uint32_t {name} = xs[{o}];")
            temps[x.key] = name
            return name
        if x.op == "mask":
            k = x.args
            if k not in slot:
                slot[k] = len(order)
                order.append(Mask(*k))
            i = slot[k]
            row = row_name(k[2])
            if k[2]:
                offsets.add(k[2])
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
                    rhs = f"{op_name('m31_' + fn)}({ops[0]}, {ops[1]})"
                elif a.ext and b.ext:
                    rhs = f"{op_name('qm31_' + fn)}({ops[0]}, {ops[1]})"
                elif fn == "mul":  # one side M31
                    q, m = (ops[0], ops[1]) if a.ext else (ops[1], ops[0])
                    rhs = f"{op_name('qm31_mul_m31')}({q}, {m})"
                else:
                    qa = ops[0] if a.ext else f"qm31_make({ops[0]}, 0, 0, 0)"
                    qb = ops[1] if b.ext else f"qm31_make({ops[1]}, 0, 0, 0)"
                    rhs = f"{op_name('qm31_' + fn)}({qa}, {qb})"
            lines.append(f"  const {ty} {name} = {rhs};")
        temps[x.key] = name
        return name

    def emit(ks) -> list:
        """The lines that add constraints ks (indices) to acc, sharing the current temps. An M31
        constraint's weighted value goes unreduced into four 64-bit sums, one multiply-add per
        coordinate (products below 2^62, the sums folded below 2^34 every three terms); the sums
        are reduced and added to acc once, at the end of the lines."""
        body = ["  uint64_t lz0 = 0, lz1 = 0, lz2 = 0, lz3 = 0;"]
        pending = 0
        for k in ks:
            c = e.constraints[k]
            v = visit(c)
            body.extend(lines)
            lines.clear()
            if c.ext:
                w = f"qm31_make(rc[{4 * k}], rc[{4 * k + 1}], rc[{4 * k + 2}], rc[{4 * k + 3}])"
                body.append(f"  acc = {op_name('qm31_add')}(acc, {op_name('qm31_mul')}({w}, {v}));")
                continue
            if pending == 3:
                body.append("  lz0 = (lz0 & P) + (lz0 >> 31); lz1 = (lz1 & P) + (lz1 >> 31); "
                            "lz2 = (lz2 & P) + (lz2 >> 31); lz3 = (lz3 & P) + (lz3 >> 31);")
                pending = 0
            body.append(f"  lz0 += (uint64_t)rc[{4 * k}] * {v}; lz1 += (uint64_t)rc[{4 * k + 1}] * {v}; "
                        f"lz2 += (uint64_t)rc[{4 * k + 2}] * {v}; lz3 += (uint64_t)rc[{4 * k + 3}] * {v};")
            pending += 1
        body.append(f"  acc = {op_name('qm31_add')}(acc, qm31_make(m31_reduce64(lz0), m31_reduce64(lz1), "
                    "m31_reduce64(lz2), m31_reduce64(lz3)));")
        return body

    # One straight-line body when it is small. The device compiler's optimizer takes time
    # superlinear in the size of one function (Poseidon2's 1,144 constraints in one body did not
    # compile in ten minutes, one instance's 143 took over a minute), so a large AIR is split, in
    # constraint order, into non-inlined device functions of about _CHUNK_NODES computed nodes; a
    # value one function computes and a later one needs passes through the thread's array xs.
    funcs, calls, xs_words = "", "", 0
    body = emit(range(len(e.constraints)))
    # one row index per mask offset in use, computed once per row
    row_params = "".join(f", uint32_t {row_name(o)}" for o in sorted(offsets))
    row_args = "".join(f", {row_name(o)}" for o in sorted(offsets))
    row_defs = "".join(
        f"    const uint32_t {row_name(o)} = "
        + ("prev_row(r, trace_log, eval_log);\n" if o == -1 else f"offset_row(r, {o}, trace_log, eval_log);\n")
        for o in sorted(offsets))
    if len(body) <= _SINGLE_LINES:
        inline = chr(10).join('  ' + l for l in body)
    else:
        chunks, owner, exported = _chunks(e.constraints, _CHUNK_NODES)
        nodes = {}

        def collect(x):
            stack = [x]
            while stack:
                y = stack.pop()
                if y.key in nodes:
                    continue
                nodes[y.key] = y
                stack.extend(a for a in y.args if isinstance(a, Expr))
        for c in e.constraints:
            collect(c)
        xslot = {}
        for key in sorted(exported, key=lambda kk: owner[kk]):
            xslot[key] = xs_words
            xs_words += 4 if nodes[key].ext else 1
        split.update(owner=owner, slot=xslot)
        for g, ks in enumerate(chunks):
            temps.clear()
            split["chunk"] = g
            lines_g = emit(ks)
            for key in [kk for kk in exported if owner[kk] == g]:
                o, t = xslot[key], temps[key]
                if nodes[key].ext:
                    lines_g.append(f"  xs[{o}] = {t}.a.a; xs[{o + 1}] = {t}.a.b; xs[{o + 2}] = {t}.b.a; "
                                   f"xs[{o + 3}] = {t}.b.b;")
                else:
                    lines_g.append(f"  xs[{o}] = {t};")
            funcs += f"""
__device__ __noinline__ qm31 cs_air_group{g}(const uint32_t* const* __restrict__ cols,
                                            const uint32_t* __restrict__ rc,
                                            const uint32_t* __restrict__ params, uint32_t r{row_params},
                                            uint32_t* xs) {{
  (void)params;
  (void)xs;
  qm31 acc = qm31_make(0, 0, 0, 0);
{chr(10).join(lines_g)}
  return acc;
}}
"""
            add = "air_qm31_add" if "qm31_add" in _SPLIT_OPS else "qm31_add"
            calls += f"    acc = {add}(acc, cs_air_group{g}(cols, rc, params, r{row_args}, xs));\n"
        split["chunk"] = None
        inline = f"    uint32_t xs[{max(xs_words, 1)}];\n" + calls.rstrip("\n")
        funcs = "".join(f"__device__ __noinline__ {ty} air_{fn}({args}) {{ return {fn}(a, b); }}\n"
                        for fn, (ty, args) in _SPLIT_OPS.items()) + funcs
    src = _PRELUDE + funcs + f"""
// AIR {name}: {len(order)} masks, {len(e.constraints)} constraints, {len(e.params)} parameters
extern "C" __global__ void __launch_bounds__(256) cs_air_composition(
    const uint32_t* const* __restrict__ cols, const uint32_t* __restrict__ rc, const uint32_t* __restrict__ params,
    const uint32_t* __restrict__ den, uint32_t eval_log, uint32_t trace_log,
    uint32_t* a0, uint32_t* a1, uint32_t* a2, uint32_t* a3) {{
  const uint32_t n = 1u << eval_log;
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {{
{row_defs}    qm31 acc = qm31_make(0, 0, 0, 0);
{inline}
    const qm31 v = qm31_mul_m31(acc, den[r >> trace_log]);
    a0[r] = m31_add(a0[r], v.a.a);
    a1[r] = m31_add(a1[r], v.a.b);
    a2[r] = m31_add(a2[r], v.b.a);
    a3[r] = m31_add(a3[r], v.b.b);
  }}
}}
"""
    frac_masks = []
    if e.logup:
        frac_src, frac_masks = _fraction_source(e)
        src += frac_src
    return Air(name, order, list(e.params), list(e.constraints), src,
               {k: list(v) for k, v in sorted(e.mask_offsets.items())}, list(e.preprocessed), list(e.logup),
               frac_masks, list(e.relations))


def _fraction_source(e: Evaluator):
    """The kernel cs_air_fractions: at every row of the trace domain, each LogUp batch's combined
    numerator and denominator (QM31) into out[8 j .. 8 j + 3] and out[8 j + 4 .. 8 j + 7], the
    values LogupTraceGenerator's columns are written from (crates/constraint-framework/src/prover/
    logup.rs:22-130). Reads trace masks only (cols[i]: the column of fraction mask i on the trace
    domain, at its row offset in coset order). Returns (source, the masks in table order)."""
    masks, slot, temps, lines, offsets = [], {}, {}, [], set()

    def row_name(o: int) -> str:
        return "r" if o == 0 else f"ro_{'m' if o < 0 else 'p'}{abs(o)}"

    def visit(root) -> str:
        stack = [root]
        while stack:
            x = stack[-1]
            if x.key in temps:
                stack.pop()
                continue
            todo = [a for a in x.args if isinstance(a, Expr) and a.key not in temps]
            if todo:
                stack.extend(todo)
                continue
            stack.pop()
            name = f"f{len(temps)}"
            if x.op == "mask":
                inter, col, off = x.args
                if inter != 1:
                    raise NotImplementedError("LogUp fractions read trace columns (interaction 1) only")
                if x.args not in slot:
                    slot[x.args] = len(masks)
                    masks.append(Mask(*x.args))
                if off:
                    offsets.add(off)
                lines.append(f"    const uint32_t {name} = __ldg(cols[{slot[x.args]}] + {row_name(off)});")
            elif x.op == "const":
                lines.append(f"    const uint32_t {name} = {x.args[0]}u;")
            elif x.op == "param":
                j = e.params.index(x.args[0])
                lines.append(f"    const qm31 {name} = qm31_make(params[{4 * j}], params[{4 * j + 1}], "
                             f"params[{4 * j + 2}], params[{4 * j + 3}]);")
            elif x.op == "secure":
                parts = ", ".join(temps[a.key] for a in x.args)
                lines.append(f"    const qm31 {name} = qm31_make({parts});")
            elif x.op == "neg":
                t = temps[x.args[0].key]
                lines.append(f"    const {'qm31' if x.ext else 'uint32_t'} {name} = "
                             f"{'qm31_neg' if x.ext else 'm31_neg'}({t});")
            else:
                a, b = x.args
                ta, tb = temps[a.key], temps[b.key]
                if not x.ext:
                    rhs = f"m31_{x.op}({ta}, {tb})"
                elif a.ext and b.ext:
                    rhs = f"qm31_{x.op}({ta}, {tb})"
                elif x.op == "mul":
                    q, m = (ta, tb) if a.ext else (tb, ta)
                    rhs = f"qm31_mul_m31({q}, {m})"
                else:
                    qa = ta if a.ext else f"qm31_make({ta}, 0, 0, 0)"
                    qb = tb if b.ext else f"qm31_make({tb}, 0, 0, 0)"
                    rhs = f"qm31_{x.op}({qa}, {qb})"
                lines.append(f"    const {'qm31' if x.ext else 'uint32_t'} {name} = {rhs};")
            temps[x.key] = name
        v = temps[root.key]
        return v if root.ext else f"qm31_make({v}, 0, 0, 0)"

    writes = []
    for j, (num, den) in enumerate(e.logup):
        for k, part in enumerate((visit(num), visit(den))):
            q = f"w{j}_{k}"
            writes.append(f"    const qm31 {q} = {part};")
            for c, coord in enumerate(("a.a", "a.b", "b.a", "b.b")):
                writes.append(f"    out[{8 * j + 4 * k + c}][r] = {q}.{coord};")
    row_defs = "".join(f"    const uint32_t {row_name(o)} = offset_row(r, {o}, log_n, log_n);\n"
                       for o in sorted(offsets))
    body = chr(10).join(lines + writes)
    src = f"""
// the LogUp batches' fractions of {len(e.logup)} interaction columns at every trace row
extern "C" __global__ void __launch_bounds__(256) cs_air_fractions(
    const uint32_t* const* __restrict__ cols, const uint32_t* __restrict__ params, uint32_t log_n,
    uint32_t* const* __restrict__ out) {{
  (void)params;
  const uint32_t n = 1u << log_n;
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {{
{row_defs}{body}
  }}
}}
"""
    return src, masks


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
        _lib.call("cs_rtc_compile_air_logup", air.source.encode(), len(names), hs, hn, len(air.masks),
                  air.n_constraints, len(air.params), len(air.fraction_masks), len(air.logup), ctypes.byref(handle),
                  log, len(log))
        self.handle = handle

    @classmethod
    def get(cls, air: Air) -> "CompiledAir":
        """One compiled kernel per distinct source (kept for the process's lifetime)."""
        key = hashlib.sha256(air.source.encode()).hexdigest()
        if key not in cls._cache:
            cls._cache[key] = cls(air)
        return cls._cache[key]

    def fractions(self, columns_by_interaction, log_n: int, params) -> list:
        """Each LogUp batch's combined (numerator, denominator) at every row of the trace domain
        (cs_rtc_air_fractions), as SecureColumnByCoords pairs. columns_by_interaction: the trace
        columns on the trace domain; parameters the fractions do not read may be left out."""
        from . import _lib
        from .backend import SecureColumnByCoords, _ptr_table, _stream
        n = 1 << log_n
        cols = [columns_by_interaction[m.interaction][m.column] for m in self.air.fraction_masks]
        if any(len(c) != n for c in cols):
            raise ValueError("fraction columns must be trace-domain columns of 2^log_n rows")
        out = [(SecureColumnByCoords.uninitialized(n), SecureColumnByCoords.uninitialized(n)) for _ in self.air.logup]
        table = [c.data for pair in out for col in pair for c in col.columns]
        pw = np.ascontiguousarray(np.asarray([params.get(p, (0, 0, 0, 0)) for p in self.air.params],
                                             np.uint32).reshape(-1))
        _lib.call("cs_rtc_air_fractions", self.handle, _ptr_table([c.data for c in cols]),
                  pw.ctypes.data if pw.size else None, log_n, _ptr_table(table), _stream())
        return out

    def composition(self, columns_by_interaction, trace_log: int, params, rc, accum, log_expansion: int = 0) -> None:
        """Adds the AIR's constraint quotients over accum's domain. params: {name: QM31}; rc: one
        QM31 weight per constraint. With log_expansion 0 the columns are evaluations on accum's
        domain, CanonicCoset(log len(accum)); with log_expansion e they are committed on
        CanonicCoset(log len(accum) + e) and accum's domain is their first len(accum) rows, that
        domain's subdomain (EvaluationMode::SubDomain)."""
        from . import _lib
        from .backend import _ptr_table, _stream
        cols = self.air.mask_columns(columns_by_interaction)
        # the kernel reads every mask column at rows below len(accum)
        if any(len(c) != len(accum) << log_expansion for c in cols):
            raise ValueError("mask columns must be evaluations on the accumulator's domain, or on the domain "
                             "it is the subdomain of")
        rcw = np.ascontiguousarray(np.asarray(rc, np.uint32).reshape(-1))
        assert rcw.size == 4 * self.air.n_constraints
        pw = np.ascontiguousarray(np.asarray([params[p] for p in self.air.params], np.uint32).reshape(-1))
        _lib.call("cs_rtc_air_composition_subdomain", self.handle, _ptr_table([c.data for c in cols]),
                  rcw.ctypes.data, pw.ctypes.data if pw.size else None, len(accum).bit_length() - 1, trace_log,
                  log_expansion, _ptr_table([c.data for c in accum.columns]), _stream())


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


# Poseidon2 (crates/examples/src/poseidon/mod.rs:34-47): 8 instances per row, a 16-word state,
# 4 + 4 full rounds around 14 partial rounds, every round constant 1234.
POSEIDON_INSTANCES_PER_ROW = 8
POSEIDON_STATE = 16
POSEIDON_PARTIAL_ROUNDS = 14
POSEIDON_HALF_FULL_ROUNDS = 4
POSEIDON_ROUND_CONST = 1234


def _apply_m4(x):
    """apply_m4 (mod.rs:74-90): the M4 MDS matrix of eprint 2023/323 section 5.1."""
    t0 = x[0] + x[1]
    t02 = t0 + t0
    t1 = x[2] + x[3]
    t12 = t1 + t1
    t2 = x[1] + x[1] + t1
    t3 = x[3] + x[3] + t0
    t4 = t12 + t12 + t3
    t5 = t02 + t02 + t2
    t6 = t3 + t5
    t7 = t2 + t4
    return [t6, t5, t7, t4]


def _apply_external_round_matrix(state) -> None:
    """apply_external_round_matrix (mod.rs:93-115): circ(2 M4, M4, M4, M4)."""
    for i in range(4):
        state[4 * i:4 * i + 4] = _apply_m4(state[4 * i:4 * i + 4])
    for j in range(4):
        s = state[j] + state[j + 4] + state[j + 8] + state[j + 12]
        for i in range(4):
            state[4 * i + j] = state[4 * i + j] + s


def _apply_internal_round_matrix(state) -> None:
    """apply_internal_round_matrix (mod.rs:118-129): s_i <- s_i 2^(i+1) + sum of the state."""
    total = state[0]
    for x in state[1:]:
        total = total + x
    for i in range(POSEIDON_STATE):
        state[i] = state[i] * (1 << (i + 1)) + total


def _pow5(x):
    x2 = x * x
    x4 = x2 * x2
    return x4 * x


def poseidon_air(e: Evaluator) -> None:
    """eval_poseidon_constraints (crates/examples/src/poseidon/mod.rs:137-187): per instance the
    round constraints (each S-box output equals its trace column), then the state lookups (the
    initial state with multiplicity 1, the final state with -1, relation `poseidon`), finalized in
    pairs. Parameters: poseidon_z, poseidon_alpha0..15 (LookupElements), shift."""
    for _ in range(POSEIDON_INSTANCES_PER_ROW):
        state = [e.next_trace_mask() for _ in range(POSEIDON_STATE)]
        initial = list(state)
        for half in range(2):
            if half == 1:
                for _ in range(POSEIDON_PARTIAL_ROUNDS):
                    state[0] = state[0] + POSEIDON_ROUND_CONST
                    _apply_internal_round_matrix(state)
                    state[0] = _pow5(state[0])
                    m = e.next_trace_mask()
                    e.add_constraint(state[0] - m)
                    state[0] = m
            for _ in range(POSEIDON_HALF_FULL_ROUNDS):
                state = [x + POSEIDON_ROUND_CONST for x in state]
                _apply_external_round_matrix(state)
                state = [_pow5(x) for x in state]
                for i in range(POSEIDON_STATE):
                    m = e.next_trace_mask()
                    e.add_constraint(state[i] - m)
                    state[i] = m
        e.add_to_relation("poseidon", 1, initial)
        e.add_to_relation("poseidon", -1, state)
    e.finalize_logup_in_pairs()


_POSEIDON_AIR = []


def poseidon_air_recorded() -> Air:
    """poseidon_air recorded once per process (its kernel is then compiled once, CompiledAir.get)."""
    if not _POSEIDON_AIR:
        _POSEIDON_AIR.append(compile_air("poseidon", poseidon_air))
    return _POSEIDON_AIR[0]


def _qm31_mul(a, b):
    """QM31 product of two 4-tuples: (a + b u)(c + d u) with u^2 = 2 + i over CM31 = M31[i]/(i^2 + 1)."""
    a0, a1, a2, a3 = (int(x) for x in a)
    b0, b1, b2, b3 = (int(x) for x in b)
    ac = ((a0 * b0 - a1 * b1) % P, (a0 * b1 + a1 * b0) % P)
    bd = ((a2 * b2 - a3 * b3) % P, (a2 * b3 + a3 * b2) % P)
    ad = ((a0 * b2 - a1 * b3) % P, (a0 * b3 + a1 * b2) % P)
    bc = ((a2 * b0 - a3 * b1) % P, (a2 * b1 + a3 * b0) % P)
    rbd = ((2 * bd[0] - bd[1]) % P, (bd[0] + 2 * bd[1]) % P)
    return ((ac[0] + rbd[0]) % P, (ac[1] + rbd[1]) % P, (ad[0] + bc[0]) % P, (ad[1] + bc[1]) % P)


def alpha_powers(alpha, n: int) -> list:
    """alpha^0 .. alpha^(n-1) (LookupElements::draw, crates/constraint-framework/src/logup.rs:70-79)."""
    out, cur = [], (1, 0, 0, 0)
    for _ in range(n):
        out.append(cur)
        cur = _qm31_mul(cur, alpha)
    return out


def lookup_params(relation: str, z, alpha, n_values: int) -> dict:
    """The parameters add_to_relation reads for `relation`: {relation}_z and {relation}_alpha{i}."""
    params = {f"{relation}_z": tuple(int(x) for x in z)}
    for i, p in enumerate(alpha_powers(alpha, n_values)):
        params[f"{relation}_alpha{i}"] = p
    return params


def logup_shift(claimed, trace_log: int) -> tuple:
    """claimed_sum / 2^trace_log, the cumsum shift of the last LogUp column (LogupAtRow::new)."""
    inv = pow(1 << trace_log, P - 2, P)
    return tuple(int(x) * inv % P for x in claimed)


def poseidon_params(lookup, claimed, trace_log: int) -> dict:
    """The parameters of poseidon_air from the drawn lookup elements (z, alpha: 8 words) and the
    claimed sum."""
    params = lookup_params("poseidon", lookup[:4], lookup[4:8], POSEIDON_STATE)
    params["shift"] = logup_shift(claimed, trace_log)
    return params
