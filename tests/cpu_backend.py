"""Test helper: the device operations of the restated host prover
(proving_gb300.prover) implemented with the CPU oracle's ops, so that host
prover can run without a GPU (CPU tests of its orchestration). Proof-level
parity does not rest on this: the oracle's own prover (oracle/oracle_prover.c)
is the independent statement the GPU proofs are compared with."""
from __future__ import annotations

import numpy as np

from proving_gb300 import prover as pr

from oracle import oracle as O


class Col:
    """An M31 column held in host memory."""

    def __init__(self, v):
        self.v = np.ascontiguousarray(v, dtype=np.uint32)

    @property
    def log_size(self):
        return self.v.size.bit_length() - 1


class SCol:
    """A QM31 column as four coordinate columns."""

    def __init__(self, coords):
        self.c = [np.ascontiguousarray(x, dtype=np.uint32) for x in coords]

    def __len__(self):
        return self.c[0].size


class Tree:
    def __init__(self, root: bytes, layers, height: int):
        self.root = root
        self.layers = layers  # leaves first: layers[i] has 2^(height - i) hashes
        self.height = height

    def hashes(self, layer_log: int, idx):
        lay = self.layers[self.height - layer_log]
        return [lay[i].tobytes() for i in idx]


class Twiddles:
    def __init__(self, domain_log: int):
        self.tw, self.itw = O.canonic_twiddles(domain_log)
        self.log_size = domain_log - 1


class _OracleLogupGenerator:
    """LogupTraceGenerator over the oracle's column generator (O.logup_gen_col, O.logup_finalize_last)."""

    def __init__(self):
        self.trace = []

    def col_from_fractions(self, fractions):
        prev = self.trace[-1] if self.trace else None
        for num, den in fractions:
            prev = O.logup_gen_col(num.c if isinstance(num, SCol) else num.v, den.c, prev)
        self.trace.append(prev)

    def finalize_last(self):
        last, claimed = O.logup_finalize_last(self.trace[-1])
        self.trace[-1] = last
        return [Col(c) for col in self.trace for c in col], tuple(int(x) for x in claimed)


class CpuOps:
    def secure_powers(self, felt, n):
        return pr.secure_powers(felt, n)

    def twiddles(self, root_log_domain: int):
        return Twiddles(root_log_domain)

    def columns_from_host(self, cols):
        return [Col(c) for c in cols]

    def log_size(self, col) -> int:
        return col.log_size

    def interpolate(self, cols, tw):
        res = O.interpolate_batch([c.v for c in cols], tw.itw)
        for c, r in zip(cols, res):
            c.v = r

    def interpolate_into(self, cols, tw):
        return [Col(r) for r in O.interpolate_batch([c.v for c in cols], tw.itw)]

    def logup_running_sum(self, values, z):
        out, claimed = O.logup_running_sum(values.v, z)
        return SCol(out), claimed

    def logup_running_sums(self, values, z):
        cols, claimed = [], []
        for v in values:
            out, cs = O.logup_running_sum(v.v, z)
            cols.append(SCol(out))
            claimed.append(tuple(int(x) for x in cs))
        return cols, claimed

    def air_composition(self, air, columns_by_interaction, trace_log, params, rc, accum, log_expansion=0):
        from oracle.air_eval import air_composition
        cols = {k: [c.v for c in v] for k, v in columns_by_interaction.items()}
        accum.c = air_composition(air, cols, len(accum).bit_length() - 1, trace_log, params, rc, out=accum.c,
                                  log_expansion=log_expansion)

    def air_fractions(self, air, columns_by_interaction, log_n, params):
        from oracle.air_eval import air_fractions
        cols = {k: [c.v for c in v] for k, v in columns_by_interaction.items()}
        full = {p: params.get(p, (0, 0, 0, 0)) for p in air.params}
        return [(SCol(num), SCol(den)) for num, den in air_fractions(air, cols, log_n, full)]

    def logup_generator(self, log_n):
        return _OracleLogupGenerator()

    def interpolate_secure_on_subdomain(self, accum, domain_log_size, tw):
        sub_log = len(accum).bit_length() - 1
        sub_itw = O.extract_subdomain_twiddles(tw.itw, domain_log_size, sub_log)
        return [Col(O.interpolate_on_subdomain(c, sub_itw, domain_log_size)) for c in accum.c]

    def logup_compositions(self, values_evals, inter_evals, trace_log, z, claimed, rcs, accum):
        for v, it, c, r in zip(values_evals, inter_evals, claimed, rcs):
            self.logup_composition(v, it, trace_log, z, c, r, accum)

    def logup_composition(self, values_eval, inter_eval, trace_log, z, claimed, rc, accum):
        accum.c = O.logup_composition(values_eval.v, [c.v for c in inter_eval], trace_log, z, claimed, rc,
                                      out=accum.c)

    def poseidon_trace(self, log_n):
        return [Col(c) for c in O.poseidon_trace(log_n)]

    def poseidon_interaction(self, trace, lookup):
        out, claimed = O.poseidon_interaction([c.v for c in trace], lookup[:4], lookup[4:])
        return [Col(c) for c in out], claimed

    def poseidon_composition(self, trace_evals, inter_evals, trace_log, lookup, claimed, rc, accum):
        accum.c = O.poseidon_composition([c.v for c in trace_evals], [c.v for c in inter_evals], trace_log,
                                         lookup, claimed, rc, out=accum.c)

    def evaluate(self, coeffs, log_size, tw):
        return [Col(e) for e in O.evaluate_batch([c.v for c in coeffs], [log_size] * len(coeffs), tw.tw)]

    def merkle_commit(self, cols, L):
        root, layers = O.merkle_commit([c.v for c in cols], L, with_layers=True)
        return Tree(root, layers, L)

    def gather(self, col, idx):
        return col.v[np.asarray(idx, dtype=np.int64)]

    def secure_zeros(self, n):
        return SCol([np.zeros(n, np.uint32) for _ in range(4)])

    def secure_len(self, col) -> int:
        return len(col)

    def secure_columns(self, col):
        return [Col(c) for c in col.c]

    def secure_coords(self, col):
        return [Col(c) for c in col.c]

    def gather_many(self, items):
        """Column values ("col", col, idx) and Merkle digests ("dig", tree, layer_log, nodes),
        the latter as (n, 8) little-endian words."""
        out = []
        for it in items:
            if it[0] == "cols":
                ix = np.asarray(it[2], dtype=np.int64)
                out.append(np.stack([c.v[ix] for c in it[1]]) if it[1] else np.zeros((0, ix.size), np.uint32))
            elif it[0] == "col":
                out.append(it[1].v[np.asarray(it[2], dtype=np.int64)])
            elif it[0] == "digs":
                tree = it[1]
                parts = [np.ascontiguousarray(tree.layers[tree.height - k][np.asarray(n, dtype=np.int64)])
                         .view("<u4").reshape(-1, 8) for k, n in it[2]]
                out.append(np.concatenate(parts) if parts else np.zeros((0, 8), np.uint32))
            else:
                tree, k, nodes = it[1], it[2], it[3]
                lay = tree.layers[tree.height - k]
                out.append(np.ascontiguousarray(lay[np.asarray(nodes, dtype=np.int64)]).view("<u4").reshape(-1, 8))
        return out

    def gather_secure(self, col, idx):
        ix = np.asarray(idx, dtype=np.int64)
        vals = [c[ix] for c in col.c]
        return [tuple(int(vals[k][i]) for k in range(4)) for i in range(len(idx))]

    def wide_fib_composition(self, evals, trace_log, rc, accum):
        eval_log = len(accum).bit_length() - 1
        accum.c = O.wide_fib_composition([e.v for e in evals], eval_log, trace_log, np.asarray(rc, np.uint32),
                                         out=accum.c)

    def interpolate_secure(self, accum, tw):
        return [Col(c) for c in O.interpolate_batch(accum.c, tw.itw)]

    def split_at_mid(self, coeff_cols):
        half = coeff_cols[0].v.size // 2
        return [Col(c.v[:half]) for c in coeff_cols], [Col(c.v[half:]) for c in coeff_cols]

    def grind(self, digest, bits):
        return O.grind(digest, bits)

    def barycentric_weights(self, log_size, point):
        return SCol(O.barycentric_weights(log_size, point[0], point[1]))

    def barycentric_eval(self, cols, weights):
        return [tuple(int(x) for x in O.barycentric_eval(c.v, weights.c)) for c in cols]

    def barycentric_eval_lazy(self, cols, weights):
        return self.barycentric_eval(cols, weights)

    def fetch_evals(self, handles):
        return list(handles)

    def accumulate_numerators(self, cols, coeffs, log_blowup):
        arr = np.asarray(coeffs, np.uint32)
        out, fl = O.accumulate_numerators([c.v for c in cols], log_blowup, arr)
        return SCol(out), fl

    def lift_and_accumulate(self, cols):
        return SCol(O.lift_and_accumulate([c.c for c in cols]))

    def compute_quotients_and_combine(self, parts, points, fls, lifting, log_blowup, tw):
        sub = O.quotients_on_subdomain([p.c for p in parts], points, fls, lifting, log_blowup)
        sub_itw = O.extract_subdomain_twiddles(tw.itw, lifting, lifting - log_blowup)
        return SCol([O.evaluate(O.interpolate_on_subdomain(c, sub_itw, lifting), lifting, tw.tw) for c in sub])

    def fold_circle_into_line(self, col, alpha, tw):
        return SCol(O.fold_circle_into_line(col.c, alpha))

    def fold_line(self, col, alpha, tw):
        n = len(col)
        return SCol(O.fold_line(col.c, O.line_domain_initial_index(n.bit_length() - 1), alpha))

    def fold_line_steps(self, col, alphas, tw):
        for a in alphas:
            col = self.fold_line(col, a, tw)
        return col

    def pack_leaves(self, cols):
        # pack_leaves_input: column coord + 4 offset holds coordinate coord of row 4 r + offset
        return [Col(cols[coord].v[off::4]) for off in range(4) for coord in range(4)]
