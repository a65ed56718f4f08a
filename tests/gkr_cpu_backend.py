"""Test helper: the CPU backend's GkrOps and MleOps
(crates/stwo/src/prover/backend/cpu/lookups/gkr.rs, cpu/lookups/mle.rs)
restated over numpy arrays, with the methods of proving_gb300.gkr.DeviceGkrOps,
so the GKR driver runs on it and on the device and the two proofs can be
compared value for value. A secure MLE is an (n, 4) int64 array of canonical
coordinates, a base MLE an (n,) array. Also the test-only
Mle::eval_at_point (crates/stwo/src/prover/lookups/mle.rs:73-104)."""
from __future__ import annotations

import numpy as np

from proving_gb300 import gkr as G
from proving_gb300 import prover as pr

P = pr.P


def _secure(a):
    a = np.asarray(a, np.int64)
    if a.ndim == 1:  # base values as QM31
        return np.stack([a % P, np.zeros_like(a), np.zeros_like(a), np.zeros_like(a)], axis=-1)
    return a % P


def _q(x):
    return np.asarray(x, np.int64).reshape(4)


class CpuGkrOps:
    def mle_from_host(self, values, base: bool = False) -> G.Mle:
        if base:
            a = np.asarray(values, np.int64).reshape(-1) % P
        else:
            a = np.asarray(values, np.int64).reshape(-1, 4) % P
        n = a.shape[0]
        if n & (n - 1):
            raise ValueError("an MLE has a power-of-two number of values")
        return G.Mle(a, n.bit_length() - 1, base)

    def values(self, mle: G.Mle, n: int):
        a = _secure(mle.data[:n])
        return [tuple(int(x) for x in r) for r in a]

    def values_many(self, requests):
        return [self.values(m, n) for m, n in requests]

    def gen_eq_evals(self, y, v) -> G.Mle:
        """gen_eq_evals (cpu/lookups/gkr.rs:230-246): for y_i from the last, each value c splits
        into c - c y_i (kept) and c y_i (appended)."""
        evals = _q(v)[None, :]
        for yi in reversed(list(y)):
            tmp = pr.qv_mul(evals, _q(yi)[None, :])
            evals = np.concatenate([pr.qv_sub(evals, tmp), tmp], axis=0)
        return G.Mle(evals, len(y))

    def fix_first_variable(self, mle: G.Mle, x) -> G.Mle:
        """MleOps::fix_first_variable (cpu/lookups/mle.rs:12-45): fold_mle_evals of the halves."""
        a = _secure(mle.data)
        half = a.shape[0] // 2
        lhs, rhs = a[:half], a[half:]
        out = pr.qv_add(pr.qv_mul(_q(x)[None, :], pr.qv_sub(rhs, lhs)), lhs)
        return G.Mle(out, mle.n_variables - 1)

    def next_layer(self, layer: G.Layer) -> G.Layer:
        """next_grand_product_layer / next_logup_layer (cpu/lookups/gkr.rs:248-281)."""
        n = layer.n_variables
        if layer.kind == G.GRAND_PRODUCT:
            a = layer.mles[0].data
            return G.Layer(G.GRAND_PRODUCT, [G.Mle(pr.qv_mul(a[0::2], a[1::2]), n - 1)])
        den = layer.mles[-1].data
        if layer.kind == G.LOGUP_SINGLES:
            num = _secure(np.ones(den.shape[0], np.int64))
        else:
            num = _secure(layer.mles[0].data)
        n0, n1, d0, d1 = num[0::2], num[1::2], den[0::2], den[1::2]
        # Fraction::new(n0, d0) + Fraction::new(n1, d1) (crates/stwo/src/core/fraction.rs:19-31)
        nn = pr.qv_add(pr.qv_mul(d1, n0), pr.qv_mul(d0, n1))
        dd = pr.qv_mul(d0, d1)
        return G.Layer(G.LOGUP_GENERIC, [G.Mle(nn, n - 1), G.Mle(dd, n - 1)])

    def sum_as_poly_evals(self, items):
        """eval_grand_product_sum / eval_logup_sum / eval_logup_singles_sum
        (cpu/lookups/gkr.rs:66-227) for each (input layer, eq evals, lambda)."""
        return [self._sum(layer, eq_mle, lam) for layer, eq_mle, lam in items]

    def _sum(self, layer: G.Layer, eq_mle: G.Mle, lam):
        n_terms = 1 << (layer.n_variables - 2)
        e = eq_mle.data[:n_terms]
        lam = _q(lam)[None, :]

        def at(col):
            c = _secure(col)
            r0i0, r0i1 = c[0:2 * n_terms:2], c[1:2 * n_terms:2]
            r1i0, r1i1 = c[2 * n_terms::2], c[2 * n_terms + 1::2]
            # inp(r, 2, x) = 2 inp(r, 1, x) - inp(r, 0, x)
            r2i0 = pr.qv_sub(pr.qv_add(r1i0, r1i0), r0i0)
            r2i1 = pr.qv_sub(pr.qv_add(r1i1, r1i1), r0i1)
            return (r0i0, r0i1), (r2i0, r2i1)

        den0, den2 = at(layer.mles[-1].data)
        if layer.kind == G.GRAND_PRODUCT:
            g0 = pr.qv_mul(den0[0], den0[1])
            g2 = pr.qv_mul(den2[0], den2[1])
        else:
            def gate(num, den):
                if num is None:  # Reciprocal::new(a) + Reciprocal::new(b) = (a + b) / (a b)
                    nn = pr.qv_add(den[0], den[1])
                else:
                    nn = pr.qv_add(pr.qv_mul(den[1], num[0]), pr.qv_mul(den[0], num[1]))
                dd = pr.qv_mul(den[0], den[1])
                return pr.qv_add(nn, pr.qv_mul(lam, dd))

            if layer.kind == G.LOGUP_SINGLES:
                num0 = num2 = None
            else:
                num0, num2 = at(layer.mles[0].data)
            g0, g2 = gate(num0, den0), gate(num2, den2)
        s0 = pr.qv_sum(pr.qv_mul(e, g0))
        s2 = pr.qv_sum(pr.qv_mul(e, g2))
        return tuple(int(x) for x in s0), tuple(int(x) for x in s2)


def mle_eval_at_point(values, point):
    """Mle::eval_at_point (mle.rs:73-104): p_i (rhs - lhs) + lhs over the halves for each
    variable, first variable first (the recursion there, unrolled: both halves are linear in
    their values)."""
    a = _secure(values)
    for p in point:
        half = a.shape[0] // 2
        a = pr.qv_add(pr.qv_mul(_q(p)[None, :], pr.qv_sub(a[half:], a[:half])), a[:half])
    return tuple(int(x) for x in a[0])
