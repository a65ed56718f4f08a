"""GKR batch prover for grand-product and LogUp lookups over the device backend.

Follows crates/stwo/src/prover/lookups/: gkr_prover.rs (Layer, EqEvals,
GkrMultivariatePolyOracle, prove_batch, correct_sum_as_poly_in_first_variable),
sumcheck.rs (prove_batch), utils.rs (UnivariatePoly, eq, fold_mle_evals,
random_linear_combination) and mle.rs (Mle). The per-element work -- the eq
evaluations, each layer of the circuit, the two sums of every sum-check round
and the fixing of a variable -- runs on the device through the library's
GkrOps / MleOps entry points (`DeviceGkrOps`); the protocol itself (channel,
round polynomials, masks) is host logic on a few field elements per round.

The driver takes any object with DeviceGkrOps' methods, so the same protocol
code runs over another implementation of the operations and the two proofs can
be compared value for value.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .prover import P, qm, qm_add, qm_inv, qm_mul, qm_mul_m31, qm_neg, qm_sub

GRAND_PRODUCT, LOGUP_GENERIC, LOGUP_MULTIPLICITIES, LOGUP_SINGLES = 0, 1, 2, 3
KIND_NAMES = {GRAND_PRODUCT: "GrandProduct", LOGUP_GENERIC: "LogUpGeneric",
              LOGUP_MULTIPLICITIES: "LogUpMultiplicities", LOGUP_SINGLES: "LogUpSingles"}

ZERO = qm(0)
ONE = qm(1)
MAX_DEGREE = 3  # sumcheck.rs MAX_DEGREE


def _is_zero(x) -> bool:
    return all(c == 0 for c in x)


def q_div(a, b):
    if _is_zero(b):
        raise ZeroDivisionError("division by zero in QM31")
    return qm_mul(a, qm_inv(b))


# ------------------------------------------------------------ univariate polynomials (utils.rs)
# A polynomial is the list of its coefficients (QM31 tuples) from degree 0 up.
# UnivariatePoly::new trims leading zeros; sums and scalings do not, which fixes
# how many coefficients a combined round polynomial sends to the channel.


def poly_new(coeffs) -> list:
    c = list(coeffs)
    while c and _is_zero(c[-1]):
        c.pop()
    return c


def poly_eval(coeffs, x):
    """horner_eval (utils.rs)."""
    acc = ZERO
    for c in reversed(coeffs):
        acc = qm_add(qm_mul(acc, x), c)
    return acc


def poly_degree(coeffs) -> int:
    return max(len(poly_new(coeffs)) - 1, 0)


def poly_add(a, b) -> list:
    n = max(len(a), len(b))
    return [qm_add(a[i], b[i]) if i < len(a) and i < len(b) else (a[i] if i < len(a) else b[i]) for i in range(n)]


def poly_scale(a, s) -> list:
    return [qm_mul(c, s) for c in a]


def poly_mul(a, b) -> list:
    if all(_is_zero(c) for c in a) or all(_is_zero(c) for c in b):
        return []
    a, b = poly_new(a), poly_new(b)
    res = [ZERO] * (len(a) + len(b) - 1)
    for i, ca in enumerate(a):
        for j, cb in enumerate(b):
            res[i + j] = qm_add(res[i + j], qm_mul(ca, cb))
    return poly_new(res)


def interpolate_lagrange(xs, ys) -> list:
    """UnivariatePoly::interpolate_lagrange (utils.rs)."""
    assert len(xs) == len(ys)
    coeffs = []
    for i, (xi, yi) in enumerate(zip(xs, ys)):
        prod = yi
        for j, xj in enumerate(xs):
            if i != j:
                prod = q_div(prod, qm_sub(xi, xj))
        term = poly_new([prod])
        for j, xj in enumerate(xs):
            if i != j:
                term = poly_mul(term, poly_add([ZERO, ONE], [qm_neg(c) for c in poly_new([xj])]))
        coeffs = poly_add(coeffs, term)
    return poly_new(coeffs)


def random_linear_combination(values, alpha):
    """v_0 + alpha v_1 + ... (utils.rs random_linear_combination = horner_eval)."""
    return poly_eval(values, alpha)


def poly_linear_combination(polys, alpha) -> list:
    """p_0 + alpha p_1 + ... (sumcheck.rs random_linear_combination): scaled and added without
    trimming, so the result has as many coefficients as the longest input."""
    acc = []
    for p in reversed(polys):
        acc = poly_add(poly_scale(acc, alpha), p)
    return acc


def eq(x, y):
    """Lagrange kernel of the boolean hypercube (utils.rs eq)."""
    assert len(x) == len(y)
    r = ONE
    for xi, yi in zip(x, y):
        r = qm_mul(r, qm_add(qm_mul(xi, yi), qm_mul(qm_sub(ONE, xi), qm_sub(ONE, yi))))
    return r


def batch_inverse(xs):
    """Inverses of nonzero QM31 values with one field inversion (prefix products)."""
    pre, acc = [], ONE
    for x in xs:
        if _is_zero(x):
            raise ZeroDivisionError("division by zero in QM31")
        pre.append(acc)
        acc = qm_mul(acc, x)
    inv = qm_inv(acc)
    out = [None] * len(xs)
    for i in range(len(xs) - 1, -1, -1):
        out[i] = qm_mul(inv, pre[i])
        inv = qm_mul(inv, xs[i])
    return out


def fold_mle_evals(assignment, eval0, eval1):
    """assignment (eval1 - eval0) + eval0 (utils.rs)."""
    return qm_add(qm_mul(assignment, qm_sub(eval1, eval0)), eval0)


# ------------------------------------------------------------ layers (gkr_prover.rs)

@dataclass
class Mle:
    """Mle (mle.rs): 2^n_variables values on the hypercube; `data` is the operations' storage."""
    data: object
    n_variables: int
    base: bool = False


@dataclass
class Layer:
    """Layer (gkr_prover.rs): mles = [column] for a grand product, [numerators, denominators]
    for generic / multiplicities LogUp, [denominators] for LogUp singles."""
    kind: int
    mles: list

    @property
    def n_variables(self) -> int:
        return self.mles[-1].n_variables

    def is_output_layer(self) -> bool:
        return self.n_variables == 0


@dataclass
class GkrMask:
    """GkrMask (gkr_verifier.rs): two values of each column of a layer."""
    columns: list  # [(v0, v1), ...]

    def reduce_at_point(self, x):
        return [fold_mle_evals(x, v0, v1) for v0, v1 in self.columns]


@dataclass
class GkrBatchProof:
    sumcheck_proofs: list = field(default_factory=list)          # per layer: round polynomials
    layer_masks_by_instance: list = field(default_factory=list)  # per instance: GkrMask per layer
    output_claims_by_instance: list = field(default_factory=list)


@dataclass
class GkrArtifact:
    ood_point: list
    claims_to_verify_by_instance: list
    n_variables_by_instance: list


class RoundConstants:
    """What correct_sum_as_poly_in_first_variable needs of y for each k = 1..|y|, with two
    batched inversions: a_k = 1 / eq(0^(n-k+1), y[..n-k+1]), the extra root
    b_k = (1 - y[n-k]) / (1 - 2 y[n-k]), the factors eq(0, y[n-k]) and eq(2, y[n-k]), and
    1 / (x - b_k) for x = 0, 1, 2."""

    def __init__(self, y):
        n = len(y)
        self.n = n
        prefix, acc = [], ONE
        for yi in y:  # prefix[m] = prod_{i <= m} (1 - y_i) = eq(0^(m+1), y[..m+1])
            acc = qm_mul(acc, qm_sub(ONE, yi))
            prefix.append(acc)
        ks = list(range(1, n + 1))
        inv = batch_inverse([prefix[n - k] for k in ks] + [qm_sub(ONE, qm_add(y[n - k], y[n - k])) for k in ks])
        self.a = {k: inv[i] for i, k in enumerate(ks)}
        self.b = {k: qm_mul(qm_sub(ONE, y[n - k]), inv[n + i]) for i, k in enumerate(ks)}
        self.eq0 = {k: eq([ZERO], [y[n - k]]) for k in ks}
        self.eq2 = {k: eq([qm(2)], [y[n - k]]) for k in ks}
        inv_b = batch_inverse([qm_sub(qm(x), self.b[k]) for k in ks for x in range(3)])
        self.inv_xb = {k: inv_b[3 * i:3 * i + 3] for i, k in enumerate(ks)}

    def correct_sum(self, f_at_0, f_at_2, claim, k: int) -> list:
        """correct_sum_as_poly_in_first_variable: r(t) of degree <= 3 with r(0), r(1) = claim - r(0),
        r(2) and the root b. It is (t - b) q(t) with q the quadratic through x, r(x) / (x - b) for
        x = 0, 1, 2 -- the polynomial interpolate_lagrange returns on those four points (it is
        unique), with one multiplication per coefficient instead of inversions."""
        assert 1 <= k <= self.n
        a = self.a[k]
        r0 = qm_mul(qm_mul(f_at_0, self.eq0[k]), a)
        r1 = qm_sub(claim, r0)
        r2 = qm_mul(qm_mul(f_at_2, self.eq2[k]), a)
        i0, i1, i2 = self.inv_xb[k]
        q0, q1, q2 = qm_mul(r0, i0), qm_mul(r1, i1), qm_mul(r2, i2)
        c2 = qm_mul_m31(qm_add(qm_sub(q2, qm_add(q1, q1)), q0), (P + 1) // 2)
        c1 = qm_sub(qm_sub(q1, q0), c2)
        b = self.b[k]
        return poly_new([qm_neg(qm_mul(b, q0)), qm_sub(q0, qm_mul(b, c1)), qm_sub(c1, qm_mul(b, c2)), c2])


class EqEvals:
    """EqEvals (gkr_prover.rs): eq((0, x), y) for x in {0,1}^(|y|-1)."""

    def __init__(self, ops, y):
        self.y = list(y)
        if not self.y:
            self.evals = ops.mle_from_host([ONE])
        else:
            v = eq([ZERO], [self.y[0]])
            self.evals = ops.gen_eq_evals(self.y[1:], v)
        self._consts = None

    @property
    def consts(self) -> RoundConstants:
        if self._consts is None:
            self._consts = RoundConstants(self.y)
        return self._consts


class GkrMultivariatePolyOracle:
    """GkrMultivariatePolyOracle (gkr_prover.rs)."""

    def __init__(self, eq_evals: EqEvals, input_layer: Layer, lam, correction=ONE):
        self.eq_evals = eq_evals
        self.input_layer = input_layer
        self.eq_fixed_var_correction = correction
        self.lam = lam

    @property
    def n_variables(self) -> int:
        return self.input_layer.n_variables - 1

    def is_constant(self) -> bool:
        return self.n_variables == 0

    def finish_sum(self, f0, f2, claim):
        """The host half of sum_as_poly_in_first_variable (cpu/lookups/gkr.rs:40-64)."""
        f0 = qm_mul(f0, self.eq_fixed_var_correction)
        f2 = qm_mul(f2, self.eq_fixed_var_correction)
        return self.eq_evals.consts.correct_sum(f0, f2, claim, self.n_variables)

    def fix_first_variable(self, ops, challenge) -> "GkrMultivariatePolyOracle":
        if self.is_constant():
            return self
        y = self.eq_evals.y
        z0 = y[len(y) - self.n_variables]
        corr = qm_mul(self.eq_fixed_var_correction, eq([challenge], [z0]))
        return GkrMultivariatePolyOracle(self.eq_evals, layer_fix_first_variable(ops, self.input_layer, challenge),
                                         self.lam, corr)

    def mask_columns(self) -> list:
        """The MLEs whose two values make the mask (try_into_mask, gkr_prover.rs)."""
        if not self.is_constant():
            raise ValueError("polynomial is not constant")
        if self.input_layer.kind == LOGUP_MULTIPLICITIES:
            raise NotImplementedError("mask of a LogUpMultiplicities layer (never reached by the reference)")
        return self.input_layer.mles

    def mask_from_values(self, values) -> GkrMask:
        cols = [tuple(v) for v in values]
        if self.input_layer.kind == LOGUP_SINGLES:
            cols = [(ONE, ONE)] + cols
        return GkrMask(cols)


def masks_of(ops, oracles) -> list:
    """try_into_mask for constant oracles, with one read of all their columns."""
    cols = [o.mask_columns() for o in oracles]
    flat = ops.values_many([(m, 2) for c in cols for m in c])
    out, i = [], 0
    for o, c in zip(oracles, cols):
        out.append(o.mask_from_values(flat[i:i + len(c)]))
        i += len(c)
    return out


def layer_fix_first_variable(ops, layer: Layer, x0) -> Layer:
    """Layer::fix_first_variable (gkr_prover.rs): multiplicities become generic LogUp."""
    if layer.n_variables == 0:
        return layer
    mles = [ops.fix_first_variable(m, x0) for m in layer.mles]
    kind = LOGUP_GENERIC if layer.kind == LOGUP_MULTIPLICITIES else layer.kind
    return Layer(kind, mles)


def output_layer_values(ops, layer: Layer):
    """Layer::try_into_output_layer_values (gkr_prover.rs)."""
    if not layer.is_output_layer():
        raise ValueError("not an output layer")
    if layer.kind == LOGUP_SINGLES:
        return [ONE, ops.values(layer.mles[0], 1)[0]]
    if layer.kind in (LOGUP_GENERIC, LOGUP_MULTIPLICITIES):
        return [ops.values(layer.mles[0], 1)[0], ops.values(layer.mles[1], 1)[0]]
    return [ops.values(layer.mles[0], 1)[0]]


def gen_layers(ops, input_layer: Layer) -> list:
    """gen_layers (gkr_prover.rs): the input layer, then each next layer down to the output."""
    layers = [input_layer]
    while not layers[-1].is_output_layer():
        layers.append(ops.next_layer(layers[-1]))
    assert len(layers) == input_layer.n_variables + 1
    return layers


def correct_sum_as_poly_in_first_variable(f_at_0, f_at_2, claim, y, k: int) -> list:
    """correct_sum_as_poly_in_first_variable (gkr_prover.rs): r(t) from f(0), f(2)."""
    assert k != 0
    n = len(y)
    assert k <= n
    a_const = qm_inv(eq([ZERO] * (n - k + 1), y[:n - k + 1]))
    yk = y[n - k]
    b_const = q_div(qm_sub(ONE, yk), qm_sub(ONE, qm_add(yk, yk)))
    r0 = qm_mul(qm_mul(f_at_0, eq([ZERO], [yk])), a_const)
    r1 = qm_sub(claim, r0)
    r2 = qm_mul(qm_mul(f_at_2, eq([qm(2)], [yk])), a_const)
    return interpolate_lagrange([ZERO, ONE, qm(2), b_const], [r0, r1, r2, ZERO])


# ------------------------------------------------------------ sum-check (sumcheck.rs)

class SumcheckError(AssertionError):
    pass


def sumcheck_prove_batch(ops, claims, oracles, lam, channel):
    """sumcheck::prove_batch: one sum-check over h = g_0 + lam g_1 + ...; returns
    (round polynomials, assignment, the constant oracles, their claims)."""
    assert oracles and len(claims) == len(oracles)
    n_variables = max(o.n_variables for o in oracles)
    claims = [qm_mul_m31(c, pow(2, n_variables - o.n_variables, P)) for c, o in zip(claims, oracles)]
    inv2 = pow(2, P - 2, P)
    round_polys, assignment = [], []
    for rnd in range(n_variables):
        remaining = n_variables - rnd
        active = [i for i, o in enumerate(oracles) if o.n_variables == remaining]
        sums = ops.sum_as_poly_evals([(oracles[i].input_layer, oracles[i].eq_evals.evals, oracles[i].lam)
                                      for i in active])
        sums = dict(zip(active, sums))
        this_round = []
        for i, (o, claim) in enumerate(zip(oracles, claims)):
            if i in sums:
                poly = o.finish_sum(sums[i][0], sums[i][1], claim)
            else:
                poly = poly_new([qm_mul_m31(claim, inv2)])
            if qm_add(poly_eval(poly, ZERO), poly_eval(poly, ONE)) != claim:
                raise SumcheckError(f"round polynomial inconsistent with its claim (i={i}, round={rnd})")
            if poly_degree(poly) > MAX_DEGREE:
                raise SumcheckError(f"round polynomial degree above {MAX_DEGREE} (i={i}, round={rnd})")
            this_round.append(poly)
        round_poly = poly_linear_combination(this_round, lam)
        channel.mix_felts(round_poly)
        challenge = channel.draw_secure_felt()
        claims = [poly_eval(p, challenge) for p in this_round]
        oracles = [o.fix_first_variable(ops, challenge) if o.n_variables == remaining else o for o in oracles]
        round_polys.append(round_poly)
        assignment.append(challenge)
    return round_polys, assignment, oracles, claims


# ------------------------------------------------------------ GKR (gkr_prover.rs prove_batch)

def prove_batch(ops, channel, input_layers) -> tuple[GkrBatchProof, GkrArtifact]:
    """Batch proves lookup circuits with GKR (gkr_prover.rs prove_batch). The input layers should
    be committed to the channel before the call."""
    n_instances = len(input_layers)
    n_layers_by_instance = [lay.n_variables for lay in input_layers]
    n_layers = max(n_layers_by_instance)
    layers_by_instance = [iter(reversed(gen_layers(ops, lay))) for lay in input_layers]
    output_claims = [None] * n_instances
    masks_by_instance = [[] for _ in range(n_instances)]
    claims_to_verify = [None] * n_instances
    sumcheck_proofs = []
    ood_point = []
    for layer in range(n_layers):
        remaining = n_layers - layer
        for inst in range(n_instances):
            if n_layers_by_instance[inst] == remaining:
                values = output_layer_values(ops, next(layers_by_instance[inst]))
                claims_to_verify[inst] = values
                output_claims[inst] = values
        for claims in claims_to_verify:
            if claims is not None:
                channel.mix_felts(claims)
        eq_evals = EqEvals(ops, ood_point)
        sumcheck_alpha = channel.draw_secure_felt()
        instance_lambda = channel.draw_secure_felt()
        oracles, sc_claims, sc_instances = [], [], []
        for inst, claims in enumerate(claims_to_verify):
            if claims is not None:
                lay = next(layers_by_instance[inst])
                oracles.append(GkrMultivariatePolyOracle(eq_evals, lay, instance_lambda))
                sc_claims.append(random_linear_combination(claims, instance_lambda))
                sc_instances.append(inst)
        round_polys, sc_ood_point, constants, _ = sumcheck_prove_batch(ops, sc_claims, oracles, sumcheck_alpha,
                                                                       channel)
        sumcheck_proofs.append(round_polys)
        masks = masks_of(ops, constants)
        for inst, mask in zip(sc_instances, masks):
            channel.mix_felts([v for col in mask.columns for v in col])
            masks_by_instance[inst].append(mask)
        challenge = channel.draw_secure_felt()
        ood_point = list(sc_ood_point) + [challenge]
        for inst, mask in zip(sc_instances, masks):
            claims_to_verify[inst] = mask.reduce_at_point(challenge)
    proof = GkrBatchProof(sumcheck_proofs, masks_by_instance, output_claims)
    return proof, GkrArtifact(ood_point, claims_to_verify, n_layers_by_instance)


# ------------------------------------------------------------ device operations

class DeviceGkrOps:
    """GkrOps / MleOps over the library (cs_gkr_*, cs_mle_fix_first_variable). A secure MLE is
    a (4, 2^n) int32 CUDA tensor (coordinate columns), a base MLE a (1, 2^n) one."""

    def __init__(self):
        import torch
        self.torch = torch

    def _stream(self):
        return ctypes.c_void_p(self.torch.cuda.current_stream().cuda_stream)

    @staticmethod
    def _table(t):
        return (ctypes.c_void_p * 4)(*[t[k].data_ptr() for k in range(t.shape[0])])

    @staticmethod
    def _u32(v):
        return (ctypes.c_uint32 * 4)(*[int(c) % P for c in v])

    def _empty(self, n: int):
        return self.torch.empty((4, n), dtype=self.torch.int32, device="cuda")

    def mle_from_host(self, values, base: bool = False) -> Mle:
        if base:
            arr = np.ascontiguousarray(np.asarray(values, np.int64).reshape(1, -1) % P, dtype=np.uint32)
        else:
            arr = np.ascontiguousarray((np.asarray(values, np.int64).reshape(-1, 4) % P).T, dtype=np.uint32)
        n = arr.shape[1]
        if n & (n - 1):
            raise ValueError("an MLE has a power-of-two number of values")
        t = self.torch.from_numpy(arr.view(np.int32)).to("cuda")
        return Mle(t, n.bit_length() - 1, base)

    def values(self, mle: Mle, n: int):
        a = mle.data[:, :n].cpu().numpy().view(np.uint32).astype(np.int64)
        if mle.base:
            return [qm(int(v)) for v in a[0]]
        return [tuple(int(x) for x in a[:, i]) for i in range(a.shape[1])]

    def values_many(self, requests):
        """values() of several (MLE, n) requests with one read-back."""
        if not requests:
            return []
        parts = [(m.data[:1, :n].expand(4, n) if m.base else m.data[:, :n]) for m, n in requests]
        a = self.torch.cat(parts, dim=1).cpu().numpy().view(np.uint32).astype(np.int64)
        out, off = [], 0
        for (m, n), part in zip(requests, parts):
            blk = a[:, off:off + n]
            out.append([qm(int(v)) for v in blk[0]] if m.base else [tuple(int(x) for x in blk[:, i]) for i in range(n)])
            off += n
        return out

    def gen_eq_evals(self, y, v) -> Mle:
        out = self._empty(1 << len(y))
        ys = np.ascontiguousarray(np.asarray(y, np.int64).reshape(-1) % P, dtype=np.uint32)
        _lib.call("cs_gkr_gen_eq_evals", ys.ctypes.data if ys.size else None, len(y), self._u32(v),
                  self._table(out), self._stream())
        return Mle(out, len(y))

    def fix_first_variable(self, mle: Mle, x) -> Mle:
        n = mle.n_variables
        if n < 1:
            raise ValueError("fix_first_variable of a constant MLE")
        out = self._empty(1 << (n - 1))
        src = (ctypes.c_void_p * 4)(*([mle.data[0].data_ptr()] * 4 if mle.base else
                                      [mle.data[k].data_ptr() for k in range(4)]))
        _lib.call("cs_mle_fix_first_variable", src, int(mle.base), n, self._u32(x), self._table(out), self._stream())
        return Mle(out, n - 1)

    def _num_den(self, layer: Layer):
        if layer.kind in (LOGUP_GENERIC, LOGUP_MULTIPLICITIES):
            num, den = layer.mles
            ntab = (ctypes.c_void_p * 4)(*([num.data[0].data_ptr()] * 4 if num.base else
                                           [num.data[k].data_ptr() for k in range(4)]))
            return ntab, self._table(den.data)
        return None, self._table(layer.mles[0].data)

    def next_layer(self, layer: Layer) -> Layer:
        n = layer.n_variables
        ntab, dtab = self._num_den(layer)
        out_den = self._empty(1 << (n - 1))
        if layer.kind == GRAND_PRODUCT:
            _lib.call("cs_gkr_next_layer", layer.kind, None, dtab, n, None, self._table(out_den), self._stream())
            return Layer(GRAND_PRODUCT, [Mle(out_den, n - 1)])
        out_num = self._empty(1 << (n - 1))
        _lib.call("cs_gkr_next_layer", layer.kind, ntab, dtab, n, self._table(out_num), self._table(out_den),
                  self._stream())
        return Layer(LOGUP_GENERIC, [Mle(out_num, n - 1), Mle(out_den, n - 1)])

    def sum_as_poly_evals(self, items):
        """(f(0), f(2)) of each (input layer, eq evals, lambda), with one read-back for all."""
        if not items:
            return []
        out = self.torch.empty(8 * len(items), dtype=self.torch.int32, device="cuda")
        for j, (layer, eq_mle, lam) in enumerate(items):
            ntab, dtab = self._num_den(layer)
            _lib.call("cs_gkr_sum_as_poly", layer.kind, self._table(eq_mle.data), ntab, dtab, layer.n_variables,
                      self._u32(lam), out.data_ptr() + 32 * j, self._stream())
        w = out.cpu().numpy().view(np.uint32).reshape(-1, 8)
        return [(tuple(int(x) for x in r[:4]), tuple(int(x) for x in r[4:])) for r in w]


# ------------------------------------------------------------ native driver

def prove_batch_native(channel, input_layers) -> tuple[GkrBatchProof, GkrArtifact]:
    """prove_batch with the protocol in native code (cs_gkr_prove_batch): the same proof and
    artifact as prove_batch over DeviceGkrOps, with one host synchronisation per sum-check round and
    no interpreter between the launches. Inputs are device MLEs (DeviceGkrOps' layout); the
    channel (proving_gb300.prover.Blake2sChannel) is advanced as prove_batch advances it."""
    import struct
    import torch
    n = len(input_layers)
    kinds = (ctypes.c_uint32 * n)(*[lay.kind for lay in input_layers])
    nvars = (ctypes.c_uint32 * n)(*[lay.n_variables for lay in input_layers])
    cols = (ctypes.c_void_p * (8 * n))()
    for i, lay in enumerate(input_layers):
        den = lay.mles[-1].data
        for k in range(4):
            cols[8 * i + 4 + k] = den[k].data_ptr()
        if lay.kind in (LOGUP_GENERIC, LOGUP_MULTIPLICITIES):
            num = lay.mles[0]
            for k in range(1 if num.base else 4):
                cols[8 * i + k] = num.data[k].data_ptr()
    state = (ctypes.c_uint32 * 9)(*struct.unpack("<8I", channel.digest), channel.n_draws)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    n_words = ctypes.c_size_t()
    # the proof's size is known only at the end: a bound from the layer sizes, retried once if short
    layers = max(lay.n_variables for lay in input_layers)
    cap = 64 + n * 64 + layers * layers * 24 + n * layers * 24 + 8 * layers
    for _ in range(2):
        snap = (ctypes.c_uint32 * 9)(*state)
        words = (ctypes.c_uint64 * cap)()
        try:
            _lib.call("cs_gkr_prove_batch", n, kinds, nvars, cols, snap, words, cap, ctypes.byref(n_words), stream)
        except _lib.CudaBackendError:
            if n_words.value > cap:
                cap = n_words.value
                continue
            raise
        break
    w = list(words[:n_words.value])
    pos = 0

    def take():
        nonlocal pos
        pos += 1
        return int(w[pos - 1])

    def felt():
        nonlocal pos
        pos += 4
        return tuple(int(x) for x in w[pos - 4:pos])

    proof = GkrBatchProof()
    for _ in range(take()):
        proof.sumcheck_proofs.append([[felt() for _ in range(take())] for _ in range(take())])
    n_inst = take()
    for _ in range(n_inst):
        proof.layer_masks_by_instance.append(
            [GkrMask([(felt(), felt()) for _ in range(take())]) for _ in range(take())])
    for _ in range(n_inst):
        proof.output_claims_by_instance.append([felt() for _ in range(take())])
    ood = [felt() for _ in range(take())]
    claims = [[felt() for _ in range(take())] for _ in range(n_inst)]
    n_vars = [take() for _ in range(n_inst)]
    channel.digest = struct.pack("<8I", *snap[:8])
    channel.n_draws = snap[8]
    return proof, GkrArtifact(ood, claims, n_vars)
