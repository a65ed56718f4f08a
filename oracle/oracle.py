"""ORACLE — test infrastructure only: ctypes bindings to the C restatement.

Used by tests/, the smoke check and bench.py's CPU-baseline leg as the checker.
Every function takes and returns numpy arrays of uint32 words (M31 values in
[0, P)) or bytes (Blake2s digests).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"

P = (1 << 31) - 1

u32p = ctypes.POINTER(ctypes.c_uint32)
u8p = ctypes.POINTER(ctypes.c_uint8)


class Channel(ctypes.Structure):
    _fields_ = [("digest", ctypes.c_uint8 * 32), ("n_draws", ctypes.c_uint32)]


def build() -> Path:
    """Compile the oracle with its Makefile (plain gcc + OpenMP)."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        L = ctypes.CDLL(str(LIB_PATH))
        vp = ctypes.c_void_p
        L.orc_num_threads.restype = ctypes.c_int
        L.orc_grind.restype = ctypes.c_uint64
        L.orc_grind.argtypes = [vp, ctypes.c_uint32]
        L.orc_verify_pow_nonce.restype = ctypes.c_int
        L.orc_verify_pow_nonce.argtypes = [vp, ctypes.c_uint32, ctypes.c_uint64]
        L.orc_channel_mix_u64.argtypes = [vp, ctypes.c_uint64]
        L.orc_blake2s.argtypes = [vp, ctypes.c_uint64, vp]
        _lib = L
    return _lib


def _p(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return ctypes.c_void_p(a.ctypes.data)


def _u32(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.uint32))


def _ptr_array(arrs):
    arr = (ctypes.c_void_p * max(1, len(arrs)))()
    for i, a in enumerate(arrs):
        arr[i] = a.ctypes.data
    return arr


def num_threads() -> int:
    return lib().orc_num_threads()


def set_num_threads(n: int) -> None:
    lib().orc_set_num_threads(ctypes.c_int(n))


# ------------------------------------------------------------------ fields

def qm31_mul(a, b):
    a, b = _u32(a), _u32(b)
    out = np.zeros(4, np.uint32)
    lib().orc_qm31_mul(_p(a), _p(b), _p(out))
    return out


def qm31_inv(a):
    a = _u32(a)
    out = np.zeros(4, np.uint32)
    lib().orc_qm31_inv(_p(a), _p(out))
    return out


def m31_mul(a, b):
    a, b = _u32(a), _u32(b)
    out = np.zeros_like(a)
    lib().orc_m31_mul_batch(_p(a), _p(b), _p(out), ctypes.c_uint64(a.size))
    return out


def circle_index_to_point(idx: int):
    out = np.zeros(2, np.uint32)
    lib().orc_circle_index_to_point(ctypes.c_uint32(idx), _p(out))
    return int(out[0]), int(out[1])


def bit_reverse(v) -> np.ndarray:
    v = _u32(v).copy()
    n = v.size
    lib().orc_bit_reverse(_p(v), ctypes.c_uint32(n.bit_length() - 1))
    return v


# ---------------------------------------------------------------- polys

def subgroup_gen(log_size: int) -> int:
    return 1 << (31 - log_size)


def canonic_half_coset_initial_index(log_size: int) -> int:
    """Initial index of CanonicCoset(log_size).half_coset() = half_odds(log_size-1)."""
    return subgroup_gen(log_size + 1)


def precompute_twiddles(initial_index: int, log_size: int):
    n = 1 << log_size
    tw = np.zeros(n, np.uint32)
    itw = np.zeros(n, np.uint32)
    lib().orc_precompute_twiddles(ctypes.c_uint32(initial_index), ctypes.c_uint32(log_size), _p(tw), _p(itw))
    return tw, itw


def canonic_twiddles(domain_log_size: int):
    """Twiddle tree rooted at CanonicCoset(domain_log_size).half_coset()."""
    return precompute_twiddles(canonic_half_coset_initial_index(domain_log_size), domain_log_size - 1)


def interpolate(evals, itw: np.ndarray) -> np.ndarray:
    v = _u32(evals).copy()
    lib().orc_interpolate(_p(v), ctypes.c_uint32(v.size.bit_length() - 1), _p(itw),
                          ctypes.c_uint32(itw.size.bit_length() - 1))
    return v


def interpolate_on_subdomain(evals, itw_sub: np.ndarray, parent_log_size: int) -> np.ndarray:
    """Interpolation on the bit-reversed prefix of CanonicCoset(parent_log_size) of the evaluations'
    size, with that subdomain's twiddle tree (extract_subdomain_twiddles)."""
    v = _u32(evals).copy()
    lib().orc_interpolate_on(_p(v), ctypes.c_uint32(v.size.bit_length() - 1), _p(itw_sub),
                             ctypes.c_uint32(itw_sub.size.bit_length() - 1),
                             ctypes.c_uint32(canonic_half_coset_initial_index(parent_log_size)))
    return v


def evaluate(coeffs, log_n: int, tw: np.ndarray) -> np.ndarray:
    c = _u32(coeffs)
    out = np.zeros(1 << log_n, np.uint32)
    lib().orc_evaluate(_p(c), ctypes.c_uint32(c.size.bit_length() - 1), _p(out), ctypes.c_uint32(log_n),
                       _p(tw), ctypes.c_uint32(tw.size.bit_length() - 1))
    return out


def interpolate_batch(cols, itw: np.ndarray):
    cols = [_u32(c).copy() for c in cols]
    logs = _u32([c.size.bit_length() - 1 for c in cols])
    lib().orc_interpolate_batch(_ptr_array(cols), _p(logs), ctypes.c_uint32(len(cols)), _p(itw),
                                ctypes.c_uint32(itw.size.bit_length() - 1))
    return cols


def evaluate_batch(coeffs, log_ns, tw: np.ndarray):
    coeffs = [_u32(c) for c in coeffs]
    outs = [np.zeros(1 << int(l), np.uint32) for l in log_ns]
    lc = _u32([c.size.bit_length() - 1 for c in coeffs])
    ln = _u32(log_ns)
    lib().orc_evaluate_batch(_ptr_array(coeffs), _p(lc), _ptr_array(outs), _p(ln), ctypes.c_uint32(len(coeffs)),
                             _p(tw), ctypes.c_uint32(tw.size.bit_length() - 1))
    return outs


def eval_at_point(coeffs, px, py):
    c, x, y = _u32(coeffs), _u32(px), _u32(py)
    out = np.zeros(4, np.uint32)
    lib().orc_eval_at_point(_p(c), ctypes.c_uint32(c.size.bit_length() - 1), _p(x), _p(y), _p(out))
    return out


# ---------------------------------------------------------------- Merkle

def merkle_build_leaves(sorted_cols, lifting_log_size: int) -> np.ndarray:
    cols = [_u32(c) for c in sorted_cols]
    logs = _u32([c.size.bit_length() - 1 for c in cols])
    n = 1 if not cols else 1 << lifting_log_size
    out = np.zeros((n, 32), np.uint8)
    lib().orc_merkle_build_leaves(_ptr_array(cols), _p(logs), ctypes.c_uint32(len(cols)),
                                  ctypes.c_uint32(lifting_log_size), _p(out))
    return out


def merkle_build_next_layer(prev: np.ndarray) -> np.ndarray:
    prev = np.ascontiguousarray(prev, dtype=np.uint8).reshape(-1, 32)
    n = prev.shape[0] // 2
    out = np.zeros((n, 32), np.uint8)
    lib().orc_merkle_build_next_layer(_p(prev), ctypes.c_uint32(n.bit_length() - 1), _p(out))
    return out


def merkle_commit(cols, lifting_log_size: int, with_layers: bool = False):
    """Returns the root (32 bytes), or (root, [layers leaves-first]) when asked."""
    cols = [_u32(c) for c in cols]
    logs = _u32([c.size.bit_length() - 1 for c in cols])
    root = np.zeros(32, np.uint8)
    layers = None
    if with_layers:
        total = (1 << (lifting_log_size + 1)) - 1 if cols else 1
        layers = np.zeros((total, 32), np.uint8)
    lib().orc_merkle_commit(_ptr_array(cols), _p(logs), ctypes.c_uint32(len(cols)),
                            ctypes.c_uint32(lifting_log_size), _p(root),
                            _p(layers) if layers is not None else None)
    if not with_layers:
        return root.tobytes()
    out, off = [], 0
    for k in range(lifting_log_size, -1, -1):
        out.append(layers[off:off + (1 << k)].copy())
        off += 1 << k
    return root.tobytes(), out


# ---------------------------------------------------------------- FRI

def fold_line(coords, line_initial_index: int, alpha):
    """coords: 4 arrays (SoA QM31) on the line domain x(coset(initial, log n))."""
    ins = [_u32(c) for c in coords]
    n = ins[0].size
    outs = [np.zeros(n // 2, np.uint32) for _ in range(4)]
    a = _u32(alpha)
    lib().orc_fold_line(_ptr_array(ins), ctypes.c_uint32(line_initial_index),
                        ctypes.c_uint32(n.bit_length() - 1), _p(a), _ptr_array(outs))
    return outs


def fold_circle_into_line(coords, alpha):
    ins = [_u32(c) for c in coords]
    n = ins[0].size
    outs = [np.zeros(n // 2, np.uint32) for _ in range(4)]
    a = _u32(alpha)
    lib().orc_fold_circle_into_line(_ptr_array(ins), ctypes.c_uint32(n.bit_length() - 1), _p(a),
                                    _ptr_array(outs))
    return outs


def line_domain_initial_index(line_log_size: int) -> int:
    """LineDomain(Coset::half_odds(line_log_size)) — the first FRI line domain."""
    return subgroup_gen(line_log_size + 2)


def double_index(idx: int) -> int:
    return (idx * 2) & ((1 << 31) - 1)


# ---------------------------------------------------------------- channel

def blake2s(data: bytes) -> bytes:
    buf = np.frombuffer(bytes(data), dtype=np.uint8).copy() if data else np.zeros(1, np.uint8)
    out = np.zeros(32, np.uint8)
    lib().orc_blake2s(_p(buf), ctypes.c_uint64(len(data)), _p(out))
    return out.tobytes()


class Blake2sChannel:
    """Blake2sChannel (crates/stwo/src/core/channel/blake2s.rs:16-118) over the C oracle."""

    def __init__(self, digest: bytes = bytes(32)):
        self.ch = Channel()
        ctypes.memmove(self.ch.digest, digest, 32)
        self.ch.n_draws = 0

    @property
    def digest(self) -> bytes:
        return bytes(self.ch.digest)

    @property
    def n_draws(self) -> int:
        return self.ch.n_draws

    def mix_u32s(self, words):
        w = _u32(words)
        lib().orc_channel_mix_u32s(ctypes.byref(self.ch), _p(w) if w.size else None, ctypes.c_uint32(w.size))

    def mix_u64(self, v: int):
        lib().orc_channel_mix_u64(ctypes.byref(self.ch), ctypes.c_uint64(v))

    def mix_felts(self, felts):
        f = _u32(felts).reshape(-1)
        lib().orc_channel_mix_felts(ctypes.byref(self.ch), _p(f), ctypes.c_uint32(f.size // 4))

    def mix_root(self, root: bytes):
        r = np.frombuffer(root, np.uint8).copy()
        lib().orc_channel_mix_root(ctypes.byref(self.ch), _p(r))

    def draw_u32s(self):
        out = np.zeros(8, np.uint32)
        lib().orc_channel_draw_u32s(ctypes.byref(self.ch), _p(out))
        return out

    def draw_secure_felt(self):
        out = np.zeros(4, np.uint32)
        lib().orc_channel_draw_secure_felt(ctypes.byref(self.ch), _p(out))
        return out

    def draw_queries(self, log_domain_size: int, n_queries: int):
        out = np.zeros(n_queries, np.uint32)
        lib().orc_channel_draw_queries(ctypes.byref(self.ch), ctypes.c_uint32(log_domain_size),
                                       ctypes.c_uint32(n_queries), _p(out))
        return out

    def verify_pow_nonce(self, n_bits: int, nonce: int) -> bool:
        d = np.frombuffer(self.digest, np.uint8).copy()
        return bool(lib().orc_verify_pow_nonce(_p(d), n_bits, nonce))


def grind(digest: bytes, n_bits: int) -> int:
    d = np.frombuffer(digest, np.uint8).copy()
    return int(lib().orc_grind(_p(d), n_bits))


def pow_prefixed_digest(digest: bytes, n_bits: int) -> bytes:
    d = np.frombuffer(digest, np.uint8).copy()
    out = np.zeros(32, np.uint8)
    lib().orc_pow_prefixed_digest(_p(d), ctypes.c_uint32(n_bits), _p(out))
    return out.tobytes()


# ------------------------------------------------------- accumulation / PCS

def _soa(coords):
    return [_u32(c) for c in coords]


def accumulate(col, other):
    col = [_u32(c).copy() for c in col]
    other = _soa(other)
    lib().orc_accumulate(_ptr_array(col), _ptr_array(other), ctypes.c_uint64(col[0].size))
    return col


def generate_secure_powers(felt, n: int):
    f = _u32(felt)
    out = np.zeros(4 * max(n, 1), np.uint32)
    lib().orc_generate_secure_powers(_p(f), ctypes.c_uint32(n), _p(out))
    return out[: 4 * n].reshape(n, 4)


def lift_and_accumulate(cols):
    """cols: list of SoA QM31 columns (4 arrays each), strictly increasing length."""
    cols = [[_u32(c).copy() for c in col] for col in cols]
    flat = [c for col in cols for c in col]
    logs = _u32([col[0].size.bit_length() - 1 for col in cols])
    lib().orc_lift_and_accumulate(_ptr_array(flat), _p(logs), ctypes.c_uint32(len(cols)))
    return cols[-1]


def barycentric_weights(log_n: int, px, py):
    out = [np.zeros(1 << log_n, np.uint32) for _ in range(4)]
    x, y = _u32(px), _u32(py)
    lib().orc_barycentric_weights(ctypes.c_uint32(log_n), _p(x), _p(y), _ptr_array(out))
    return out


def barycentric_eval(evals, weights):
    e = _u32(evals)
    w = _soa(weights)
    out = np.zeros(4, np.uint32)
    lib().orc_barycentric_eval(_p(e), ctypes.c_uint32(e.size.bit_length() - 1), _ptr_array(w), _p(out))
    return out


def line_coeffs(py, value, alpha):
    y, v, a = _u32(py), _u32(value), _u32(alpha)
    out = np.zeros(12, np.uint32)
    lib().orc_line_coeffs(_p(y), _p(v), _p(a), _p(out))
    return out.reshape(3, 4)


def accumulate_numerators(cols, log_blowup: int, coeffs):
    """cols: the batch's columns (same log size); coeffs: (n_terms, 3, 4) (a, b, c)."""
    cols = [_u32(c) for c in cols]
    co = np.ascontiguousarray(np.asarray(coeffs, np.uint32).reshape(-1))
    log_size = cols[0].size.bit_length() - 1
    rows = 1 << (log_size - log_blowup)
    out = [np.zeros(rows, np.uint32) for _ in range(4)]
    fl = np.zeros(4, np.uint32)
    lib().orc_accumulate_numerators(_ptr_array(cols), ctypes.c_uint32(len(cols)), ctypes.c_uint32(log_size),
                                    ctypes.c_uint32(log_blowup), _p(co), _ptr_array(out), _p(fl))
    return out, fl


def quotients_on_subdomain(accs, points, first_linear, lifting_log_size: int, log_blowup: int):
    """accs: per sample point a SoA column; points: per point (x[4], y[4])."""
    accs = [[_u32(c) for c in a] for a in accs]
    flat = [c for a in accs for c in a]
    logs = _u32([a[0].size.bit_length() - 1 for a in accs])
    pts = np.ascontiguousarray(np.asarray([np.concatenate([_u32(x), _u32(y)]) for x, y in points],
                                          np.uint32).reshape(-1))
    fl = np.ascontiguousarray(np.asarray(first_linear, np.uint32).reshape(-1))
    rows = 1 << (lifting_log_size - log_blowup)
    out = [np.zeros(rows, np.uint32) for _ in range(4)]
    lib().orc_quotients_on_subdomain(_ptr_array(flat), _p(logs), ctypes.c_uint32(len(accs)), _p(pts), _p(fl),
                                     ctypes.c_uint32(lifting_log_size), ctypes.c_uint32(log_blowup), _ptr_array(out))
    return out


def decompose(coords):
    ins = _soa(coords)
    n = ins[0].size
    out = [np.zeros(n, np.uint32) for _ in range(4)]
    lam = np.zeros(4, np.uint32)
    lib().orc_decompose(_ptr_array(ins), ctypes.c_uint32(n.bit_length() - 1), _ptr_array(out), _p(lam))
    return out, lam


def random_point_from_t(t):
    tt = _u32(t)
    x, y = np.zeros(4, np.uint32), np.zeros(4, np.uint32)
    lib().orc_random_point_from_t(_p(tt), _p(x), _p(y))
    return x, y


def extract_subdomain_twiddles(buf: np.ndarray, domain_log_size: int, subdomain_log_size: int) -> np.ndarray:
    """TwiddleBuffer::extract_subdomain_twiddles (crates/stwo/src/prover/poly/twiddles.rs:40-76)."""
    dh, sh = domain_log_size - 1, subdomain_log_size - 1
    bh = buf.size.bit_length() - 1
    assert sh <= dh <= bh
    skip = bh - dh
    bsz = 1 << bh
    out = []
    for layer in range(sh):
        root_layer = skip + layer
        start = bsz - (bsz >> root_layer)
        out.append(buf[start:start + (1 << (sh - 1 - layer))])
    out.append(buf[-1:])
    return np.concatenate(out).astype(np.uint32)


# ------------------------------------------------------------ Wide-Fibonacci

def wide_fib_trace(a0, b0, n_cols: int):
    a, b = _u32(a0), _u32(b0)
    n = a.size
    cols = [np.zeros(n, np.uint32) for _ in range(n_cols)]
    lib().orc_wide_fib_trace(_p(a), _p(b), ctypes.c_uint32(n.bit_length() - 1), ctypes.c_uint32(n_cols),
                             _ptr_array(cols))
    return cols


def wide_fib_composition(cols, eval_log: int, trace_log: int, rc, out=None):
    """rc: (n_cols - 2, 4) reversed random-coefficient powers; out: SoA accumulator (added to)."""
    cols = [_u32(c) for c in cols]
    r = np.ascontiguousarray(np.asarray(rc, np.uint32).reshape(-1))
    if out is None:
        out = [np.zeros(1 << eval_log, np.uint32) for _ in range(4)]
    out = [_u32(o).copy() for o in out]
    lib().orc_wide_fib_composition(_ptr_array(cols), ctypes.c_uint32(len(cols)), ctypes.c_uint32(eval_log),
                                   ctypes.c_uint32(trace_log), _p(r), _ptr_array(out))
    return out


def prev_rows(trace_log: int, eval_log: int) -> np.ndarray:
    """The previous-row index of every row of a bit-reversed evaluation domain (orc_prev_row)."""
    out = np.zeros(1 << eval_log, np.uint64)
    lib().orc_prev_rows(ctypes.c_uint32(trace_log), ctypes.c_uint32(eval_log), _p(out))
    return out.astype(np.int64)


def offset_rows(offset: int, trace_log: int, eval_log: int) -> np.ndarray:
    """The row `offset` trace steps from every row of a bit-reversed evaluation domain
    (orc_offset_row)."""
    out = np.zeros(1 << eval_log, np.uint64)
    lib().orc_offset_rows(ctypes.c_int64(offset), ctypes.c_uint32(trace_log), ctypes.c_uint32(eval_log), _p(out))
    return out.astype(np.int64)


def vanishing_inverses(eval_log: int, trace_log: int, log_expansion: int = 0) -> np.ndarray:
    """1 / V_trace at every row of CanonicCoset(eval_log) in bit-reversed order, each row's point
    computed from its index (the denominators of evaluate_constraint_quotients_on_domain,
    crates/constraint-framework/src/prover/component_prover.rs:101-108). With log_expansion e the
    domain is CanonicCoset(eval_log + e).circle_domain().split(e).0 (subdomain_eval_domain,
    component_prover.rs:234-238): the larger domain's initial point, the same step."""
    n = 1 << eval_log
    hs = n >> 1
    half_init = 1 << (31 - (eval_log + log_expansion + 1))
    half_step = (1 << (31 - (eval_log - 1))) if eval_log >= 1 else 0
    mask = (1 << 31) - 1
    nat = bit_reverse(np.arange(n, dtype=np.uint32)).astype(np.int64) if n > 1 else np.zeros(1, np.int64)
    xs = np.zeros(n, np.int64)
    for r in range(n):
        j = int(nat[r])
        t = (half_init + j * half_step) & mask if j < hs else (-(half_init + (j - hs) * half_step)) & mask
        xs[r] = int(circle_index_to_point(t)[0])
    for _ in range(trace_log - 1):
        xs = (2 * xs * xs - 1) % P
    return np.asarray([pow(int(x), P - 2, P) for x in xs], np.int64)


def logup_running_sum(values, z):
    v, zz = _u32(values), _u32(z)
    n = v.size
    out = [np.zeros(n, np.uint32) for _ in range(4)]
    claimed = np.zeros(4, np.uint32)
    lib().orc_logup_running_sum(_p(v), ctypes.c_uint32(n.bit_length() - 1), _p(zz), _ptr_array(out), _p(claimed))
    return out, claimed


def logup_combine(values, alpha_powers, z):
    """LookupElements::combine per row: sum_i alpha_powers[i] values[i] - z (4 coordinate arrays)."""
    vs = [_u32(v) for v in values]
    n = vs[0].size
    aw = np.ascontiguousarray(np.asarray(alpha_powers, np.uint32).reshape(-1))
    zz = _u32(z)
    out = [np.zeros(n, np.uint32) for _ in range(4)]
    lib().orc_logup_combine(_ptr_array(vs), ctypes.c_uint32(len(vs)), ctypes.c_uint32(n.bit_length() - 1), _p(aw),
                            _p(zz), _ptr_array(out))
    return out


def logup_gen_col(numerator, denominator, prev=None):
    """LogupColGenerator (write_frac for every row, finalize_col): numerator / denominator + prev.
    numerator: 4 coordinate arrays (QM31) or one M31 array; denominator, prev: 4 arrays each."""
    den = [_u32(c) for c in denominator]
    n = den[0].size
    out = [np.zeros(n, np.uint32) for _ in range(4)]
    if isinstance(numerator, (list, tuple)):
        keep = [_u32(c) for c in numerator]
        num, num_m31 = _ptr_array(keep), None
    else:
        keep = [_u32(numerator)]
        num, num_m31 = None, _p(keep[0])
    pvs = [_u32(c) for c in prev] if prev is not None else []
    pv = _ptr_array(pvs) if prev is not None else None
    lib().orc_logup_gen_col(num, num_m31, _ptr_array(den), pv, ctypes.c_uint32(n.bit_length() - 1), _ptr_array(out))
    del keep, pvs
    return out


def logup_finalize_last(col):
    """LogupTraceGenerator::finalize_last on a copy of col: (the running-sum column, claimed sum)."""
    out = [_u32(c).copy() for c in col]
    n = out[0].size
    claimed = np.zeros(4, np.uint32)
    lib().orc_logup_finalize_last(_ptr_array(out), ctypes.c_uint32(n.bit_length() - 1), _p(claimed))
    return out, claimed


# ---------------------------------------------------------------- Poseidon2 AIR

POSEIDON_COLS = 1264
POSEIDON_INTERACTION_COLS = 32
POSEIDON_CONSTRAINTS = 1144


def poseidon_m4(x):
    v = _u32(x).copy()
    lib().orc_poseidon_m4(_p(v))
    return v


def poseidon_external(s):
    v = _u32(s).copy()
    lib().orc_poseidon_external(_p(v))
    return v


def poseidon_internal(s):
    v = _u32(s).copy()
    lib().orc_poseidon_internal(_p(v))
    return v


def poseidon_trace(log_n: int):
    cols = [np.zeros(1 << log_n, np.uint32) for _ in range(POSEIDON_COLS)]
    lib().orc_poseidon_trace(ctypes.c_uint32(log_n), _ptr_array(cols))
    return cols


def poseidon_interaction(trace, z, alpha):
    t = [_u32(c) for c in trace]
    n = t[0].size
    zz, aa = _u32(z), _u32(alpha)
    out = [np.zeros(n, np.uint32) for _ in range(POSEIDON_INTERACTION_COLS)]
    claimed = np.zeros(4, np.uint32)
    lib().orc_poseidon_interaction(_ptr_array(t), ctypes.c_uint32(n.bit_length() - 1), _p(zz), _p(aa),
                                   _ptr_array(out), _p(claimed))
    return out, claimed


def poseidon_composition(trace, inter, trace_log: int, lookup, claimed, rc, out=None):
    """trace / inter on the evaluation domain; lookup = z || alpha (8 words); rc: (1144, 4) powers.
    Adds the row quotients into out (4 coordinate arrays), created when None."""
    t = [_u32(c) for c in trace]
    it = [_u32(c) for c in inter]
    n = t[0].size
    lk, cl, r = _u32(lookup), _u32(claimed), _u32(np.asarray(rc).reshape(-1))
    if out is None:
        out = [np.zeros(n, np.uint32) for _ in range(4)]
    out = [_u32(o) for o in out]
    lib().orc_poseidon_composition(_ptr_array(t), _ptr_array(it), ctypes.c_uint32(n.bit_length() - 1),
                                   ctypes.c_uint32(trace_log), _p(lk), _p(cl), _p(r), _ptr_array(out))
    return out


def logup_composition(values, inter, trace_log: int, z, claimed, rc, out=None):
    """A single-column LogUp component's constraint quotients on the evaluation domain of `values`,
    added to out (4 coordinate arrays, created when None)."""
    v = _u32(values)
    it = [_u32(c) for c in inter]
    n = v.size
    if out is None:
        out = [np.zeros(n, np.uint32) for _ in range(4)]
    out = [_u32(o) for o in out]
    zz, cl, r = _u32(z), _u32(claimed), _u32(rc)
    lib().orc_logup_composition(_p(v), _ptr_array(it), ctypes.c_uint32(n.bit_length() - 1), ctypes.c_uint32(trace_log),
                                _p(zz), _p(cl), _p(r), _ptr_array(out))
    return out


# ------------------------------------------------------------ whole proofs (oracle_prover.c)

class ProofError(RuntimeError):
    """A status other than 0 from the oracle's prover (1: constraints not satisfied)."""


_PROOF_CAPACITY = 1 << 23


def _fri_words(fri):
    """(pow_bits, log_blowup_factor, log_last_layer_degree_bound, n_queries[, fold_step])."""
    f = list(fri) + [1] * (5 - len(fri))
    return np.asarray(f, np.uint32)


def prove_fib_and_lookups(fri, fib_traces, fib_log_sizes, lookup_values=(), lookup_log_sizes=(), check=True):
    """The whole proof of Wide-Fibonacci components (fib_traces[k]: the columns of component k,
    evaluations on its trace domain) and single-column LogUp components (their looked-up values),
    by the oracle's restatement of prove_ex. Returns (proof bytes as u64 LE felts, claimed sums)."""
    cols = [_u32(c) for t in fib_traces for c in t]
    n_cols = _u32([len(t) for t in fib_traces])
    logs = _u32(list(fib_log_sizes))
    vals = [_u32(v) for v in lookup_values]
    llogs = _u32(list(lookup_log_sizes)) if len(lookup_log_sizes) else np.zeros(1, np.uint32)
    claimed = np.zeros((max(1, len(vals)), 4), np.uint32)
    words = np.zeros(_PROOF_CAPACITY, np.uint64)
    n = ctypes.c_size_t(0)
    fw = _fri_words(fri)
    L = lib()
    L.orc_prove_fib_and_lookups.restype = ctypes.c_int
    rc = L.orc_prove_fib_and_lookups(_p(fw), ctypes.c_uint32(len(fib_traces)), _p(n_cols), _p(logs),
                                     _ptr_array(cols) if cols else None, ctypes.c_uint32(len(vals)), _p(llogs),
                                     _ptr_array(vals) if vals else None, ctypes.c_int(1 if check else 0),
                                     _p(claimed), _p(words), ctypes.c_size_t(words.size), ctypes.byref(n))
    if rc != 0:
        raise ProofError(f"orc_prove_fib_and_lookups returned {rc}")
    return (words[:n.value].astype("<u8").tobytes(),
            [tuple(int(x) for x in row) for row in claimed[:len(vals)]])


def prove_poseidon(fri, log_n_rows: int) -> bytes:
    """The Poseidon2 AIR's proof at 2^log_n_rows rows by the oracle's restatement of prove_ex (the
    words the reference computes before its sanity check, which this AIR fails when lifted)."""
    words = np.zeros(_PROOF_CAPACITY, np.uint64)
    n = ctypes.c_size_t(0)
    fw = _fri_words(fri)
    L = lib()
    L.orc_prove_poseidon.restype = ctypes.c_int
    rc = L.orc_prove_poseidon(_p(fw), ctypes.c_uint32(log_n_rows), _p(words), ctypes.c_size_t(words.size),
                              ctypes.byref(n))
    if rc != 0:
        raise ProofError(f"orc_prove_poseidon returned {rc}")
    return words[:n.value].astype("<u8").tobytes()
