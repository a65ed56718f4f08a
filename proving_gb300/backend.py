"""Host-side mirror of the reference backend trait family over the C ABI.

Names, argument meanings and error behaviour follow the reference:
`ColumnOps::bit_reverse_column`, `PolyOps::{precompute_twiddles,
interpolate_columns, evaluate_polynomials}`, `MerkleOpsLifted::{build_leaves,
build_next_layer}`, `MerkleProverLifted::commit`, `PackLeavesOps`,
`FriOps::{fold_line, fold_circle_into_line}`, `GrindOps::grind`
(crates/stwo/src/prover/backend/mod.rs:17-35 and the files cited per method).
Misuse raises (the reference panics). Columns live in HBM as torch int32
tensors holding M31 words; torch is used only for device memory and streams.
"""
from __future__ import annotations

import ctypes
import threading
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib

P = (1 << 31) - 1
M31_CIRCLE_LOG_ORDER = 31


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t: torch.Tensor) -> int:
    assert t.is_cuda and t.is_contiguous()
    return t.data_ptr()


def _ptr_table(ts) -> ctypes.Array:
    """Device pointers of the tensors (BaseColumn data: 1-D contiguous CUDA int32, checked when the
    column was made)."""
    return (ctypes.c_void_p * max(1, len(ts)))(*[t.data_ptr() for t in ts])


def _u32_table(vals) -> ctypes.Array:
    arr = (ctypes.c_uint32 * max(1, len(vals)))()
    for i, v in enumerate(vals):
        arr[i] = int(v)
    return arr


def subgroup_gen(log_size: int) -> int:
    return 1 << (M31_CIRCLE_LOG_ORDER - log_size)


# ------------------------------------------------------------------ columns

class BaseColumn:
    """BaseColumn (crates/stwo/src/prover/backend/simd/column.rs:26-30): 2^k M31 words in HBM."""

    def __init__(self, data: torch.Tensor):
        assert data.dtype == torch.int32 and data.dim() == 1 and data.is_cuda
        self.data = data
        self._log_size = data.numel().bit_length() - 1

    @classmethod
    def rows_of(cls, block: torch.Tensor) -> list:
        """The rows of a contiguous (n_cols, 2^k) int32 CUDA block as columns (checked once)."""
        assert block.dtype == torch.int32 and block.dim() == 2 and block.is_cuda and block.is_contiguous()
        log_size = block.shape[1].bit_length() - 1
        cols = []
        for row in block.unbind(0):
            c = cls.__new__(cls)
            c.data, c._log_size = row, log_size
            cols.append(c)
        return cols

    @classmethod
    def zeros(cls, length: int, device="cuda"):
        return cls(torch.zeros(length, dtype=torch.int32, device=device))

    @classmethod
    def uninitialized(cls, length: int, device="cuda"):
        return cls(torch.empty(length, dtype=torch.int32, device=device))

    @classmethod
    def from_cpu(cls, values: np.ndarray, device="cuda"):
        v = np.ascontiguousarray(values, dtype=np.uint32).view(np.int32)
        return cls(torch.from_numpy(v).to(device, non_blocking=False))

    def to_cpu(self) -> np.ndarray:
        return self.data.cpu().numpy().view(np.uint32)

    def __len__(self):
        return self.data.numel()

    @property
    def log_size(self) -> int:
        return self._log_size

    def at(self, i: int) -> int:
        return int(self.data[i].item()) & 0xFFFFFFFF


class _WideFibProofParams(ctypes.Structure):
    """cs_wide_fib_proof_params (include/stwo_cuda.h)."""
    _fields_ = [("n_components", ctypes.c_uint32), ("n_cols", ctypes.c_void_p), ("log_sizes", ctypes.c_void_p),
                ("lifting_log_size", ctypes.c_uint32), ("pow_bits", ctypes.c_uint32),
                ("log_blowup_factor", ctypes.c_uint32), ("log_last_layer_degree_bound", ctypes.c_uint32),
                ("n_queries", ctypes.c_uint32), ("d_twiddles", ctypes.c_void_p), ("d_itwiddles", ctypes.c_void_p),
                ("twiddle_log_size", ctypes.c_uint32), ("flags", ctypes.c_uint32), ("fold_step", ctypes.c_uint32)]


PROVE_PLAIN = 1  # CS_PROVE_PLAIN


class _AirComponent(ctypes.Structure):
    """cs_air_component (include/stwo_cuda.h)."""
    _fields_ = [("kernel", ctypes.c_void_p), ("log_size", ctypes.c_uint32), ("constraint_log_degree", ctypes.c_uint32),
                ("n_cols", ctypes.c_uint32), ("offsets", ctypes.c_void_p), ("offsets_start", ctypes.c_void_p),
                ("n_masks", ctypes.c_uint32), ("mask_cols", ctypes.c_void_p), ("mask_trees", ctypes.c_void_p),
                ("program", ctypes.c_void_p), ("n_nodes", ctypes.c_uint32), ("constraints", ctypes.c_void_p),
                ("n_constraints", ctypes.c_uint32), ("params", ctypes.c_void_p), ("param_kinds", ctypes.c_void_p),
                ("n_params", ctypes.c_uint32), ("n_batches", ctypes.c_uint32), ("n_frac_cols", ctypes.c_uint32),
                ("frac_cols", ctypes.c_void_p), ("inter_two", ctypes.c_void_p)]


PROVE_MIX_CLAIMED = 2  # CS_PROVE_MIX_CLAIMED


class SecureColumnByCoords:
    """SecureColumnByCoords (crates/stwo/src/prover/secure_column.rs:13-15): 4 coordinate columns."""

    def __init__(self, columns):
        assert len(columns) == 4
        self.columns = [c if isinstance(c, BaseColumn) else BaseColumn(c) for c in columns]

    @classmethod
    def zeros(cls, length: int):
        return cls(BaseColumn.rows_of(torch.zeros((4, length), dtype=torch.int32, device="cuda")))

    @classmethod
    def uninitialized(cls, length: int):
        return cls(BaseColumn.rows_of(torch.empty((4, length), dtype=torch.int32, device="cuda")))

    @classmethod
    def from_cpu(cls, coords):
        return cls([BaseColumn.from_cpu(c) for c in coords])

    def to_cpu(self):
        return [c.to_cpu() for c in self.columns]

    def __len__(self):
        return len(self.columns[0])

    def at(self, i: int):
        return [c.at(i) for c in self.columns]


@dataclass
class Coset:
    """Coset initial_index + <G_{2^log_size}> (crates/stwo/src/core/circle.rs:262-282)."""
    initial_index: int
    log_size: int

    @staticmethod
    def half_odds(log_size: int) -> "Coset":
        return Coset(subgroup_gen(log_size + 2), log_size)


def canonic_half_coset(log_size: int) -> Coset:
    """CanonicCoset(log_size).half_coset() (crates/stwo/src/core/poly/circle/canonic.rs:61-63)."""
    return Coset.half_odds(log_size - 1)


class TwiddleTree:
    """TwiddleTree (crates/stwo/src/prover/poly/twiddles.rs:10-15) resident in HBM."""

    def __init__(self, root_coset: Coset, twiddles: torch.Tensor, itwiddles: torch.Tensor):
        self.root_coset = root_coset
        self.twiddles = twiddles
        self.itwiddles = itwiddles

    @property
    def log_size(self) -> int:
        return self.root_coset.log_size


# ------------------------------------------------------------------ backend

class LogupTraceGenerator:
    """LogupTraceGenerator (crates/constraint-framework/src/prover/logup.rs:22-130) over device
    columns of 2^log_size rows (bit-reversed circle-domain order): each col_from_fractions adds one
    interaction column, num / den plus the previous column (LogupColGenerator::write_frac for every
    row, then finalize_col, through cs_logup_gen_col); finalize_last turns the last column into the
    shifted running sum (cs_logup_finalize_last) and returns every column's four coordinate
    BaseColumns with the claimed sum, as the reference returns the trace and claimed_sum."""

    def __init__(self, log_size: int):
        self.log_size = log_size
        self.trace: list = []

    def col_from_fractions(self, fractions) -> None:
        """One interaction column from a batch of fractions [(numerator, denominator), ...], summed
        per row (the reference's caller writes the batch's combined fraction, e.g. n0 d1 + n1 d0 over
        d0 d1 for a pair): numerator a SecureColumnByCoords or a BaseColumn of M31 numerators
        (multiplicities), denominator a SecureColumnByCoords."""
        assert fractions, "an interaction column needs at least one fraction"
        n = 1 << self.log_size
        out = SecureColumnByCoords.uninitialized(n)
        out_tab = _ptr_table([c.data for c in out.columns])
        prev = _ptr_table([c.data for c in self.trace[-1].columns]) if self.trace else None
        for numerator, denominator in fractions:
            assert len(denominator) == n and len(numerator) == n
            if isinstance(numerator, SecureColumnByCoords):
                num_tab, num_m31 = _ptr_table([c.data for c in numerator.columns]), None
            else:
                num_tab, num_m31 = None, _ptr(numerator.data)
            # later fractions of the batch add to the column itself (each row reads prev, then writes)
            _lib.call("cs_logup_gen_col", num_tab, num_m31, _ptr_table([c.data for c in denominator.columns]), prev,
                      self.log_size, out_tab, _stream())
            prev = out_tab
        self.trace.append(out)

    def finalize_last(self):
        assert self.trace, "no interaction column to finalize"
        claimed = (ctypes.c_uint32 * 4)()
        _lib.call("cs_logup_finalize_last", _ptr_table([c.data for c in self.trace[-1].columns]), self.log_size,
                  claimed, _stream())
        return [c for col in self.trace for c in col.columns], tuple(int(x) for x in claimed)


def logup_combine(values, alpha_powers, z) -> "SecureColumnByCoords":
    """LookupElements::combine (crates/constraint-framework/src/logup.rs:80-94) per row of the M31
    columns `values`: sum_i alpha_powers[i] values[i] - z (cs_logup_combine)."""
    out = SecureColumnByCoords.uninitialized(len(values[0]))
    aw = np.ascontiguousarray(np.asarray(alpha_powers, np.uint32).reshape(-1))
    assert aw.size == 4 * len(values)
    _lib.call("cs_logup_combine", _ptr_table([v.data for v in values]), len(values), values[0].log_size,
              aw.ctypes.data_as(ctypes.c_void_p), _u32_table(z), _ptr_table([c.data for c in out.columns]),
              _stream())
    return out


_tls = threading.local()


def _words_buffer(cap: int) -> np.ndarray:
    """This thread's buffer for a native prover's felt words, kept across proofs so its pages are
    faulted in once (the proof bytes returned are a copy)."""
    b = getattr(_tls, "words", None)
    if b is None or b.size < cap:
        b = np.empty(cap, np.uint64)
        _tls.words = b
    return b


class CudaBackend:
    """The GB300 backend. Every method enqueues on torch's current CUDA stream."""

    # ColumnOps -------------------------------------------------------------
    @staticmethod
    def bit_reverse_column(col: BaseColumn) -> None:
        _lib.call("cs_bit_reverse_m31", _ptr(col.data), col.log_size, _stream())

    # PolyOps ---------------------------------------------------------------
    @staticmethod
    def precompute_twiddles(coset: Coset) -> TwiddleTree:
        n = 1 << coset.log_size
        tw = torch.empty(n, dtype=torch.int32, device="cuda")
        itw = torch.empty(n, dtype=torch.int32, device="cuda")
        _lib.call("cs_precompute_twiddles", coset.initial_index, coset.log_size, _ptr(tw), _ptr(itw), _stream())
        return TwiddleTree(coset, tw, itw)

    @staticmethod
    def interpolate_columns(columns, twiddles: TwiddleTree) -> None:
        """In place: bit-reversed evaluations on CanonicCoset(log) -> coefficients.
        Columns of several sizes are grouped by size, one batched call per size."""
        by_size = {}
        for c in columns:
            by_size.setdefault(c.log_size, []).append(c)
        for log_size, cols in by_size.items():
            tab = _ptr_table([c.data for c in cols])
            _lib.call("cs_interpolate_columns", tab, len(cols), log_size, _ptr(twiddles.itwiddles),
                      twiddles.log_size, _stream())

    @staticmethod
    def interpolate_columns_into(columns, twiddles: TwiddleTree, out=None):
        """Out of place: the coefficients of `columns` (kept) in new columns."""
        if out is None:
            out = [BaseColumn.uninitialized(len(c)) for c in columns]
        by_size = {}
        for i, c in enumerate(columns):
            by_size.setdefault(c.log_size, []).append(i)
        for log_size, idxs in by_size.items():
            _lib.call("cs_interpolate_columns_into", _ptr_table([columns[i].data for i in idxs]),
                      _ptr_table([out[i].data for i in idxs]), len(idxs), log_size, _ptr(twiddles.itwiddles),
                      twiddles.log_size, _stream())
        return out

    @staticmethod
    def evaluate_polynomials(coeffs, log_size: int, twiddles: TwiddleTree, out=None):
        """Evaluates coefficient columns on CanonicCoset(log_size); returns new columns."""
        if out is None:
            out = [BaseColumn.uninitialized(1 << log_size) for _ in coeffs]
        by_size = {}
        for i, c in enumerate(coeffs):
            by_size.setdefault(c.log_size, []).append(i)
        for lc, idxs in by_size.items():
            src = _ptr_table([coeffs[i].data for i in idxs])
            dst = _ptr_table([out[i].data for i in idxs])
            _lib.call("cs_evaluate_columns", src, dst, len(idxs), lc, log_size, _ptr(twiddles.twiddles),
                      twiddles.log_size, _stream())
        return out

    # MerkleOpsLifted ---------------------------------------------------------
    @staticmethod
    def build_leaves(columns, lifting_log_size: int) -> torch.Tensor:
        """Columns sorted by length; returns (2^L, 8) int32 digests."""
        n = 1 if not columns else 1 << lifting_log_size
        out = torch.empty((n, 8), dtype=torch.int32, device="cuda")
        tab = _ptr_table([c.data for c in columns])
        logs = _u32_table([c.log_size for c in columns])
        _lib.call("cs_merkle_build_leaves", tab, logs, len(columns), lifting_log_size, _ptr(out), _stream())
        return out

    @staticmethod
    def build_next_layer(prev: torch.Tensor) -> torch.Tensor:
        n = prev.shape[0] // 2
        out = torch.empty((n, 8), dtype=torch.int32, device="cuda")
        _lib.call("cs_merkle_build_next_layer", _ptr(prev), n.bit_length() - 1, _ptr(out), _stream())
        return out

    @staticmethod
    def merkle_commit(columns, lifting_log_size: int) -> "MerkleProverLifted":
        """MerkleProverLifted::commit (crates/stwo/src/prover/vcs_lifted/prover.rs:35-80), no leaf packing."""
        total = (1 << (lifting_log_size + 1)) - 1 if columns else 1
        layers = torch.empty((total, 8), dtype=torch.int32, device="cuda")
        tab = _ptr_table([c.data for c in columns])
        logs = _u32_table([c.log_size for c in columns])
        _lib.call("cs_merkle_commit", tab, logs, len(columns), lifting_log_size, _ptr(layers), _stream())
        return MerkleProverLifted(layers, lifting_log_size if columns else 0)

    @staticmethod
    def pack_leaves_input(values) -> list:
        n = len(values[0])
        outs = [BaseColumn.uninitialized(n // 4) for _ in range(16)]
        ins = _ptr_table([v.data for v in values])
        o = _ptr_table([c.data for c in outs])
        _lib.call("cs_pack_leaves_input", ins, n.bit_length() - 1, o, _stream())
        return outs

    # FriOps -------------------------------------------------------------------
    @staticmethod
    def set_fold_plan(log_values_per_thread: int) -> None:
        """cs_fold_set_plan: 2^3 or 2^4 values per thread in the register fold launches."""
        _lib.call("cs_fold_set_plan", log_values_per_thread)

    @staticmethod
    def get_fold_plan() -> int:
        v = ctypes.c_uint32()
        _lib.call("cs_fold_get_plan", ctypes.byref(v))
        return v.value

    @staticmethod
    def fold_line(values: SecureColumnByCoords, alphas, twiddles: TwiddleTree) -> SecureColumnByCoords:
        """fold_line on the line domain x(half_odds(log n)); alphas as in FriOps::fold_line: one
        fold per challenge, only the last layer returned."""
        alphas = [tuple(a) for a in alphas]
        if not alphas:
            raise ValueError("fold_line needs at least one challenge")
        n = len(values)
        dst = SecureColumnByCoords.uninitialized(n >> len(alphas))
        words = _u32_table([w for a in alphas for w in a])
        _lib.call("cs_fold_line_steps", _ptr_table([c.data for c in values.columns]), n.bit_length() - 1,
                  len(alphas), words, _ptr_table([c.data for c in dst.columns]), _ptr(twiddles.itwiddles),
                  twiddles.log_size, _stream())
        return dst

    @staticmethod
    def fold_line_device_alpha(values: SecureColumnByCoords, d_alpha: torch.Tensor,
                               twiddles: TwiddleTree) -> SecureColumnByCoords:
        """fold_line with the challenge in device memory (4 words)."""
        n = len(values)
        dst = SecureColumnByCoords.uninitialized(n // 2)
        _lib.call("cs_fold_line_device_alpha", _ptr_table([c.data for c in values.columns]), n.bit_length() - 1,
                  _ptr(d_alpha), _ptr_table([c.data for c in dst.columns]), _ptr(twiddles.itwiddles),
                  twiddles.log_size, _stream())
        return dst

    @staticmethod
    def fold_circle_into_line_device_alpha(src: SecureColumnByCoords, d_alpha: torch.Tensor,
                                           twiddles: TwiddleTree) -> SecureColumnByCoords:
        """fold_circle_into_line with the challenge in device memory (4 words)."""
        n = len(src)
        dst = SecureColumnByCoords.uninitialized(n // 2)
        _lib.call("cs_fold_circle_into_line_device_alpha", _ptr_table([c.data for c in src.columns]),
                  n.bit_length() - 1, _ptr(d_alpha), _ptr_table([c.data for c in dst.columns]),
                  _ptr(twiddles.itwiddles), twiddles.log_size, _stream())
        return dst

    @staticmethod
    def fold_circle_into_line(src: SecureColumnByCoords, alpha, twiddles: TwiddleTree) -> SecureColumnByCoords:
        n = len(src)
        dst = SecureColumnByCoords.uninitialized(n // 2)
        a = _u32_table(alpha)
        _lib.call("cs_fold_circle_into_line", _ptr_table([c.data for c in src.columns]), n.bit_length() - 1, a,
                  _ptr_table([c.data for c in dst.columns]), _ptr(twiddles.itwiddles), twiddles.log_size, _stream())
        return dst

    @staticmethod
    def decompose(src: SecureColumnByCoords):
        """FriOps::decompose: returns (g, lambda)."""
        n = len(src)
        dst = SecureColumnByCoords.uninitialized(n)
        lam = (ctypes.c_uint32 * 4)()
        _lib.call("cs_decompose", _ptr_table([c.data for c in src.columns]), n.bit_length() - 1,
                  _ptr_table([c.data for c in dst.columns]), lam, _stream())
        return dst, np.array(list(lam), np.uint32)

    # AccumulationOps -------------------------------------------------------------
    @staticmethod
    def accumulate(col: SecureColumnByCoords, other: SecureColumnByCoords) -> None:
        _lib.call("cs_accumulate", _ptr_table([c.data for c in col.columns]),
                  _ptr_table([c.data for c in other.columns]), len(col).bit_length() - 1, _stream())

    @staticmethod
    def generate_secure_powers(felt, n_powers: int) -> np.ndarray:
        out = np.empty((max(1, n_powers), 4), np.uint32)
        _lib.call("cs_generate_secure_powers", _u32_table(felt), n_powers, out.ctypes.data)
        return out[:n_powers]

    @staticmethod
    def lift_and_accumulate(cols):
        """Columns with strictly increasing sizes, updated in place; returns the last (or None)."""
        if not cols:
            return None
        tab = _ptr_table([c.data for col in cols for c in col.columns])
        logs = _u32_table([len(c).bit_length() - 1 for c in cols])
        _lib.call("cs_lift_and_accumulate", tab, logs, len(cols), _stream())
        return cols[-1]

    # out-of-domain sampling ------------------------------------------------------
    @staticmethod
    def barycentric_weights(log_size: int, point) -> SecureColumnByCoords:
        px, py = point
        out = SecureColumnByCoords.uninitialized(1 << log_size)
        _lib.call("cs_barycentric_weights", log_size, _u32_table(px), _u32_table(py),
                  _ptr_table([c.data for c in out.columns]), _stream())
        return out

    @staticmethod
    def barycentric_eval_at_point(evals, weights: SecureColumnByCoords) -> torch.Tensor:
        out = torch.empty((len(evals), 4), dtype=torch.int32, device="cuda")
        _lib.call("cs_barycentric_eval", _ptr_table([e.data for e in evals]), len(evals),
                  len(weights).bit_length() - 1, _ptr_table([c.data for c in weights.columns]), _ptr(out),
                  _stream())
        return out

    @staticmethod
    def eval_at_point(coeffs, point) -> torch.Tensor:
        px, py = point
        out = torch.empty((len(coeffs), 4), dtype=torch.int32, device="cuda")
        _lib.call("cs_eval_at_point", _ptr_table([c.data for c in coeffs]), len(coeffs),
                  coeffs[0].log_size, _u32_table(px), _u32_table(py), _ptr(out), _stream())
        return out

    # QuotientOps -------------------------------------------------------------------
    @staticmethod
    def accumulate_numerators(columns, line_coeffs, log_blowup: int):
        """One sample batch: columns (same size) and their (a, b, c) line coefficients (n, 3, 4).
        Returns (partial_numerators_acc, first_linear_term_acc)."""
        log_size = columns[0].log_size
        out = SecureColumnByCoords.uninitialized(1 << (log_size - log_blowup))
        co = np.ascontiguousarray(np.asarray(line_coeffs, np.uint32).reshape(-1))
        fl = (ctypes.c_uint32 * 4)()
        _lib.call("cs_accumulate_numerators", _ptr_table([c.data for c in columns]), len(columns), log_size,
                  log_blowup, co.ctypes.data, _ptr_table([c.data for c in out.columns]), fl, _stream())
        return out, np.array(list(fl), np.uint32)

    @staticmethod
    def interpolate_on_subdomain(columns, domain_log_size: int, twiddles: TwiddleTree) -> None:
        _lib.call("cs_interpolate_columns_on_subdomain", _ptr_table([c.data for c in columns]), len(columns),
                  columns[0].log_size, domain_log_size, _ptr(twiddles.itwiddles), twiddles.log_size, _stream())

    @staticmethod
    def quotients_on_subdomain(accs, points, first_linear, lifting_log_size: int, log_blowup: int):
        out = SecureColumnByCoords.uninitialized(1 << (lifting_log_size - log_blowup))
        tab = _ptr_table([c.data for a in accs for c in a.columns])
        logs = _u32_table([len(a).bit_length() - 1 for a in accs])
        pts = np.ascontiguousarray(np.concatenate([np.concatenate([np.asarray(x, np.uint32), np.asarray(y, np.uint32)])
                                                   for x, y in points]))
        fl = np.ascontiguousarray(np.asarray(first_linear, np.uint32).reshape(-1))
        _lib.call("cs_quotients_on_subdomain", tab, logs, len(accs), pts.ctypes.data, fl.ctypes.data,
                  lifting_log_size, log_blowup, _ptr_table([c.data for c in out.columns]), _stream())
        return out

    @classmethod
    def compute_quotients_and_combine(cls, accs, points, first_linear, lifting_log_size: int, log_blowup: int,
                                      twiddles: TwiddleTree) -> SecureColumnByCoords:
        """QuotientOps::compute_quotients_and_combine (crates/stwo/src/prover/pcs/quotient_ops.rs:47-52)."""
        q = cls.quotients_on_subdomain(accs, points, first_linear, lifting_log_size, log_blowup)
        cls.interpolate_on_subdomain(q.columns, lifting_log_size, twiddles)
        return SecureColumnByCoords(cls.evaluate_polynomials(q.columns, lifting_log_size, twiddles))

    # AIR (Wide-Fibonacci) ---------------------------------------------------------
    @staticmethod
    def wide_fib_trace(a: BaseColumn, b: BaseColumn, n_cols: int):
        cols = BaseColumn.rows_of(torch.empty((n_cols, len(a)), dtype=torch.int32, device="cuda"))
        _lib.call("cs_wide_fib_trace", _ptr(a.data), _ptr(b.data), a.log_size, n_cols,
                  _ptr_table([c.data for c in cols]), _stream())
        return cols

    @staticmethod
    def wide_fib_composition(evals, trace_log: int, rc, accum: SecureColumnByCoords) -> None:
        """Adds the Wide-Fibonacci constraint quotients to accum (evaluation domain of accum's size)."""
        r = np.ascontiguousarray(np.asarray(rc, np.uint32).reshape(-1))
        _lib.call("cs_wide_fib_composition", _ptr_table([c.data for c in evals]), len(evals),
                  len(accum).bit_length() - 1, trace_log, r.ctypes.data,
                  _ptr_table([c.data for c in accum.columns]), _stream())

    @staticmethod
    def logup_running_sum(values: BaseColumn, z):
        """LogUp interaction column (last-column finalization) for fractions 1 / (z - v)."""
        out = SecureColumnByCoords.uninitialized(len(values))
        claimed = (ctypes.c_uint32 * 4)()
        _lib.call("cs_logup_running_sum", _ptr(values.data), values.log_size, _u32_table(z),
                  _ptr_table([c.data for c in out.columns]), claimed, _stream())
        return out, np.array(list(claimed), np.uint32)

    @staticmethod
    def logup_running_sums(values, z):
        """logup_running_sum for several columns of any sizes in one batch of launches. Returns the
        running-sum columns and the claimed sums as an (n, 4) device tensor (not read back)."""
        outs = [SecureColumnByCoords.uninitialized(len(v)) for v in values]
        claimed = torch.empty((max(1, len(values)), 4), dtype=torch.int32, device="cuda")
        _lib.call("cs_logup_running_sums", len(values), _ptr_table([v.data for v in values]),
                  _u32_table([v.log_size for v in values]), _u32_table(z),
                  _ptr_table([c.data for o in outs for c in o.columns]), _ptr(claimed), _stream())
        return outs, claimed[:len(values)]

    @staticmethod
    def logup_composition(values: BaseColumn, inter: SecureColumnByCoords, trace_log: int, z, claimed, rc,
                          accum: SecureColumnByCoords) -> None:
        """Adds a single-column LogUp component's constraint quotients (evaluation domain of `values`)."""
        _lib.call("cs_logup_composition", _ptr(values.data), _ptr_table([c.data for c in inter.columns]),
                  values.log_size, trace_log, _u32_table(z), _u32_table(claimed), _u32_table(rc),
                  _ptr_table([c.data for c in accum.columns]), _stream())

    @staticmethod
    def logup_compositions(values, inters, trace_log: int, z, claimed, rcs, accum: SecureColumnByCoords) -> None:
        """logup_composition for several components of the same trace size, summed per row before
        they are added to the accumulator (one launch per 24 components)."""
        if not values:
            return
        _lib.call("cs_logup_compositions", len(values), _ptr_table([v.data for v in values]),
                  _ptr_table([c.data for it in inters for c in it.columns]), values[0].log_size, trace_log,
                  _u32_table(z), _u32_table([w for c in claimed for w in c]), _u32_table([w for r in rcs for w in r]),
                  _ptr_table([c.data for c in accum.columns]), _stream())

    @staticmethod
    def _proof_params(n_cols, log_sizes, lifting_log_size: int, fri_params, twiddles: TwiddleTree, plain=False):
        params = _WideFibProofParams()
        keep = ((ctypes.c_uint32 * max(1, len(n_cols)))(*n_cols), (ctypes.c_uint32 * max(1, len(log_sizes)))(*log_sizes))
        params.n_components = len(n_cols)
        params.n_cols = ctypes.cast(keep[0], ctypes.c_void_p)
        params.log_sizes = ctypes.cast(keep[1], ctypes.c_void_p)
        params.lifting_log_size = lifting_log_size
        # (pow_bits, log_blowup_factor, log_last_layer_degree_bound, n_queries[, fold_step])
        params.pow_bits, params.log_blowup_factor, params.log_last_layer_degree_bound, params.n_queries = fri_params[:4]
        params.fold_step = fri_params[4] if len(fri_params) > 4 else 1
        params.d_twiddles = twiddles.twiddles.data_ptr()
        params.d_itwiddles = twiddles.itwiddles.data_ptr()
        params.twiddle_log_size = twiddles.log_size
        params.flags = PROVE_PLAIN if plain else 0
        return params, keep

    @staticmethod
    def prove_wide_fib_native(traces, log_sizes, fri_params, twiddles: TwiddleTree, plain=False) -> bytes:
        """cs_prove_wide_fib: the whole proof of Wide-Fibonacci components with the host work in
        native code. traces[k]: component k's columns (BaseColumns of 2^log_sizes[k] evaluations,
        interpolated in place). fri_params: (pow_bits, log_blowup_factor,
        log_last_layer_degree_bound, n_queries[, fold_step]). Returns the proof bytes (u64 LE felts)."""
        return CudaBackend.prove_fib_and_lookups_native(traces, log_sizes, [], [], fri_params, twiddles, plain)[0]

    @staticmethod
    def prove_fib_and_lookups_native(traces, log_sizes, lookup_values, lookup_logs, fri_params,
                                     twiddles: TwiddleTree, plain=False):
        """cs_prove_fib_and_lookups: Wide-Fibonacci components and single-column LogUp components
        (lookup_values: BaseColumns on their trace domains, kept). Returns (proof bytes, claimed sums)."""
        cols = [c for t in traces for c in t]
        lifting = max(list(log_sizes) + list(lookup_logs)) + fri_params[1]
        params, keep = CudaBackend._proof_params([len(t) for t in traces], log_sizes, lifting, fri_params, twiddles,
                                                 plain)
        n = ctypes.c_size_t(0)
        cap = 1 << 22
        words = _words_buffer(cap)
        claimed = np.zeros((max(1, len(lookup_values)), 4), np.uint32)
        _lib.call("cs_prove_fib_and_lookups", ctypes.byref(params), _ptr_table([c.data for c in cols]),
                  len(lookup_values), _ptr_table([v.data for v in lookup_values]), _u32_table(lookup_logs),
                  claimed.ctypes.data, words.ctypes.data, cap, ctypes.byref(n), _stream())
        del keep
        return (words[:n.value].astype("<u8").tobytes(),
                [tuple(int(x) for x in row) for row in claimed[:len(lookup_values)]])

    @staticmethod
    def prove_air_native(components, trace, lifting_log_size: int, fri_params, twiddles: TwiddleTree,
                         plain=False, mix_claimed=False) -> bytes:
        """cs_prove_air: components written against the constraint evaluator, proved in native code.
        components: dicts with kernel (handle), log_size, degree, offsets (per trace column),
        masks ((column, tree) per kernel mask), nodes ((n, 5) program), constraints (nodes),
        params (QM31 words), kinds (per parameter), n_batches, frac_cols, inter_two; trace: every
        component's columns in order (BaseColumns on their trace domains). Returns the proof bytes."""
        keep = []

        def arr(values, dtype):
            a = np.ascontiguousarray(np.asarray(values, dtype).reshape(-1))
            keep.append(a)
            return a.ctypes.data if a.size else None
        comps = (_AirComponent * len(components))()
        for k, spec in enumerate(components):
            c = comps[k]
            handle = spec["kernel"]
            c.kernel = handle.value if isinstance(handle, ctypes.c_void_p) else handle
            c.log_size, c.constraint_log_degree = spec["log_size"], spec["degree"]
            offs = spec["offsets"]
            c.n_cols = len(offs)
            c.offsets = arr([x for o in offs for x in o], np.int32)
            c.offsets_start = arr(np.cumsum([0] + [len(o) for o in offs]), np.uint32)
            c.n_masks = len(spec["masks"])
            c.mask_cols = arr([m[0] for m in spec["masks"]], np.uint32)
            c.mask_trees = arr([m[1] for m in spec["masks"]], np.uint32)
            c.program, c.n_nodes = arr(spec["nodes"], np.uint32), len(spec["nodes"])
            c.constraints, c.n_constraints = arr(spec["constraints"], np.uint32), len(spec["constraints"])
            c.params, c.param_kinds = arr(spec["params"], np.uint32), arr(spec["kinds"], np.uint32)
            c.n_params = len(spec["kinds"])
            c.n_batches = spec["n_batches"]
            c.n_frac_cols, c.frac_cols = len(spec["frac_cols"]), arr(spec["frac_cols"], np.uint32)
            c.inter_two = arr(spec["inter_two"], np.uint32)
        params, keep2 = CudaBackend._proof_params([], [], lifting_log_size, fri_params, twiddles, plain)
        if mix_claimed:
            params.flags |= PROVE_MIX_CLAIMED
        n = ctypes.c_size_t(0)
        cap = 1 << 22
        words = _words_buffer(cap)
        _lib.call("cs_prove_air", ctypes.byref(params), comps, len(components), _ptr_table([c.data for c in trace]),
                  words.ctypes.data, cap, ctypes.byref(n), _stream())
        del keep, keep2
        return words[:n.value].astype("<u8").tobytes()

    @staticmethod
    def prove_poseidon_native(log_n_rows: int, fri_params, twiddles: TwiddleTree, plain=False) -> bytes:
        """cs_prove_poseidon: the Poseidon2 AIR's proof (2^log_n_rows rows, 8 instances per row), trace
        generated on the device, the words the reference computes before its sanity check."""
        params, keep = CudaBackend._proof_params([], [], log_n_rows + 2, fri_params, twiddles, plain)
        n = ctypes.c_size_t(0)
        cap = 1 << 22
        words = _words_buffer(cap)
        _lib.call("cs_prove_poseidon", log_n_rows, ctypes.byref(params), words.ctypes.data, cap, ctypes.byref(n),
                  _stream())
        del keep
        return words[:n.value].astype("<u8").tobytes()

    # Poseidon2 AIR ------------------------------------------------------------
    POSEIDON_COLS = 1264
    POSEIDON_INTERACTION_COLS = 32
    POSEIDON_CONSTRAINTS = 1144

    @classmethod
    def poseidon_trace(cls, log_n: int):
        """gen_trace (crates/examples/src/poseidon/mod.rs:195-275): 1264 columns of 2^log_n words,
        held in one (1264, 2^log_n) device block."""
        block = torch.empty((cls.POSEIDON_COLS, 1 << log_n), dtype=torch.int32, device="cuda")
        cols = BaseColumn.rows_of(block)
        _lib.call("cs_poseidon_trace", log_n, _ptr_table([c.data for c in cols]), _stream())
        return cols

    @classmethod
    def poseidon_interaction(cls, trace, lookup):
        """gen_interaction_trace (mod.rs:277-303): 32 interaction columns and the claimed sum.
        lookup: z || alpha (8 words)."""
        n = len(trace[0])
        block = torch.empty((cls.POSEIDON_INTERACTION_COLS, n), dtype=torch.int32, device="cuda")
        out = BaseColumn.rows_of(block)
        claimed = (ctypes.c_uint32 * 4)()
        _lib.call("cs_poseidon_interaction", _ptr_table([c.data for c in trace]), trace[0].log_size,
                  _u32_table(lookup), _ptr_table([c.data for c in out]), claimed, _stream())
        return out, np.array(list(claimed), np.uint32)

    @staticmethod
    def poseidon_composition(trace_evals, inter_evals, trace_log: int, lookup, claimed, rc,
                             accum: SecureColumnByCoords) -> None:
        """Adds the Poseidon constraint quotients on the evaluation domain of the given columns to
        accum (FrameworkComponent::evaluate_constraint_quotients_on_domain). rc: (1144, 4) words."""
        rc_arr = np.ascontiguousarray(np.asarray(rc, np.uint32).reshape(-1))
        _lib.call("cs_poseidon_composition", _ptr_table([c.data for c in trace_evals]),
                  _ptr_table([c.data for c in inter_evals]), trace_evals[0].log_size, trace_log,
                  _u32_table(lookup), _u32_table(claimed), rc_arr.ctypes.data_as(ctypes.c_void_p),
                  _ptr_table([c.data for c in accum.columns]), _stream())

    # Decommitment -------------------------------------------------------------
    @staticmethod
    def gather_words(tensors, slots: np.ndarray, indices: np.ndarray) -> np.ndarray:
        """Word k = tensors[slots[k]].flatten()[indices[k]] for contiguous int32 device tensors, read
        in one batched call (cs_gather_u32): the element-wise Column::at reads of
        MerkleProverLifted::decommit (crates/stwo/src/prover/vcs_lifted/prover.rs:97-162)."""
        slots = np.ascontiguousarray(slots, np.uint32)
        indices = np.ascontiguousarray(indices, np.uint32)
        out = np.empty(slots.size, np.uint32)
        if slots.size == 0:
            return out
        lengths = (ctypes.c_uint64 * len(tensors))(*[t.numel() for t in tensors])
        _lib.call("cs_gather_u32", _ptr_table(tensors), lengths, len(tensors), slots.ctypes.data_as(ctypes.c_void_p),
                  indices.ctypes.data_as(ctypes.c_void_p), slots.size, out.ctypes.data_as(ctypes.c_void_p), _stream())
        return out

    # GrindOps -----------------------------------------------------------------
    @staticmethod
    def grind(digest: bytes, pow_bits: int, max_nonce: int = 1 << 48) -> int:
        d = (ctypes.c_uint8 * 32).from_buffer_copy(digest)
        out = ctypes.c_uint64(0)
        _lib.call("cs_grind_blake2s", d, pow_bits, max_nonce, ctypes.byref(out), _stream())
        return out.value


class MerkleProverLifted:
    """Layer stack of a committed lifted tree (crates/stwo/src/prover/vcs_lifted/prover.rs:18-22).
    `layers` holds leaves first; `layer(k)` returns the layer with 2^k digests."""

    def __init__(self, layers: torch.Tensor, lifting_log_size: int):
        self.all = layers
        self.lifting_log_size = lifting_log_size

    def layer(self, k: int) -> torch.Tensor:
        L = self.lifting_log_size
        off = sum(1 << j for j in range(k + 1, L + 1))
        return self.all[off:off + (1 << k)]

    def root(self) -> bytes:
        return self.all[-1].cpu().numpy().view(np.uint32).astype("<u4").tobytes()


def digests_to_bytes(t: torch.Tensor) -> np.ndarray:
    """(n, 8) int32 digests -> (n, 32) uint8 (little-endian words = Blake2s digest bytes)."""
    return t.cpu().numpy().astype("<i4").view(np.uint8).reshape(-1, 32)
