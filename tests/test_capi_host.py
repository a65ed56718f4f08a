"""CPU-only checks of the C ABI: the library loads, exports every function the
public header declares, and rejects bad arguments before touching a device."""
import ctypes
from pathlib import Path

import pytest

from proving_gb300 import _lib

ROOT = Path(__file__).resolve().parent.parent
HEADERS = sorted((ROOT / "include").glob("*.h"))


@pytest.fixture(scope="module")
def lib():
    from proving_gb300 import build
    build.build()
    return _lib.load()


def declared():
    names = []
    for h in HEADERS:
        names += _lib.exported_names_from_header(h)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared()
    assert "cs_interpolate_columns" in names and "cs_merkle_build_leaves" in names
    assert len(names) >= 20


def test_every_declared_symbol_is_exported(lib):
    for name in declared():
        assert hasattr(lib, name), f"{name} declared in include/ but not exported"


def test_bindings_cover_header():
    # every declared function has a ctypes signature in the Python mirror
    assert set(declared()) <= set(_lib.SIGNATURES), set(declared()) - set(_lib.SIGNATURES)


def test_version(lib):
    assert b"sm_103a" in lib.cs_version()


def _status(lib, name, *args):
    return getattr(lib, name)(*args)


def test_invalid_arguments_are_rejected_on_host(lib):
    INVALID = 1
    null = ctypes.c_void_p(0)
    # log size out of range
    assert _status(lib, "cs_interpolate_columns", null, 0, 0, null, 10, null) == INVALID
    assert b"log_size" in lib.cs_last_error()
    # twiddle tree too small for the domain
    tab = (ctypes.c_void_p * 1)(1 << 20)
    assert _status(lib, "cs_interpolate_columns", tab, 1, 12, ctypes.c_void_p(1 << 21), 5, null) == INVALID
    # evaluate with fewer output than input coefficients
    assert _status(lib, "cs_evaluate_columns", tab, tab, 1, 10, 8, ctypes.c_void_p(1 << 21), 12, null) == INVALID
    # grind beyond 32 bits
    d = (ctypes.c_uint8 * 32)()
    out = ctypes.c_uint64()
    assert _status(lib, "cs_grind_blake2s", d, 33, 1 << 20, ctypes.byref(out), null) == INVALID
    # Merkle columns not sorted by length
    logs = (ctypes.c_uint32 * 2)(5, 4)
    cols = (ctypes.c_void_p * 2)(1 << 20, 1 << 21)
    assert _status(lib, "cs_merkle_build_leaves", cols, logs, 2, 5, ctypes.c_void_p(1 << 22), null) == INVALID
    assert b"sorted" in lib.cs_last_error()
    # empty tree must be committed at height 0 (prover.rs:41-50)
    assert _status(lib, "cs_merkle_build_leaves", null, null, 0, 3, ctypes.c_void_p(1 << 22), null) == INVALID
    # fold_line domain not covered by the twiddle tree
    src = (ctypes.c_void_p * 4)(1 << 20, 1 << 21, 1 << 22, 1 << 23)
    alpha = (ctypes.c_uint32 * 4)(1, 2, 3, 4)
    assert _status(lib, "cs_fold_line", src, 12, alpha, src, ctypes.c_void_p(1 << 24), 10, null) == INVALID
    # batched LogUp running sums: a log size of 0 and a null output coordinate
    vals = (ctypes.c_void_p * 2)(1 << 20, 1 << 21)
    outs = (ctypes.c_void_p * 8)(*[1 << (22 + k) for k in range(8)])
    z = (ctypes.c_uint32 * 4)(1, 2, 3, 4)
    assert _status(lib, "cs_logup_running_sums", 2, vals, (ctypes.c_uint32 * 2)(4, 0), z, outs,
                   ctypes.c_void_p(1 << 30), null) == INVALID
    assert b"log size" in lib.cs_last_error()
    outs[5] = None
    assert _status(lib, "cs_logup_running_sums", 2, vals, (ctypes.c_uint32 * 2)(4, 5), z, outs,
                   ctypes.c_void_p(1 << 30), null) == INVALID
    assert b"coordinate" in lib.cs_last_error()


def test_gkr_arguments_are_checked_on_host(lib):
    INVALID = 1
    null = ctypes.c_void_p(0)
    q = (ctypes.c_uint32 * 4)(1, 2, 3, 4)
    cols = (ctypes.c_void_p * 4)(*[1 << (22 + k) for k in range(4)])
    ys = (ctypes.c_uint32 * (4 * 29))()
    # more eq variables than the kernel's parameter block holds
    assert _status(lib, "cs_gkr_gen_eq_evals", ys, 29, q, cols, null) == INVALID
    # unknown layer kind, a layer of one value, a misaligned column
    assert _status(lib, "cs_gkr_next_layer", 4, cols, cols, 5, cols, cols, null) == INVALID
    assert _status(lib, "cs_gkr_next_layer", 1, cols, cols, 0, cols, cols, null) == INVALID
    odd = (ctypes.c_void_p * 4)((1 << 22) + 4, 1 << 23, 1 << 24, 1 << 25)
    assert _status(lib, "cs_gkr_next_layer", 0, null, odd, 5, null, cols, null) == INVALID
    assert b"aligned" in lib.cs_last_error()
    # a generic LogUp layer needs its numerators
    assert _status(lib, "cs_gkr_next_layer", 1, null, cols, 5, cols, cols, null) == INVALID
    # the sum-check sums need an input layer of at least 4 values
    assert _status(lib, "cs_gkr_sum_as_poly", 0, cols, null, cols, 1, q, ctypes.c_void_p(1 << 30), null) == INVALID
    assert _status(lib, "cs_mle_fix_first_variable", cols, 0, 0, q, cols, null) == INVALID
    # the native batch prover: no instance, an unknown kind, 0 variables, a null column
    n_words = ctypes.c_size_t()
    state = (ctypes.c_uint32 * 9)()
    tab = (ctypes.c_void_p * 8)(*[1 << (22 + k) for k in range(8)])
    for kinds, nv, n in (((0,), (5,), 0), ((7,), (5,), 1), ((1,), (0,), 1)):
        assert _status(lib, "cs_gkr_prove_batch", n, (ctypes.c_uint32 * 1)(*kinds), (ctypes.c_uint32 * 1)(*nv),
                       tab, state, null, 0, ctypes.byref(n_words), null) == INVALID
    tab[5] = None
    assert _status(lib, "cs_gkr_prove_batch", 1, (ctypes.c_uint32 * 1)(0), (ctypes.c_uint32 * 1)(4), tab, state,
                   null, 0, ctypes.byref(n_words), null) == INVALID
    assert b"null column" in lib.cs_last_error()


def test_error_raises_in_python_mirror(lib):
    with pytest.raises(_lib.CudaBackendError) as e:
        _lib.call("cs_bit_reverse_m31", ctypes.c_void_p(0), 4, ctypes.c_void_p(0))
    assert "CS_ERR_INVALID_ARG" in str(e.value)


def test_gather_checks_every_request_on_host(lib):
    # slots and indices are validated against the table before any device work
    INVALID = 1
    null = ctypes.c_void_p(0)
    table = (ctypes.c_void_p * 2)(1 << 20, 1 << 21)
    lengths = (ctypes.c_uint64 * 2)(16, 4)
    out = (ctypes.c_uint32 * 2)()
    slot = (ctypes.c_uint32 * 2)(0, 2)
    idx = (ctypes.c_uint32 * 2)(3, 0)
    assert _status(lib, "cs_gather_u32", table, lengths, 2, slot, idx, 2, out, null) == INVALID
    assert b"slot" in lib.cs_last_error()
    slot = (ctypes.c_uint32 * 2)(0, 1)
    idx = (ctypes.c_uint32 * 2)(15, 4)
    assert _status(lib, "cs_gather_u32", table, lengths, 2, slot, idx, 2, out, null) == INVALID
    assert b"word 4" in lib.cs_last_error()
    # nothing to read: no device work at all
    assert _status(lib, "cs_gather_u32", null, null, 0, null, null, 0, null, null) == 0


def test_fft_plans_are_validated_and_stored_on_host(lib):
    from proving_gb300 import autotune
    INVALID = 1

    def set_plan(inv, log_n, n_layers, plan):
        arr = (ctypes.c_uint32 * max(1, len(plan)))(*plan)
        return _status(lib, "cs_fft_set_plan", inv, log_n, n_layers, arr, len(plan))

    assert set_plan(1, 20, 20, [10, 9]) == INVALID           # covers 19 of 20 layers
    assert set_plan(1, 20, 20, [8, 12]) == INVALID           # a strided pass above 11 layers
    assert set_plan(1, 20, 20, [2, 9, 9]) == INVALID         # first pass below 3 layers
    assert set_plan(1, 20, 20, [13, 7]) == INVALID           # contiguous pass above 12 layers
    default = autotune.get_plan(True, 20, 20)
    assert sum(default) == 20
    assert set_plan(1, 20, 20, [6, 7, 7]) == 0
    assert autotune.get_plan(True, 20, 20) == (6, 7, 7)
    assert set_plan(1, 20, 20, []) == 0                      # removed: back to the default
    assert autotune.get_plan(True, 20, 20) == default
    for n in range(1, 25):
        for plan in autotune.candidate_plans(n):
            assert sum(plan) == n and plan[0] <= 12 and all(t <= 11 for t in plan[1:])


def test_host_blake2s_matches_hashlib(lib):
    # the native prover's channel hash (RFC 7693), every block-boundary case
    import hashlib
    import os
    for msg in [b"", b"a", b"x" * 63, b"y" * 64, b"z" * 65, b"w" * 128, os.urandom(200)]:
        out = (ctypes.c_uint8 * 32)()
        _lib.call("cs_host_blake2s", msg, len(msg), out)
        assert bytes(out) == hashlib.blake2s(msg).digest()


def test_native_prover_checks_arguments_on_host(lib):
    from proving_gb300.backend import _WideFibProofParams
    p = _WideFibProofParams()
    n_cols = (ctypes.c_uint32 * 1)(2)   # fewer than 3 columns
    logs = (ctypes.c_uint32 * 1)(5)
    p.n_components, p.n_cols, p.log_sizes = 1, ctypes.cast(n_cols, ctypes.c_void_p), ctypes.cast(logs, ctypes.c_void_p)
    p.lifting_log_size, p.pow_bits, p.log_blowup_factor, p.log_last_layer_degree_bound, p.n_queries = 6, 10, 1, 0, 3
    p.d_twiddles, p.d_itwiddles, p.twiddle_log_size = 1 << 20, 1 << 21, 6
    cols = (ctypes.c_void_p * 2)(1 << 22, 1 << 23)
    n = ctypes.c_size_t(0)
    assert _status(lib, "cs_prove_wide_fib", ctypes.byref(p), cols, None, 0, ctypes.byref(n), None) == 1
    assert b"columns" in lib.cs_last_error()


@pytest.mark.parametrize("fold_step,blowup,word", [(9, 1, b"fold_step"), (6, 1, b"fold_step"), (1, 2, b"blowup")])
def test_native_prover_checks_fri_parameters_on_host(lib, fold_step, blowup, word):
    # fold steps above 8 or past the last layer, and a blowup the hand-written AIR does not take,
    # are refused before any device work
    from proving_gb300.backend import _WideFibProofParams
    p = _WideFibProofParams()
    n_cols = (ctypes.c_uint32 * 1)(3)
    logs = (ctypes.c_uint32 * 1)(5)
    p.n_components, p.n_cols, p.log_sizes = 1, ctypes.cast(n_cols, ctypes.c_void_p), ctypes.cast(logs, ctypes.c_void_p)
    p.lifting_log_size, p.pow_bits, p.log_blowup_factor, p.log_last_layer_degree_bound, p.n_queries = \
        5 + blowup, 10, blowup, 0, 3
    p.d_twiddles, p.d_itwiddles, p.twiddle_log_size = 1 << 20, 1 << 21, 8
    p.fold_step = fold_step
    cols = (ctypes.c_void_p * 3)(1 << 22, 1 << 23, 1 << 24)
    n = ctypes.c_size_t(0)
    assert _status(lib, "cs_prove_wide_fib", ctypes.byref(p), cols, None, 0, ctypes.byref(n), None) == 1
    assert word in lib.cs_last_error()


def test_merkle_entry_points_reject_misaligned_digest_buffers(lib):
    # digests move as 16-byte words: a 4-byte-aligned offset into a buffer is refused on the host
    # instead of faulting the device
    INVALID = 1
    null = ctypes.c_void_p(0)
    odd = ctypes.c_void_p((1 << 22) + 4)
    even = ctypes.c_void_p(1 << 23)
    assert _status(lib, "cs_merkle_build_layers", odd, 5, null) == INVALID
    assert b"aligned" in lib.cs_last_error()
    assert _status(lib, "cs_merkle_build_next_layer", odd, 4, even, null) == INVALID
    assert b"aligned" in lib.cs_last_error()
    assert _status(lib, "cs_merkle_build_next_layer", even, 4, odd, null) == INVALID
    logs = (ctypes.c_uint32 * 1)(5)
    cols = (ctypes.c_void_p * 1)(1 << 20)
    assert _status(lib, "cs_merkle_build_leaves", cols, logs, 1, 5, odd, null) == INVALID
    assert b"aligned" in lib.cs_last_error()
    assert _status(lib, "cs_merkle_commit", cols, logs, 1, 5, odd, null) == INVALID
    assert b"aligned" in lib.cs_last_error()


def test_merkle_height_limits_agree(lib):
    # leaves, layers and commit accept trees up to height 30 and refuse 31 (checked before any
    # device work: a null buffer is refused after the height check)
    INVALID = 1
    null = ctypes.c_void_p(0)
    assert _status(lib, "cs_merkle_build_layers", ctypes.c_void_p(1 << 22), 31, null) == INVALID
    assert b"too large" in lib.cs_last_error()
    logs = (ctypes.c_uint32 * 1)(31)
    cols = (ctypes.c_void_p * 1)(1 << 20)
    assert _status(lib, "cs_merkle_build_leaves", cols, logs, 1, 31, ctypes.c_void_p(1 << 22), null) == INVALID
    assert b"too large" in lib.cs_last_error()


def test_mixed_size_fft_checks_arguments_on_host(lib):
    INVALID = 1
    null = ctypes.c_void_p(0)
    cols = (ctypes.c_void_p * 2)(1 << 20, 1 << 21)
    logs = (ctypes.c_uint32 * 2)(5, 0)  # a column of log size 0
    assert _status(lib, "cs_interpolate_columns_multi", cols, cols, logs, 2, ctypes.c_void_p(1 << 22), 10,
                   null) == INVALID
    logs = (ctypes.c_uint32 * 2)(5, 12)  # beyond the twiddle tree
    assert _status(lib, "cs_interpolate_columns_multi", cols, cols, logs, 2, ctypes.c_void_p(1 << 22), 10,
                   null) == INVALID
    assert b"twiddle" in lib.cs_last_error()
    # evaluate may not write over its coefficients
    assert _status(lib, "cs_evaluate_columns_multi", cols, cols, (ctypes.c_uint32 * 2)(5, 6), 1, 2,
                   ctypes.c_void_p(1 << 22), 10, null) == INVALID
    assert b"aliases" in lib.cs_last_error()


def test_native_prover_rejects_unknown_flags(lib):
    from proving_gb300.backend import _WideFibProofParams
    p = _WideFibProofParams()
    n_cols = (ctypes.c_uint32 * 1)(4)
    logs = (ctypes.c_uint32 * 1)(5)
    p.n_components, p.n_cols, p.log_sizes = 1, ctypes.cast(n_cols, ctypes.c_void_p), ctypes.cast(logs, ctypes.c_void_p)
    p.lifting_log_size, p.pow_bits, p.log_blowup_factor, p.log_last_layer_degree_bound, p.n_queries = 6, 10, 1, 0, 3
    p.d_twiddles, p.d_itwiddles, p.twiddle_log_size, p.flags = 1 << 20, 1 << 21, 6, 6
    cols = (ctypes.c_void_p * 4)(1 << 22, 1 << 23, 1 << 24, 1 << 25)
    n = ctypes.c_size_t(0)
    assert _status(lib, "cs_prove_wide_fib", ctypes.byref(p), cols, None, 0, ctypes.byref(n), None) == 1
    assert b"flags" in lib.cs_last_error()


def test_fri_tail_checks_arguments_on_host(lib):
    # cs_fri_commit_fold_tail: layers of at most 2^10 values, at most log_size layers, trees 16-byte
    # aligned; rejected before any launch
    INVALID = 1
    null = ctypes.c_void_p(0)
    state, alphas, itw = ctypes.c_void_p(1 << 20), ctypes.c_void_p(1 << 21), ctypes.c_void_p(1 << 22)
    evals = (ctypes.c_void_p * 12)(*[(1 << 24) + (k << 12) for k in range(12)])
    trees = (ctypes.c_void_p * 2)(1 << 26, 1 << 27)
    assert _status(lib, "cs_fri_commit_fold_tail", state, alphas, evals, trees, 11, 2, itw, 12, null) == INVALID
    assert b"log 11" in lib.cs_last_error()
    assert _status(lib, "cs_fri_commit_fold_tail", state, alphas, evals, trees, 3, 4, itw, 12, null) == INVALID
    assert _status(lib, "cs_fri_commit_fold_tail", state, alphas, evals, trees, 3, 0, itw, 12, null) == INVALID
    assert _status(lib, "cs_fri_commit_fold_tail", state, alphas, evals, trees, 5, 2, itw, 4, null) == INVALID
    bad = (ctypes.c_void_p * 2)(1 << 26, (1 << 27) + 8)
    assert _status(lib, "cs_fri_commit_fold_tail", state, alphas, evals, bad, 5, 2, itw, 12, null) == INVALID
    assert b"16-byte" in lib.cs_last_error()
    assert _status(lib, "cs_fri_commit_fold_tail", null, alphas, evals, trees, 5, 2, itw, 12, null) == INVALID


def test_logup_generator_checks_arguments_on_host(lib):
    INVALID = 1
    null = ctypes.c_void_p(0)
    four = (ctypes.c_void_p * 4)(1 << 20, 1 << 21, 1 << 22, 1 << 23)
    out = (ctypes.c_void_p * 4)(1 << 24, 1 << 25, 1 << 26, 1 << 27)
    m31 = ctypes.c_void_p(1 << 28)
    # exactly one numerator
    assert _status(lib, "cs_logup_gen_col", four, m31, four, null, 5, out, null) == INVALID
    assert b"exactly one numerator" in lib.cs_last_error()
    assert _status(lib, "cs_logup_gen_col", null, null, four, null, 5, out, null) == INVALID
    assert _status(lib, "cs_logup_gen_col", null, m31, four, null, 31, out, null) == INVALID
    vals = (ctypes.c_void_p * 1)(1 << 20)
    z = (ctypes.c_uint32 * 4)(1, 2, 3, 4)
    assert _status(lib, "cs_logup_combine", vals, 0, 5, z, z, out, null) == INVALID
    assert _status(lib, "cs_logup_combine", (ctypes.c_void_p * 1)(0), 1, 5, z, z, out, null) == INVALID
    claimed = (ctypes.c_uint32 * 4)()
    assert _status(lib, "cs_logup_finalize_last", out, 0, claimed, null) == INVALID
    assert _status(lib, "cs_logup_finalize_last", out, 29, claimed, null) == INVALID


def test_fold_plan_is_checked_and_kept(lib):
    INVALID = 1
    v = ctypes.c_uint32(0)
    assert _status(lib, "cs_fold_get_plan", ctypes.byref(v)) == 0
    old = v.value
    assert old in (3, 4)
    assert _status(lib, "cs_fold_set_plan", 5) == INVALID
    assert _status(lib, "cs_fold_set_plan", 2) == INVALID
    assert _status(lib, "cs_fold_get_plan", ctypes.c_void_p(0)) == INVALID
    for want in (3, 4, old):
        assert _status(lib, "cs_fold_set_plan", want) == 0
        assert _status(lib, "cs_fold_get_plan", ctypes.byref(v)) == 0 and v.value == want


def test_prove_air_checks_arguments_on_host(lib):
    # cs_prove_air: null tables, no components and a component without a kernel are rejected before
    # any device work
    INVALID = 1
    null = ctypes.c_void_p(0)
    from proving_gb300.backend import _AirComponent, _WideFibProofParams
    params = _WideFibProofParams()
    comps = (_AirComponent * 1)()
    trace = (ctypes.c_void_p * 1)(1 << 20)
    n = ctypes.c_size_t(0)
    assert _status(lib, "cs_prove_air", null, comps, 1, trace, null, 0, ctypes.byref(n), null) == INVALID
    assert _status(lib, "cs_prove_air", ctypes.byref(params), comps, 0, trace, null, 0, ctypes.byref(n), null) == INVALID
    assert _status(lib, "cs_prove_air", ctypes.byref(params), comps, 1, trace, null, 0, ctypes.byref(n), null) == INVALID
    assert b"kernel" in lib.cs_last_error()
