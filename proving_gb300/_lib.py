"""ctypes binding of libstwo_cuda.so — the C ABI declared in include/stwo_cuda.h.

The library is built in-tree (python -m proving_gb300.build). Loading fails
loudly when it is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_build" / "libstwo_cuda.so"

CS_OK = 0
STATUS_NAMES = {0: "CS_OK", 1: "CS_ERR_INVALID_ARG", 2: "CS_ERR_OOM", 3: "CS_ERR_DEVICE", 4: "CS_ERR_TIMEOUT",
                5: "CS_ERR_NOT_FOUND"}

vp = ctypes.c_void_p
u32 = ctypes.c_uint32
u64 = ctypes.c_uint64
sz = ctypes.c_size_t
pp = ctypes.POINTER(ctypes.c_void_p)

# name -> argtypes; every function returns cs_status (int) unless listed in _RESTYPES.
SIGNATURES = {
    "cs_last_error": [],
    "cs_version": [],
    "cs_malloc": [pp, sz],
    "cs_free": [vp],
    "cs_memset_zero": [vp, sz, vp],
    "cs_memcpy_h2d": [vp, vp, sz, vp],
    "cs_memcpy_d2h": [vp, vp, sz, vp],
    "cs_memcpy_d2d": [vp, vp, sz, vp],
    "cs_stream_synchronize": [vp],
    "cs_bit_reverse_m31": [vp, u32, vp],
    "cs_precompute_twiddles": [u32, u32, vp, vp, vp],
    "cs_kernel_launch_count": [],
    "cs_interpolate_columns": [vp, u32, u32, vp, u32, vp],
    "cs_interpolate_columns_into": [vp, vp, u32, u32, vp, u32, vp],
    "cs_evaluate_columns": [vp, vp, u32, u32, u32, vp, u32, vp],
    "cs_interpolate_columns_multi": [vp, vp, vp, u32, vp, u32, vp],
    "cs_evaluate_columns_multi": [vp, vp, vp, u32, u32, vp, u32, vp],
    "cs_merkle_build_leaves": [vp, vp, u32, u32, vp, vp],
    "cs_merkle_build_next_layer": [vp, u32, vp, vp],
    "cs_merkle_build_layers": [vp, u32, vp],
    "cs_merkle_commit": [vp, vp, u32, u32, vp, vp],
    "cs_pack_leaves_input": [vp, u32, vp, vp],
    "cs_fold_line": [vp, u32, vp, vp, vp, u32, vp],
    "cs_fold_circle_into_line": [vp, u32, vp, vp, vp, u32, vp],
    "cs_grind_blake2s": [vp, u32, u64, ctypes.POINTER(ctypes.c_uint64), vp],
    "cs_interpolate_columns_on_subdomain": [vp, u32, u32, u32, vp, u32, vp],
    "cs_accumulate": [vp, vp, u32, vp],
    "cs_generate_secure_powers": [vp, u32, vp],
    "cs_lift_and_accumulate": [vp, vp, u32, vp],
    "cs_barycentric_weights": [u32, vp, vp, vp, vp],
    "cs_barycentric_eval": [vp, u32, u32, vp, vp, vp],
    "cs_eval_at_point": [vp, u32, u32, vp, vp, vp, vp],
    "cs_accumulate_numerators": [vp, u32, u32, u32, vp, vp, vp, vp],
    "cs_quotients_on_subdomain": [vp, vp, u32, vp, vp, u32, u32, vp, vp],
    "cs_decompose": [vp, u32, vp, vp, vp],
    "cs_wide_fib_composition": [vp, u32, u32, u32, vp, vp, vp],
    "cs_wide_fib_trace": [vp, vp, u32, u32, vp, vp],
    "cs_grind_blake2s_noalloc": [vp, u32, u32, u64, vp, vp],
    "cs_logup_running_sum": [vp, u32, vp, vp, vp, vp],
    "cs_gather_u32": [vp, vp, u32, vp, vp, u32, vp, vp],
    "cs_poseidon_trace": [u32, vp, vp],
    "cs_poseidon_interaction": [vp, u32, vp, vp, vp, vp],
    "cs_poseidon_composition": [vp, vp, u32, u32, vp, vp, vp, vp, vp],
    "cs_int_peak_probe": [u32, u32, u32, vp, vp],
    "cs_fold_set_plan": [u32],
    "cs_fold_get_plan": [vp],
    "cs_fft_set_plan": [u32, u32, u32, vp, u32],
    "cs_fft_get_plan": [u32, u32, u32, vp, vp],
    "cs_fold_line_device_alpha": [vp, u32, vp, vp, vp, u32, vp],
    "cs_fold_line_steps": [vp, u32, u32, vp, vp, vp, u32, vp],
    "cs_fold_circle_into_line_device_alpha": [vp, u32, vp, vp, vp, u32, vp],
    "cs_channel_mix_root": [vp, vp, vp],
    "cs_channel_draw_secure_felt": [vp, vp, vp],
    "cs_fri_commit_fold_tail": [vp, vp, vp, vp, u32, u32, vp, u32, vp],
    "cs_logup_running_sums": [u32, vp, vp, vp, vp, vp, vp],
    "cs_logup_combine": [vp, u32, u32, vp, vp, vp, vp],
    "cs_logup_gen_col": [vp, vp, vp, vp, u32, vp, vp],
    "cs_logup_finalize_last": [vp, u32, vp, vp],
    "cs_gkr_gen_eq_evals": [vp, u32, vp, vp, vp],
    "cs_mle_fix_first_variable": [vp, u32, u32, vp, vp, vp],
    "cs_gkr_next_layer": [u32, vp, vp, u32, vp, vp, vp],
    "cs_gkr_sum_as_poly": [u32, vp, vp, vp, u32, vp, vp, vp],
    "cs_gkr_prove_batch": [u32, vp, vp, vp, vp, vp, sz, ctypes.POINTER(sz), vp],
    "cs_rtc_available": [],
    "cs_rtc_compile_air": [vp, u32, vp, vp, u32, u32, u32, vp, vp, ctypes.c_size_t],
    "cs_rtc_air_composition": [vp, vp, vp, vp, u32, u32, vp, vp],
    "cs_rtc_air_composition_subdomain": [vp, vp, vp, vp, u32, u32, u32, vp, vp],
    "cs_rtc_release": [vp],
    "cs_rtc_kernel_shape": [vp, vp, vp, vp],
    "cs_rtc_compile_air_logup": [vp, u32, vp, vp, u32, u32, u32, u32, u32, vp, vp, ctypes.c_size_t],
    "cs_rtc_air_fractions": [vp, vp, vp, u32, vp, vp],
    "cs_prove_air": [vp, vp, u32, vp, vp, ctypes.c_size_t, vp, vp],
    "cs_prove_wide_fib": [vp, vp, vp, ctypes.c_size_t, vp, vp],
    "cs_prove_fib_and_lookups": [vp, vp, u32, vp, vp, vp, vp, ctypes.c_size_t, vp, vp],
    "cs_prove_poseidon": [u32, vp, vp, ctypes.c_size_t, vp, vp],
    "cs_host_blake2s": [vp, ctypes.c_size_t, vp],
    "cs_logup_compositions": [u32, vp, vp, u32, u32, vp, vp, vp, vp, vp],
    "cs_logup_composition": [vp, vp, u32, u32, vp, vp, vp, vp, vp],
}
_RESTYPES = {"cs_last_error": ctypes.c_char_p, "cs_version": ctypes.c_char_p,
             "cs_kernel_launch_count": ctypes.c_uint64}

_lib = None


def exported_names_from_header(header: Path) -> list[str]:
    """Function names declared in include/stwo_cuda.h (for the export test)."""
    import re
    text = header.read_text()
    return sorted(set(re.findall(r"^\s*(?:cs_status|const char \*|uint64_t)\s*(cs_\w+)\s*\(", text, re.M)))


def load(path: Path | None = None):
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise ImportError(f"{p} is missing: build it with `python -m proving_gb300.build` (no CPU fallback exists)")
    L = ctypes.CDLL(str(p))
    for name, args in SIGNATURES.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = _RESTYPES.get(name, ctypes.c_int)
    if path is None:
        _lib = L
    return L


class CudaBackendError(RuntimeError):
    def __init__(self, fn: str, status: int, msg: str):
        super().__init__(f"{fn} -> {STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


def check(fn: str, status: int):
    if status != CS_OK:
        raise CudaBackendError(fn, status, load().cs_last_error().decode(errors="replace"))


def call(name: str, *args):
    check(name, getattr(load(), name)(*args))
