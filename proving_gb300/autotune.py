"""The FFT pass-plan autotuner.

A column of 2^log_n words whose FFT runs n_layers layers is processed in passes
of consecutive layers, each staged once through shared memory (fft.cu). The
library's default split is the fewest passes with the layers spread evenly.
`tune` times candidate splits for the shapes a workload uses, on scratch
columns of the workload's width, installs the fastest for each shape
(cs_fft_set_plan, process-wide) and returns what it measured. Results of the
FFT do not depend on the plan.
"""
from __future__ import annotations

import ctypes

from . import _lib

MAX_CONTIGUOUS, MAX_STRIDED, MIN_FIRST = 12, 11, 3


def candidate_plans(n_layers: int, min_part: int = 5) -> list[tuple[int, ...]]:
    """Splits into the fewest passes and one more, first pass <= 12 (>= 3 when more follow),
    later passes <= 11, every pass at least min_part layers (or all layers in one pass)."""
    fewest = 1
    while n_layers > MAX_CONTIGUOUS + (fewest - 1) * MAX_STRIDED:
        fewest += 1
    out = []

    def rec(prefix, left, passes_left):
        if passes_left == 0:
            if left == 0:
                out.append(tuple(prefix))
            return
        first = not prefix
        hi = MAX_CONTIGUOUS if first else MAX_STRIDED
        lo = max(min_part if passes_left > 1 or not first else 1, MIN_FIRST if first else 1)
        for t in range(lo, min(hi, left) + 1):
            rec(prefix + [t], left - t, passes_left - 1)

    for n_pass in (fewest, fewest + 1):
        if n_pass == 1:
            if n_layers <= MAX_CONTIGUOUS:
                out.append((n_layers,))
            continue
        rec([], n_layers, n_pass)
    return out


def get_plan(inverse: bool, log_n: int, n_layers: int) -> tuple[int, ...]:
    buf = (ctypes.c_uint32 * 32)()
    n = ctypes.c_uint32(0)
    _lib.call("cs_fft_get_plan", int(inverse), log_n, n_layers, buf, ctypes.byref(n))
    return tuple(buf[i] for i in range(n.value))


def set_plan(inverse: bool, log_n: int, n_layers: int, plan) -> None:
    arr = (ctypes.c_uint32 * max(1, len(plan)))(*plan)
    _lib.call("cs_fft_set_plan", int(inverse), log_n, n_layers, arr, len(plan))


def tune(shapes, n_cols: int, reps: int = 5, warmup: int = 2) -> dict:
    """shapes: (inverse, log_n, n_layers) triples. Times every candidate split on n_cols scratch
    columns and installs the fastest per shape. Returns {shape: {"default": plan, "best": plan,
    "ms": {plan: ms}}}."""
    import torch
    from .backend import CudaBackend, canonic_half_coset
    report = {}
    for inverse, log_n, n_layers in shapes:
        tree = CudaBackend.precompute_twiddles(canonic_half_coset(log_n + 1))
        src = torch.randint(0, (1 << 31) - 1, (n_cols, 1 << (log_n if inverse else n_layers)),
                            dtype=torch.int64, device="cuda").to(torch.int32)
        dst = torch.empty((n_cols, 1 << log_n), dtype=torch.int32, device="cuda")
        vp = ctypes.c_void_p
        t_src = (vp * n_cols)(*[src[i].data_ptr() for i in range(n_cols)])
        t_dst = (vp * n_cols)(*[dst[i].data_ptr() for i in range(n_cols)])
        st = vp(torch.cuda.current_stream().cuda_stream)

        def run():
            if inverse:
                _lib.call("cs_interpolate_columns_into", t_src, t_dst, n_cols, log_n, tree.itwiddles.data_ptr(),
                          tree.log_size, st)
            else:
                _lib.call("cs_evaluate_columns", t_src, t_dst, n_cols, n_layers, log_n, tree.twiddles.data_ptr(),
                          tree.log_size, st)

        set_plan(inverse, log_n, n_layers, [])
        default = get_plan(inverse, log_n, n_layers)
        timings = {}
        for plan in candidate_plans(n_layers):
            set_plan(inverse, log_n, n_layers, plan)
            for _ in range(warmup):
                run()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            a.record()
            for _ in range(reps):
                run()
            b.record()
            torch.cuda.synchronize()
            timings[plan] = a.elapsed_time(b) / reps
        best = min(timings, key=timings.get)
        set_plan(inverse, log_n, n_layers, best)
        report[(inverse, log_n, n_layers)] = {"default": default, "best": best, "ms": timings}
        del src, dst
    return report
