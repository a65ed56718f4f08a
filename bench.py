"""Commit-stage microbenchmark of the Stwo prover hot path on GB300, with whole proofs of the
other workloads beside it.

Headline workload (one step = one commit stage of 256 columns of 2^20 rows):
  256 M31 columns of 2^20 rows (uniform in [0, P), seeded), interpolate, evaluate
  on the 4x blown-up canonic domain (log 22), lifted Blake2s Merkle tree over the
  256-wide leaves (height 22), then 22 FRI folds (fold_circle_into_line + 21
  fold_line) of a seeded QM31 column of log 22 with seeded QM31 challenges.
  The unit is commit steps/s: a step is not a whole proof. Whole proofs (Wide-Fibonacci
  100 x 2^14, the 600 + 120-column mixed-size trace, Poseidon2 at 2^18 rows) and the
  serving mix are reported in proofs/s with p50/p99 beside it.

`value` times the step with the trace already resident in HBM; `e2e` times the
same step through the C ABI with the trace in pinned host memory, including the
host->device copy of the trace and FRI column and the device->host read of the
Merkle root and the last FRI value. The trace (1 GiB) and the extended
evaluation (4 GiB) exceed L2 (129 MB), so no L2 flush is needed between steps.

--impl reference times the CPU restatement of the reference (the oracle; the
Rust reference cannot be built: neither machine has cargo) on whole steps
of the same workload, with all host threads. --gpus N starts N replicas (one
process per GPU, torch.distributed.run) when it is not already running under a
launcher.
"""
from __future__ import annotations

import argparse
import ctypes
import hashlib
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "proofs/s, p50/p99 prove latency on 1 GB300: batched vs plain CUDA, bit-exact"
UNIT = "commit steps/s"
PROOF_UNIT = "proofs/s"
N_COLS, LOG_ROWS, LOG_BLOWUP = 256, 20, 2
LOG_EXT = LOG_ROWS + LOG_BLOWUP
FRI_LOG = 22


def workload_name():
    return (f"commit-stage microbench: {N_COLS} M31 cols x 2^{LOG_ROWS}, interpolate, evaluate on log {LOG_EXT}, "
            f"lifted Blake2s Merkle over {N_COLS}-wide leaves, {FRI_LOG} FRI folds of a QM31 col of log {FRI_LOG}")


# DRAM bytes (read + write) measured with ncu on the 256 x 2^20 workload
# (profiles/launch_list_commit_stage_256x2^20.md): one merkle_leaves_kernel launch, and the two
# fft_tile_kernel launches of one evaluate
LEAVES_TRAFFIC_BYTES = 4425.2e6
EVALUATE_TRAFFIC_BYTES = 13935.0e6


def set_shape(n_cols: int, log_rows: int):
    global N_COLS, LOG_ROWS, LOG_EXT, FRI_LOG
    N_COLS, LOG_ROWS = n_cols, log_rows
    LOG_EXT = LOG_ROWS + LOG_BLOWUP
    FRI_LOG = LOG_EXT


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ----------------------------------------------------------------- clocks

class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            parts = [p.strip() for p in l.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx = max(mx, float(parts[1]))
            except ValueError:
                continue
            for name, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------------- GPU arm

class CommitStage:
    """Device buffers and the step, all through the C ABI (proving_gb300._lib)."""

    def __init__(self, torch, seed: int = 2026):
        from proving_gb300 import _lib
        from proving_gb300.backend import canonic_half_coset, subgroup_gen
        self.torch, self.L = torch, _lib
        dev = torch.device("cuda", torch.cuda.current_device())
        g = torch.Generator(device=dev)
        g.manual_seed(seed)
        P = (1 << 31) - 1
        self.evals = torch.randint(0, P, (N_COLS, 1 << LOG_ROWS), generator=g, device=dev, dtype=torch.int64).to(
            torch.int32)
        self.fri_src = torch.randint(0, P, (4, 1 << FRI_LOG), generator=g, device=dev, dtype=torch.int64).to(
            torch.int32)
        self.alphas = np.random.default_rng(seed).integers(0, P, (FRI_LOG, 4), dtype=np.int64).astype(np.uint32)
        self.coeffs = torch.empty_like(self.evals)
        self.ext = torch.empty((N_COLS, 1 << LOG_EXT), dtype=torch.int32, device=dev)
        total = (1 << (LOG_EXT + 1)) - 1
        self.layers = torch.empty((total, 8), dtype=torch.int32, device=dev)
        # FRI layers: 2^21, 2^20, ..., 2^0 QM31 values (4 coordinate arrays each)
        self.fri_layers = [torch.empty((4, 1 << k), dtype=torch.int32, device=dev) for k in range(FRI_LOG - 1, -1, -1)]
        root = canonic_half_coset(LOG_EXT + 1)
        self.tw_log = root.log_size
        self.tw = torch.empty(1 << self.tw_log, dtype=torch.int32, device=dev)
        self.itw = torch.empty_like(self.tw)
        _lib.call("cs_precompute_twiddles", root.initial_index, root.log_size, self.tw.data_ptr(),
                  self.itw.data_ptr(), self.stream())
        vp = ctypes.c_void_p
        self.t_evals = (vp * N_COLS)(*[self.evals[i].data_ptr() for i in range(N_COLS)])
        self.t_coeffs = (vp * N_COLS)(*[self.coeffs[i].data_ptr() for i in range(N_COLS)])
        self.t_ext = (vp * N_COLS)(*[self.ext[i].data_ptr() for i in range(N_COLS)])
        self.logs = (ctypes.c_uint32 * N_COLS)(*([LOG_EXT] * N_COLS))
        self.fri_tabs = [(vp * 4)(*[self.fri_src[k].data_ptr() for k in range(4)])]
        for lay in self.fri_layers:
            self.fri_tabs.append((vp * 4)(*[lay[k].data_ptr() for k in range(4)]))
        self.alpha_tabs = [(ctypes.c_uint32 * 4)(*[int(x) for x in a]) for a in self.alphas]
        self.line_alphas = (ctypes.c_uint32 * (4 * (FRI_LOG - 1)))(*[int(x) for a in self.alphas[1:] for x in a])
        self.layer_ptr = []
        off = 0
        for k in range(LOG_EXT, -1, -1):
            self.layer_ptr.append(self.layers[off].data_ptr())
            off += 1 << k
        torch.cuda.synchronize()

    def stream(self):
        return ctypes.c_void_p(self.torch.cuda.current_stream().cuda_stream)

    def step(self, ev=None, inputs=None):
        """One commit-stage pass. ev: optional list of 6 CUDA events bracketing the stages.
        inputs: optional (trace pointer table, FRI column pointer table) to read instead of the
        resident inputs (the double-buffered end-to-end leg)."""
        call, st = self.L.call, self.stream()
        t_evals, fri_src = inputs if inputs else (self.t_evals, self.fri_tabs[0])
        rec = (lambda i: ev[i].record()) if ev else (lambda i: None)
        rec(0)
        call("cs_interpolate_columns_into", t_evals, self.t_coeffs, N_COLS, LOG_ROWS, self.itw.data_ptr(),
             self.tw_log, st)
        rec(1)
        call("cs_evaluate_columns", self.t_coeffs, self.t_ext, N_COLS, LOG_ROWS, LOG_EXT, self.tw.data_ptr(),
             self.tw_log, st)
        rec(2)
        call("cs_merkle_build_leaves", self.t_ext, self.logs, N_COLS, LOG_EXT, self.layer_ptr[0], st)
        rec(3)
        # every node layer in the commit layout; the layers of up to 2^10 nodes in one launch
        call("cs_merkle_build_layers", self.layer_ptr[0], LOG_EXT, st)
        rec(4)
        call("cs_fold_circle_into_line", fri_src, FRI_LOG, self.alpha_tabs[0], self.fri_tabs[1],
             self.itw.data_ptr(), self.tw_log, st)
        # FriOps::fold_line with the 21 remaining challenges: one call, the folds in registers and shuffles
        call("cs_fold_line_steps", self.fri_tabs[1], FRI_LOG - 1, FRI_LOG - 1, self.line_alphas,
             self.fri_tabs[FRI_LOG], self.itw.data_ptr(), self.tw_log, st)
        rec(5)

    def root(self) -> bytes:
        return self.layers[-1].cpu().numpy().astype("<i4").tobytes()


class MixedCommit:
    """The batched mixed-size trace: 600 M31 columns with log sizes
    10 + min(12, G), G geometric with mean ~6 (so the mean log size is ~16),
    plus 120 QM31 interaction columns (480 M31 columns) with sizes drawn the
    same way; blowup 2; lifted Blake2s commit of all 1,080 columns at the
    largest extended size. Column contents are seeded uniform M31 (the commit's
    cost does not depend on them)."""

    def __init__(self, torch, seed: int = 7):
        from proving_gb300 import _lib
        from proving_gb300.backend import canonic_half_coset
        from proving_gb300.synthetic import seeded_log_sizes
        self.torch, self.L = torch, _lib
        logs = list(seeded_log_sizes(seed, 600, 10, 22, 16.0))
        inter = seeded_log_sizes(seed + 1, 120, 10, 22, 16.0)
        logs += [int(l) for l in inter for _ in range(4)]
        self.logs = [int(l) for l in logs]
        self.max_ext = max(self.logs) + 1
        dev = torch.device("cuda", torch.cuda.current_device())
        g = torch.Generator(device=dev)
        g.manual_seed(seed)
        P = (1 << 31) - 1
        self.evals = [torch.randint(0, P, (1 << l,), generator=g, device=dev, dtype=torch.int64).to(torch.int32)
                      for l in self.logs]
        self.coeffs = [torch.empty_like(e) for e in self.evals]
        self.ext = [torch.empty(1 << (l + 1), dtype=torch.int32, device=dev) for l in self.logs]
        self.layers = torch.empty(((1 << (self.max_ext + 1)) - 1, 8), dtype=torch.int32, device=dev)
        root = canonic_half_coset(self.max_ext + 1)
        self.tw_log = root.log_size
        self.tw = torch.empty(1 << self.tw_log, dtype=torch.int32, device=dev)
        self.itw = torch.empty_like(self.tw)
        _lib.call("cs_precompute_twiddles", root.initial_index, root.log_size, self.tw.data_ptr(),
                  self.itw.data_ptr(), self.stream())
        vp = ctypes.c_void_p
        self.groups = {}
        for i, l in enumerate(self.logs):
            self.groups.setdefault(l, []).append(i)
        self.tabs = {}
        for l, idx in self.groups.items():
            self.tabs[l] = ((vp * len(idx))(*[self.evals[i].data_ptr() for i in idx]),
                            (vp * len(idx))(*[self.coeffs[i].data_ptr() for i in idx]),
                            (vp * len(idx))(*[self.ext[i].data_ptr() for i in idx]))
        self.all_ext = (vp * len(self.logs))(*[e.data_ptr() for e in self.ext])
        self.all_logs = (ctypes.c_uint32 * len(self.logs))(*[l + 1 for l in self.logs])
        self.elements = sum(1 << l for l in self.logs)
        torch.cuda.synchronize()

    def stream(self):
        return ctypes.c_void_p(self.torch.cuda.current_stream().cuda_stream)

    def step(self, plain: bool = False):
        call, st, vp = self.L.call, self.stream(), ctypes.c_void_p
        for l, idx in self.groups.items():
            ev, co, ex = self.tabs[l]
            if plain:
                # one launch per column per stage
                for k in range(len(idx)):
                    call("cs_interpolate_columns_into", ctypes.byref(vp(ev[k])), ctypes.byref(vp(co[k])), 1, l,
                         self.itw.data_ptr(), self.tw_log, st)
                    call("cs_evaluate_columns", ctypes.byref(vp(co[k])), ctypes.byref(vp(ex[k])), 1, l, l + 1,
                         self.tw.data_ptr(), self.tw_log, st)
            else:
                call("cs_interpolate_columns_into", ev, co, len(idx), l, self.itw.data_ptr(), self.tw_log, st)
                call("cs_evaluate_columns", co, ex, len(idx), l, l + 1, self.tw.data_ptr(), self.tw_log, st)
        call("cs_merkle_commit", self.all_ext, self.all_logs, len(self.logs), self.max_ext, self.layers.data_ptr(), st)


def time_steps(torch, fn, steps: int, warmup: int):
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(steps):
        fn()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / steps


def batched_vs_plain(torch, cs, steps: int = 5, warmup: int = 2):
    """The BASELINE comparison: batched launches (one per stage and size) and the
    same captured in a CUDA graph, against plain one-launch-per-column stages."""
    out = {}
    plain_ms = time_steps(torch, lambda: plain_commit_step(cs), steps, warmup)
    batched_ms = time_steps(torch, cs.step, steps, warmup)
    out["commit_stage"] = {"plain_ms": round(plain_ms, 4), "batched_ms": round(batched_ms, 4),
                           "batched_speedup": round(plain_ms / batched_ms, 3)}
    mixed = MixedCommit(torch)
    m_plain = time_steps(torch, lambda: mixed.step(plain=True), steps, warmup)
    m_batched = time_steps(torch, mixed.step, steps, warmup)
    graph = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    from proving_gb300.serving import collector_paused
    with torch.cuda.stream(s), collector_paused():
        mixed.step()
        torch.cuda.synchronize()
        with torch.cuda.graph(graph, stream=s):
            mixed.step()
    torch.cuda.current_stream().wait_stream(s)
    m_graph = time_steps(torch, graph.replay, steps, warmup)
    out["mixed_commit"] = {
        "workload": "600 M31 + 120 QM31 (480 M31) columns, log sizes 10..22 geometric (mean ~16), blowup 2, "
                    "lifted Blake2s commit",
        "columns": len(mixed.logs), "distinct_sizes": len(mixed.groups), "trace_elements": mixed.elements,
        "plain_ms": round(m_plain, 4), "batched_ms": round(m_batched, 4), "graph_ms": round(m_graph, 4),
        "plain_commits_per_s": round(1e3 / m_plain, 3), "batched_commits_per_s": round(1e3 / m_batched, 3),
        "graph_commits_per_s": round(1e3 / m_graph, 3),
        "batched_speedup": round(m_plain / m_batched, 3), "graph_speedup": round(m_plain / m_graph, 3)}
    del mixed
    return out


def plain_commit_step(cs):
    """The commit stage with one launch per column for interpolate and evaluate."""
    call, st, vp = cs.L.call, cs.stream(), ctypes.c_void_p
    for k in range(N_COLS):
        call("cs_interpolate_columns_into", ctypes.byref(vp(cs.t_evals[k])), ctypes.byref(vp(cs.t_coeffs[k])), 1,
             LOG_ROWS, cs.itw.data_ptr(), cs.tw_log, st)
    for k in range(N_COLS):
        call("cs_evaluate_columns", ctypes.byref(vp(cs.t_coeffs[k])), ctypes.byref(vp(cs.t_ext[k])), 1, LOG_ROWS,
             LOG_EXT, cs.tw.data_ptr(), cs.tw_log, st)
    call("cs_merkle_build_leaves", cs.t_ext, cs.logs, N_COLS, LOG_EXT, cs.layer_ptr[0], st)
    for k in range(LOG_EXT, 0, -1):
        call("cs_merkle_build_next_layer", cs.layer_ptr[LOG_EXT - k], k - 1, cs.layer_ptr[LOG_EXT - k + 1], st)
    call("cs_fold_circle_into_line", cs.fri_tabs[0], FRI_LOG, cs.alpha_tabs[0], cs.fri_tabs[1], cs.itw.data_ptr(),
         cs.tw_log, st)
    for j in range(1, FRI_LOG):
        call("cs_fold_line", cs.fri_tabs[j], FRI_LOG - j, cs.alpha_tabs[j], cs.fri_tabs[j + 1], cs.itw.data_ptr(),
             cs.tw_log, st)


def wide_fib_prove_native(torch, n_proofs: int = 20, log_n: int = 14, n_cols: int = 100, plain: bool = False):
    """The Wide-Fibonacci proof (100 x 2^14) through the native prover (cs_prove_wide_fib): the same proof bytes as the restated
    prover, the host work in C++. Trace generated on the device from seeded inputs inside the
    timed region. Returns wall-clock latencies in ms."""
    from proving_gb300 import prover as pr
    from proving_gb300.backend import BaseColumn, CudaBackend
    from proving_gb300.synthetic import m31_column
    ops = pr.GpuOps()
    tw = ops.twiddles(log_n + 2)
    fp = (10, 1, 0, 70)
    lat = []
    for k in range(n_proofs + 2):
        a = BaseColumn.from_cpu(m31_column(100 + k, log_n))
        b = BaseColumn.from_cpu(m31_column(200 + k, log_n))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        trace = CudaBackend.wide_fib_trace(a, b, n_cols)
        CudaBackend.prove_wide_fib_native([trace], [log_n], fp, tw, plain=plain)
        torch.cuda.synchronize()
        if k >= 2:
            lat.append((time.perf_counter() - t0) * 1e3)
    return lat


def wide_fib_prove_latency(torch, n_proofs: int = 8, log_n: int = 14, n_cols: int = 100):
    """Full Wide-Fibonacci proves (100 columns x 2^14 rows, blowup 2,
    70 queries, pow 10) through the restated prover on the CUDA backend; the
    trace is generated on the device from seeded inputs. Returns wall-clock
    latencies in ms (host orchestration included)."""
    from proving_gb300 import prover as pr
    from proving_gb300.backend import BaseColumn, CudaBackend
    from proving_gb300.synthetic import m31_column
    ops = pr.GpuOps()
    fp = pr.FriParams(pow_bits=10, log_blowup_factor=1, log_last_layer_degree_bound=0, n_queries=70, fold_step=1)
    cfg = pr.PcsConfig(fp, trace_lifting_log_size=log_n + 1)
    tw = ops.twiddles(log_n + 2)
    lat = []
    for k in range(n_proofs + 2):
        a = BaseColumn.from_cpu(m31_column(100 + k, log_n))
        b = BaseColumn.from_cpu(m31_column(200 + k, log_n))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        trace = CudaBackend.wide_fib_trace(a, b, n_cols)
        proof = pr.prove_wide_fib(ops, trace, log_n, cfg, pr.Blake2sChannel(), tw)
        torch.cuda.synchronize()
        if k >= 2:
            lat.append((time.perf_counter() - t0) * 1e3)
    return lat


def wide_fib_generic_native_latency(torch, n_proofs: int = 8, log_n: int = 14, n_cols: int = 100):
    """The same Wide-Fibonacci proves through the native generic prover (cs_prove_air via
    air_prover.prove_native: the NVRTC kernel of wide_fib_air, the constraints at the OODS point from
    its node program). The first proof is checked against the restated prover's bytes. Returns
    wall-clock latencies in ms."""
    from proving_gb300 import air_prover as ap
    from proving_gb300 import framework as fw
    from proving_gb300 import prover as pr
    from proving_gb300.backend import BaseColumn, CudaBackend
    from proving_gb300.synthetic import m31_column
    ops = pr.GpuOps()
    fp = pr.FriParams(pow_bits=10, log_blowup_factor=1, log_last_layer_degree_bound=0, n_queries=70, fold_step=1)
    cfg = pr.PcsConfig(fp, trace_lifting_log_size=log_n + 1)
    tw = ops.twiddles(log_n + 2)
    air = fw.compile_air(f"wide_fib_{n_cols}", fw.wide_fib_air, n_cols)
    fw.CompiledAir.get(air)
    comp = ap.FrameworkComponent(ap.TraceLocationAllocator(), air, log_n)
    lat = []
    for k in range(n_proofs + 2):
        a = BaseColumn.from_cpu(m31_column(100 + k, log_n))
        b = BaseColumn.from_cpu(m31_column(200 + k, log_n))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        trace = CudaBackend.wide_fib_trace(a, b, n_cols)
        words = ap.prove_native([comp], trace, cfg, tw)
        torch.cuda.synchronize()
        if k >= 2:
            lat.append((time.perf_counter() - t0) * 1e3)
        if k == 0:
            want = pr.prove_wide_fib(ops, CudaBackend.wide_fib_trace(a, b, n_cols), log_n, cfg, pr.Blake2sChannel(), tw)
            if words != want.to_bytes():
                raise RuntimeError("native generic prover proof differs from the restated prover's")
    return lat


def wide_fib_generic_latency(torch, n_proofs: int = 8, log_n: int = 14, n_cols: int = 100):
    """The same Wide-Fibonacci proves through the generic prover API (proving_gb300.air_prover: the
    AIR recorded by the constraint evaluator, its composition kernel compiled with NVRTC once,
    before the timed proofs). The first proof is checked against the restated prover's bytes.
    Returns wall-clock latencies in ms."""
    from proving_gb300 import air_prover as ap
    from proving_gb300 import framework as fw
    from proving_gb300 import prover as pr
    from proving_gb300.backend import BaseColumn, CudaBackend
    from proving_gb300.synthetic import m31_column
    ops = pr.GpuOps()
    fp = pr.FriParams(pow_bits=10, log_blowup_factor=1, log_last_layer_degree_bound=0, n_queries=70, fold_step=1)
    cfg = pr.PcsConfig(fp, trace_lifting_log_size=log_n + 1)
    tw = ops.twiddles(log_n + 2)
    air = fw.compile_air(f"wide_fib_{n_cols}", fw.wide_fib_air, n_cols)
    fw.CompiledAir.get(air)
    lat = []
    for k in range(n_proofs + 2):
        a = BaseColumn.from_cpu(m31_column(100 + k, log_n))
        b = BaseColumn.from_cpu(m31_column(200 + k, log_n))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        trace = CudaBackend.wide_fib_trace(a, b, n_cols)
        ch = pr.Blake2sChannel()
        scheme = ap.CommitmentSchemeProver(ops, cfg, tw)
        scheme.commit([], ch)
        scheme.commit(trace, ch)
        proof = ap.prove([ap.FrameworkComponent(ap.TraceLocationAllocator(), air, log_n)], ch, scheme)
        torch.cuda.synchronize()
        if k >= 2:
            lat.append((time.perf_counter() - t0) * 1e3)
        if k == 0:
            want = pr.prove_wide_fib(ops, CudaBackend.wide_fib_trace(a, b, n_cols), log_n, cfg, pr.Blake2sChannel(), tw)
            if proof.to_bytes() != want.to_bytes():
                raise RuntimeError("generic prover proof differs from the restated prover's")
    return lat


def mixed_prove_leg(torch, n_proofs: int = 2, arms=("batched", "plain", "native", "native_plain")):
    """The batched mixed-size trace as a full proof (mixed_trace_shape: Wide-Fibonacci
    components holding 480 M31 columns and 120 single-column LogUp components, each with one M31
    value column and one QM31 running-sum column, log sizes 10..22 geometric, mean ~16) proved by
    prove_fib_and_lookups with log_blowup 1, 70 queries, pow 10, one lifted tree per phase.
    Traces and lookup values are generated on the device from seeds inside the timed region.
    Arms: the batched path (one launch per stage and size), the plain path (one launch per column
    for the per-column stages), both with the restated prover's host orchestration, and the batched
    kernels under the native prover (cs_prove_fib_and_lookups); all give the same proof bytes."""
    from proving_gb300 import prover as pr
    from proving_gb300.backend import BaseColumn, CudaBackend
    from proving_gb300.synthetic import m31_column, mixed_trace_shape
    comps, lookup_logs = mixed_trace_shape()
    max_log = max([l for _, l in comps] + lookup_logs)
    fp = pr.FriParams(pow_bits=10, log_blowup_factor=1, log_last_layer_degree_bound=0, n_queries=70, fold_step=1)
    cfg = pr.PcsConfig(fp, trace_lifting_log_size=max_log + 1)
    seeds = [(BaseColumn.from_cpu(m31_column(300 + i, l)), BaseColumn.from_cpu(m31_column(400 + i, l)))
             for i, (_, l) in enumerate(comps)]
    host_values = [m31_column(500 + k, l) for k, l in enumerate(lookup_logs)]
    out = {"workload": f"{sum(n for n, _ in comps)} Wide-Fibonacci columns in {len(comps)} components + "
                       f"{len(lookup_logs)} LogUp components (value column + QM31 running sum), log sizes 10..22 "
                       f"geometric (mean ~16), log_blowup 1, 70 queries, pow 10, lifting {max_log + 1}",
           "base_columns": sum(n for n, _ in comps) + len(lookup_logs), "interaction_columns": len(lookup_logs)}
    digests = {}
    for name, ops in (("batched", pr.GpuOps()), ("plain", pr.PlainGpuOps())):
        if name not in arms:
            continue
        tw = ops.twiddles(max_log + 2)
        lat = []
        for k in range(n_proofs + 1):
            values = [BaseColumn.from_cpu(v) for v in host_values]
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            traces = [CudaBackend.wide_fib_trace(a, b, n) for (a, b), (n, _) in zip(seeds, comps)]
            proof = pr.prove_fib_and_lookups(ops, traces, [l for _, l in comps], values, lookup_logs, cfg,
                                             pr.Blake2sChannel(), tw)
            torch.cuda.synchronize()
            if k >= 1:
                lat.append((time.perf_counter() - t0) * 1e3)
            del traces, values
        digests[name] = hashlib.sha256(proof.to_bytes()).hexdigest()
        out[name] = {"proofs_per_s": round(1e3 / statistics.median(lat), 3), "p50_ms": round(statistics.median(lat), 3),
                     "max_ms": round(max(lat), 3)}
        del proof, tw
        torch.cuda.empty_cache()
    from proving_gb300 import _lib
    for name in ("native", "native_plain"):
        if name not in arms:
            continue
        # the host work in native code (cs_prove_fib_and_lookups): batched stages, or with CS_PROVE_PLAIN
        # one launch per column for every per-column stage
        ops = pr.GpuOps()
        tw = ops.twiddles(max_log + 2)
        fpt = (fp.pow_bits, fp.log_blowup_factor, fp.log_last_layer_degree_bound, fp.n_queries)
        lat, launches = [], []
        for k in range(n_proofs + 1):
            values = [BaseColumn.from_cpu(v) for v in host_values]
            torch.cuda.synchronize()
            n0 = _lib.load().cs_kernel_launch_count()
            t0 = time.perf_counter()
            traces = [CudaBackend.wide_fib_trace(a, b, n) for (a, b), (n, _) in zip(seeds, comps)]
            words, _ = CudaBackend.prove_fib_and_lookups_native(traces, [l for _, l in comps], values, lookup_logs,
                                                                 fpt, tw, plain=name == "native_plain")
            torch.cuda.synchronize()
            if k >= 1:
                lat.append((time.perf_counter() - t0) * 1e3)
                launches.append(_lib.load().cs_kernel_launch_count() - n0)
            del traces, values
        digest = hashlib.sha256(words).hexdigest()
        out[name] = {"proofs_per_s": round(1e3 / statistics.median(lat), 3),
                     "p50_ms": round(statistics.median(lat), 3), "max_ms": round(max(lat), 3),
                     "kernel_launches_per_proof": int(statistics.median(launches)),
                     "same_proof_bytes": (digest == next(iter(digests.values())) if digests else None)}
        digests[name] = digest
        del tw
        torch.cuda.empty_cache()
    if "native" in out and "native_plain" in out:
        out["native_batched_over_plain"] = round(out["native_plain"]["p50_ms"] / out["native"]["p50_ms"], 3)
    out["proof_sha256"] = next(iter(digests.values())) if digests else None
    out["all_arms_same_proof_bytes"] = len(set(digests.values())) == 1
    if "plain" in arms:
        out["same_proof_bytes"] = digests["batched"] == digests["plain"]
        out["batched_speedup"] = round(out["plain"]["p50_ms"] / out["batched"]["p50_ms"], 3)
    return out


def int_peaks(torch):
    """Measured integer-pipe throughput (cs_int_peak_probe): thread operations per second for
    3-input adds, 3-input logic and funnel shifts (the ALU pipe) and multiply-adds (the FMA pipe),
    the denominator of the integer-bound kernels."""
    from proving_gb300 import _lib
    blocks, iters = 152 * 8, 1 << 14
    out = torch.empty(blocks * 256, dtype=torch.int32, device="cuda")
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    res = {}
    for kind, name in enumerate(("iadd3", "lop3", "shf", "imad")):
        fn = lambda: _lib.call("cs_int_peak_probe", kind, blocks, iters, out.data_ptr(), st)
        ms = time_steps(torch, fn, 3, 2)
        res[f"{name}_tops"] = round(blocks * 256 * 8 * iters / (ms / 1e3) / 1e12, 3)
    return res


def poseidon_prove_leg(torch, log_n_rows: int = 18, n_proofs: int = 2):
    """The Poseidon2 AIR at 8 permutations per row, 2^log_n_rows rows (1264 trace
    columns), log_blowup_factor 1, 70 queries, pow 10, through prove_poseidon + prove_ex on the
    CUDA backend (trace, interaction trace and constraint quotients on the device). The
    reference's own prove of this AIR stops at its sanity check (lifted protocol, constraint
    degree 5), so the proof is built with check=False. Reports the wall-clock latency and the
    device time of the constraint-quotient kernel alone."""
    from proving_gb300 import poseidon as ps
    from proving_gb300 import prover as pr
    from proving_gb300.backend import CudaBackend, SecureColumnByCoords
    ops = pr.GpuOps()
    fp = pr.FriParams(pow_bits=10, log_blowup_factor=1, log_last_layer_degree_bound=0, n_queries=70, fold_step=1)
    cfg = ps.poseidon_pcs_config(log_n_rows + 3, fp)
    tw = ops.twiddles(log_n_rows + ps.LOG_EXPAND + fp.log_blowup_factor)
    lat, nat, nplain = [], [], []
    fpt = (fp.pow_bits, fp.log_blowup_factor, fp.log_last_layer_degree_bound, fp.n_queries)
    for k in range(n_proofs + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ps.prove_poseidon(ops, log_n_rows, cfg, pr.Blake2sChannel(), tw, check=False)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        CudaBackend.prove_poseidon_native(log_n_rows, fpt, tw)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        CudaBackend.prove_poseidon_native(log_n_rows, fpt, tw, plain=True)
        torch.cuda.synchronize()
        if k >= 1:
            lat.append((t1 - t0) * 1e3)
            nat.append((t2 - t1) * 1e3)
            nplain.append((time.perf_counter() - t2) * 1e3)
    # the same proof through the native generic prover: the AIR recorded by the constraint evaluator
    # (its composition and fraction kernels compiled once with NVRTC, before the timed proofs), the
    # interaction trace from its fractions; bytes checked against cs_prove_poseidon
    from proving_gb300 import air_prover as ap
    from proving_gb300 import framework as fw
    air = fw.poseidon_air_recorded()
    fw.CompiledAir.get(air)
    comp = ap.FrameworkComponent(ap.TraceLocationAllocator(), air, log_n_rows, constraint_log_degree=ps.LOG_EXPAND)
    gen = []
    for k in range(n_proofs + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        words = ap.prove_native([comp], CudaBackend.poseidon_trace(log_n_rows), cfg, tw)
        torch.cuda.synchronize()
        if k >= 1:
            gen.append((time.perf_counter() - t0) * 1e3)
        if k == 0 and words != CudaBackend.prove_poseidon_native(log_n_rows, fpt, tw):
            raise RuntimeError("native generic Poseidon2 proof differs from cs_prove_poseidon's")
    torch.cuda.empty_cache()
    # the constraint-quotient kernel alone on the evaluation domain CanonicCoset(log_n_rows + 2)
    eval_log = log_n_rows + ps.LOG_EXPAND
    trace = CudaBackend.poseidon_trace(log_n_rows)
    lookup = [1, 2, 3, 4, 4, 3, 2, 1]
    inter, claimed = CudaBackend.poseidon_interaction(trace, lookup)
    coeffs = ops.interpolate_into(trace, tw)
    del trace
    t_eval = ops.evaluate(coeffs, eval_log, tw)
    del coeffs
    ops.interpolate(inter, tw)
    i_eval = ops.evaluate(inter, eval_log, tw)
    rc = np.random.default_rng(1).integers(0, (1 << 31) - 1, (ps.N_CONSTRAINTS, 4)).astype(np.uint32)
    acc = SecureColumnByCoords.zeros(1 << eval_log)
    ms = time_steps(torch, lambda: CudaBackend.poseidon_composition(t_eval, i_eval, log_n_rows, lookup, claimed, rc,
                                                                     acc), 3, 1)
    read_bytes = 4 * (ps.N_COLUMNS + ps.N_INTERACTION_COLUMNS) * (1 << eval_log) + 4 * 4 * (1 << eval_log)
    out = {"workload": f"Poseidon2 AIR, 8 permutations/row, 2^{log_n_rows} rows (2^{log_n_rows + 3} permutations), "
                       "1264 trace + 32 interaction columns, log_blowup 1, 70 queries, pow 10; prove_poseidon + "
                       "prove_ex (the reference's sanity check fails for this AIR; proof built without it)",
           "proofs_per_s": round(1e3 / statistics.median(nat), 3), "p50_ms": round(statistics.median(nat), 3),
           "max_ms": round(max(nat), 3), "prover": "native (cs_prove_poseidon); restated beside it",
           "restated": {"proofs_per_s": round(1e3 / statistics.median(lat), 3),
                        "p50_ms": round(statistics.median(lat), 3)},
           "native_plain": {"proofs_per_s": round(1e3 / statistics.median(nplain), 3),
                            "p50_ms": round(statistics.median(nplain), 3)},
           "generic_native": {"proofs_per_s": round(1e3 / statistics.median(gen), 3),
                              "p50_ms": round(statistics.median(gen), 3),
                              "note": "cs_prove_air over the NVRTC kernels of poseidon_air (composition and "
                                      "LogUp fractions); bytes checked against cs_prove_poseidon"},
           "composition_kernel": {"eval_rows": 1 << eval_log, "ms": round(ms, 4),
                                  "gb_per_s": round(read_bytes / ms / 1e6, 1),
                                  "rows_per_s": round((1 << eval_log) / ms * 1e3, 1)}}
    del t_eval, i_eval, acc
    torch.cuda.empty_cache()
    return out


def _verify_wide_fib_proof(args):
    """Restated verifier on one served Wide-Fibonacci proof (run in a spawned worker)."""
    words, log_n = args
    from oracle.verifier import parse_proof, verify_wide_fib_components
    verify_wide_fib_components(parse_proof(words, log_n + 1), [100], [log_n])
    return True


def serving_leg(n_requests: int = 200, rate_fracs=(0.25, 0.5, 0.9)):
    """Serving: seeded Poisson streams of proof requests, half Wide-Fibonacci (100 columns) and half
    Poseidon2 (8 permutations per row), log_n_rows uniform in [12, 20]. Arms, all native provers:
    plain (1 worker, one launch per column for every per-column stage, CS_PROVE_PLAIN), batched_serial
    (1 worker, batched stages), served (4 worker threads of one process, a CUDA stream each, HBM-budget
    admission in arrival order: the stages of different requests overlap on the device), and at
    saturation served_processes (4 worker processes, a CUDA context each). First every arm serves the
    stream all at once (capacity); then Poisson streams at fractions of the served capacity. Every
    proof of every arm is compared with the same request proved alone (batched_serial at saturation),
    and every served Wide-Fibonacci proof is accepted by the restated verifier."""
    import multiprocessing as mp
    from proving_gb300 import serving
    out = {"workload": f"{n_requests} requests per run, 50% Wide-Fibonacci (100 cols) / 50% Poseidon2 "
                       "(8 perms/row), log_n_rows uniform in [12, 20]; Poisson arrivals",
           "arms": "plain: 1 worker, one launch per column per stage (native, CS_PROVE_PLAIN); batched_serial: "
                   "1 worker, batched stages (native); served: 4 worker threads (one CUDA context, a stream "
                   "each), HBM-budget admission in arrival order (native); served_processes: 4 worker "
                   "processes, a CUDA context each"}
    # warm-up outside the timed streams: the kernels of every tile size load on their first launch
    warm = [serving.ProofRequest(-1 - i, log_n, 1 + i, kind)
            for i, (log_n, kind) in enumerate((l, k) for l in (12, 16, 20) for k in ("wide_fib", "poseidon"))]
    serving.run_stream(4, [(0.0, r) for r in warm], max_log=20, native=True)
    serving.run_stream(1, [(0.0, r) for r in warm], max_log=20, native=True, plain=True)

    def stream(rate):
        reqs = serving.poisson_requests(n_requests, rate if rate else 1.0, 12, 20, seed=5, poseidon_share=0.5)
        return [(0.0 if rate is None else g, r) for g, r in reqs]

    arms = {"plain": dict(n_workers=1, plain=True), "batched_serial": dict(n_workers=1),
            "served": dict(n_workers=4)}
    alone, same, kinds = {}, True, {}
    sat = {}
    for name in ("batched_serial", "plain", "served"):
        done, wall = serving.run_stream(arms[name]["n_workers"], stream(None), max_log=20, native=True,
                                        plain=arms[name].get("plain", False))
        sat[name] = serving.summarize(done, wall)
        for r in done:
            kinds[r.request_id] = (r.kind, r.log_n_rows)
            if name == "batched_serial":
                alone[r.request_id] = r.proof_bytes()
            else:
                same = same and r.error is None and r.proof_bytes() == alone.get(r.request_id)
        if name == "served":
            served_done = done
    svc = serving.ProcessProverService(n_workers=4, max_log_n_rows=20)
    try:
        done, wall = svc.run(stream(None))
    finally:
        svc.close()
    sat["served_processes"] = serving.summarize(done, wall)
    same = same and all(r.error is None and r.proof_bytes() == alone.get(r.request_id) for r in done)
    out["saturation"] = sat
    capacity = sat["served"]["proofs_per_s"]
    out["capacity_proofs_per_s"] = capacity
    sweep = {}
    for frac in rate_fracs:
        rate = frac * capacity
        row = {"rate_per_s": round(rate, 2)}
        for name in ("plain", "batched_serial", "served"):
            done, wall = serving.run_stream(arms[name]["n_workers"], stream(rate), max_log=20, native=True,
                                            plain=arms[name].get("plain", False))
            row[name] = serving.summarize(done, wall)
            same = same and all(r.error is None and r.proof_bytes() == alone.get(r.request_id) for r in done)
        sweep[f"{frac:.2f}"] = row
    out["sweep"] = sweep
    out["same_proof_bytes"] = bool(same)
    # the restated verifier on every served Wide-Fibonacci proof (spawned workers: CUDA is initialised here)
    items = [(r.proof_bytes(), r.log_n_rows) for r in served_done if r.kind == "wide_fib"]
    with mp.get_context("spawn").Pool(min(8, os.cpu_count() or 1)) as pool:
        ok = pool.map(_verify_wide_fib_proof, items)
    out["verified_wide_fib_proofs"] = int(sum(ok))
    out["served_over_plain"] = round(sat["served"]["proofs_per_s"] / sat["plain"]["proofs_per_s"], 3)
    out["batched_serial_over_plain"] = round(sat["batched_serial"]["proofs_per_s"] / sat["plain"]["proofs_per_s"], 3)
    return out


def replica_throughput(dist, elapsed_ms: float, steps: int, world: int, device="cpu"):
    """Whole-job throughput of `world` independent replicas (one per GPU, no data-path collective):
    every rank processed `steps` units, and the job took the slowest rank's time, so the time is
    the maximum over ranks (an all-reduce, the only collective). Returns (max_ms, units per s)."""
    import torch
    t = torch.tensor([float(elapsed_ms)], dtype=torch.float64, device=device)
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    max_ms = float(t.item())
    return max_ms, world * steps / (max_ms / 1e3)


def run_gpu(args):
    import torch
    from proving_gb300 import _lib
    from proving_gb300 import build as cuda_build

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
        # replicas hold every GPU while they run: only the headline step and its end-to-end form are
        # timed, the per-config legs run in single-GPU runs
        for leg in ("skip_prove", "skip_plain", "skip_poseidon", "skip_mixed_prove", "skip_gkr", "skip_serving"):
            setattr(args, leg, True)
    else:
        dist = None
        torch.cuda.set_device(0)
    if rank == 0 or world == 1:
        cuda_build.build()
    if dist:
        dist.barrier()
    L = _lib.load()

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    # the FFT pass plans for this workload's two shapes, picked by the autotuner before timing
    from proving_gb300 import autotune
    tuned = {} if args.skip_autotune else autotune.tune([(True, LOG_ROWS, LOG_ROWS), (False, LOG_EXT, LOG_ROWS)],
                                                        n_cols=N_COLS)
    fft_plans = {f"{'interpolate' if inv else 'evaluate'} 2^{log_n} ({n} layers)":
                 {"default": list(r["default"]), "best": list(r["best"]),
                  "default_ms": round(r["ms"][tuple(r["default"])], 4), "best_ms": round(r["ms"][r["best"]], 4),
                  "candidates": len(r["ms"])}
                 for (inv, log_n, n), r in tuned.items()}
    cs = CommitStage(torch)
    for _ in range(args.warmup):
        cs.step()
    barrier()

    n_ev = 6
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(n_ev)] for _ in range(args.steps)]
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = L.cs_kernel_launch_count()
    with ClockSampler(torch.cuda.current_device()) as clk:
        barrier()
        start.record()
        for k in range(args.steps):
            cs.step(evs[k])
        end.record()
        barrier()
    launches = L.cs_kernel_launch_count() - launches0
    elapsed_ms = start.elapsed_time(end)
    stage_names = ["interpolate", "evaluate", "merkle_leaves", "merkle_nodes", "fri_folds"]
    stage_ms = {n: statistics.mean(evs[k][i].elapsed_time(evs[k][i + 1]) for k in range(args.steps))
                for i, n in enumerate(stage_names)}
    step_lat = [evs[k][0].elapsed_time(evs[k][5]) for k in range(args.steps)]
    max_ms, value = replica_throughput(dist, elapsed_ms, args.steps, world, device="cuda")

    # ---- e2e through the C ABI with host buffers: every step copies its trace and FRI column from
    # pinned host memory and reads its Merkle root and last FRI value back. Inputs are double
    # buffered: step k + 1's copy runs on a copy stream while step k computes.
    host_evals = torch.empty((N_COLS, 1 << LOG_ROWS), dtype=torch.int32, pin_memory=True)
    host_evals.copy_(cs.evals.cpu())
    host_fri = torch.empty((4, 1 << FRI_LOG), dtype=torch.int32, pin_memory=True)
    host_fri.copy_(cs.fri_src.cpu())
    host_out = torch.empty((max(args.steps, args.warmup, 1), 16), dtype=torch.int32, pin_memory=True)
    h2d = host_evals.numel() * 4 + host_fri.numel() * 4
    d2h = 32 + 16
    evals2, fri2 = torch.empty_like(cs.evals), torch.empty_like(cs.fri_src)
    vp = ctypes.c_void_p
    buffers = [(cs.evals, cs.fri_src, (cs.t_evals, cs.fri_tabs[0])),
               (evals2, fri2, ((vp * N_COLS)(*[evals2[i].data_ptr() for i in range(N_COLS)]),
                               (vp * 4)(*[fri2[k].data_ptr() for k in range(4)])))]
    copy_stream = torch.cuda.Stream()

    def e2e_run(n_steps: int, lat=None, start=None):
        comp = torch.cuda.current_stream()
        if start is not None:
            copy_stream.wait_event(start)  # the first copy is inside the timed region
        st_copy, st_comp = vp(copy_stream.cuda_stream), vp(comp.cuda_stream)
        copied = [torch.cuda.Event() for _ in range(2)]
        freed = [torch.cuda.Event() for _ in range(2)]

        starts, ends = [], []

        def copy_in(b):
            dev_evals, dev_fri, _ = buffers[b]
            if lat is not None:
                starts.append(torch.cuda.Event(enable_timing=True))
                starts[-1].record(copy_stream)
            _lib.call("cs_memcpy_h2d", dev_evals.data_ptr(), host_evals.data_ptr(), h2d - host_fri.numel() * 4,
                      st_copy)
            _lib.call("cs_memcpy_h2d", dev_fri.data_ptr(), host_fri.data_ptr(), host_fri.numel() * 4, st_copy)
            copied[b].record(copy_stream)

        copy_in(0)
        for k in range(n_steps):
            b = k % 2
            if k + 1 < n_steps:
                if k >= 1:
                    copy_stream.wait_event(freed[1 - b])
                copy_in(1 - b)
            comp.wait_event(copied[b])
            cs.step(inputs=buffers[b][2])
            freed[b].record(comp)
            _lib.call("cs_memcpy_d2h", host_out[k].data_ptr(), cs.layers[-1].data_ptr(), 32, st_comp)
            _lib.call("cs_memcpy_d2h", host_out[k].data_ptr() + 32, cs.fri_layers[-1].data_ptr(), 16, st_comp)
            if lat is not None:
                ends.append(torch.cuda.Event(enable_timing=True))
                ends[-1].record(comp)
        _lib.call("cs_stream_synchronize", st_comp)
        if lat is not None:
            # per step: from the start of its input copy to its result in host memory
            lat.extend(a.elapsed_time(e) for a, e in zip(starts, ends))

    e_lat = [float("nan")]
    e2e_ms = float("nan")
    if not args.skip_e2e:
        e2e_run(max(1, args.warmup))
        barrier()
        e_start, e_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e_lat = []
        e_start.record()
        e2e_run(args.steps, e_lat, e_start)
        e_end.record()
        barrier()
        e2e_ms = e_start.elapsed_time(e_end)
        # the root read back by the last step is the resident step's root
        assert bytes(host_out[args.steps - 1, :8].numpy().astype("<i4").tobytes()) == cs.root()
    _, e2e_value = replica_throughput(dist, e2e_ms, args.steps, world, device="cuda")

    peaks_int = int_peaks(torch)
    from proving_gb300.serving import collector_paused
    with collector_paused():
        wf_lat = wide_fib_prove_latency(torch) if not args.skip_prove else []
        wf_generic = wide_fib_generic_latency(torch) if not args.skip_prove else []
        wf_generic_native = wide_fib_generic_native_latency(torch) if not args.skip_prove else []
        wf_native = wide_fib_prove_native(torch) if not args.skip_prove else []
        wf_plain = wide_fib_prove_native(torch, plain=True) if not args.skip_prove else []
    bvp = batched_vs_plain(torch, cs) if not args.skip_plain else None
    with collector_paused():
        poseidon_res = poseidon_prove_leg(torch, args.poseidon_log_rows) if not args.skip_poseidon else None
        mixed_res = mixed_prove_leg(torch) if not args.skip_mixed_prove else None
    gkr_res = gkr_leg(torch) if not args.skip_gkr else None
    # last: its threaded arm proves in this process, and the other legs measure a fresh state
    serving_res = serving_leg() if not args.skip_serving else None
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    hbm, peak_kind = peaks()
    default_shape = (N_COLS, LOG_ROWS, LOG_EXT) == (256, 20, 22)
    # dominant kernel: the evaluate FFT (fft_tile_kernel, two tile passes per step); algorithmic
    # bytes per column are 4 n_in + 4 n_out (coefficients read once, the blown-up evaluation written)
    eval_ms = stage_ms["evaluate"]
    eval_bytes = N_COLS * 4 * ((1 << LOG_ROWS) + (1 << LOG_EXT))
    achieved = eval_bytes / (eval_ms / 1e3) / 1e9
    eval_traffic = EVALUATE_TRAFFIC_BYTES if default_shape else None
    # the Blake2s leaf hashing (one launch per step): 4 bytes per column value read, 32 per leaf written
    leaf_ms = stage_ms["merkle_leaves"]
    leaf_bytes = N_COLS * (1 << LOG_EXT) * 4 + (1 << LOG_EXT) * 32
    leaf_gbs = leaf_bytes / (leaf_ms / 1e3) / 1e9
    leaf_comp = (1 << LOG_EXT) * ((N_COLS * 4 + 63) // 64)
    traffic = LEAVES_TRAFFIC_BYTES if default_shape else None
    fold_bytes = 16 * (1 << FRI_LOG) + 16 * (1 << (FRI_LOG - 1)) + 16 * (1 << (FRI_LOG - 1)) + 16
    # the CPU baseline is timed once, on rank 0 of a single-GPU run
    cpu = cpu_baseline(args) if not args.no_cpu_baseline and world == 1 else None
    ff = lambda x: float(f"{x:.6g}")
    res = {
        "metric": METRIC, "value": ff(value), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ff(max_ms / args.steps), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32 (M31 field words)", "data": "synthetic (seeded)",
        "config": {"workload": workload_name(), "n_cols": N_COLS, "log_rows": LOG_ROWS, "log_blowup": LOG_BLOWUP,
                   "merkle_height": LOG_EXT, "fri_log_size": FRI_LOG, "fri_folds": FRI_LOG,
                   "l2": "inputs larger than L2 (1 GiB trace, 4 GiB extension); no flush",
                   "parallelism": f"replicas x{world}"},
        "latency_ms": {"p50": ff(float(np.percentile(step_lat, 50))), "p99": ff(float(np.percentile(step_lat, 99))),
                       "e2e_p50": ff(float(np.percentile(e_lat, 50))), "e2e_p99": ff(float(np.percentile(e_lat, 99)))},
        "stages_ms": {k: ff(v) for k, v in stage_ms.items()},
        "e2e": {"value": ff(e2e_value), "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": {"bound": "hbm", "kernel": "fft_tile_kernel (evaluate: 2 tile passes per step)",
                     "achieved": ff(achieved), "peak": hbm, "unit": "GB/s", "frac": ff(achieved / hbm),
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json)", "traffic": eval_traffic,
                     "algorithmic_bytes_per_evaluate": eval_bytes, "launches_per_evaluate": 2,
                     "note": "achieved and traffic are per evaluate (both passes); the passes are bound by "
                             "integer issue (about 11.4 thread instructions per butterfly, most of them the "
                             "M31 multiply-reduce and the two reduced additions), and traffic counts the "
                             "intermediate of the two-pass FFT written once and read once"},
        "leaves_roofline": {"bound": "hbm", "kernel": "merkle_leaves_kernel", "achieved": ff(leaf_gbs), "peak": hbm,
                            "unit": "GB/s", "frac": ff(leaf_gbs / hbm), "traffic": traffic,
                            "algorithmic_bytes_per_launch": leaf_bytes,
                            "note": "Blake2s leaf hashing is integer-pipe bound; see int_pipe"},
        "fold_roofline": {"bound": "hbm", "kernels": "fold_circle_wide_kernel + fold_line_regs_kernel (3 launches: 2^22 -> 2^21, 12 folds, 9 folds; 16 values a thread)",
                          "achieved": ff(fold_bytes / (stage_ms["fri_folds"] / 1e3) / 1e9), "peak": hbm,
                          "unit": "GB/s", "frac": ff(fold_bytes / (stage_ms["fri_folds"] / 1e3) / 1e9 / hbm),
                          "algorithmic_bytes": fold_bytes,
                          "note": "fold_circle_into_line 16 n + 16 n/2 bytes, then fold_line with 21 challenges "
                                  "16 n/2 + 16 bytes (input read once, last layer written); the FRI column was "
                                  "last touched a step earlier, so it is read from HBM"},
        "int_pipe": {"kernel": "merkle_leaves_kernel", "compressions_per_launch": leaf_comp,
                     "gcompressions_per_s": ff(leaf_comp / (leaf_ms / 1e3) / 1e9),
                     "int_ops_per_compression": 1120,
                     "tops_achieved": ff(leaf_comp * 1120 / (leaf_ms / 1e3) / 1e12),
                     "alu_peak_tops_measured": max(peaks_int["iadd3_tops"], peaks_int["lop3_tops"],
                                                   peaks_int["shf_tops"]),
                     "fma_peak_tops_measured": peaks_int["imad_tops"],
                     "note": "1120 = 10 rounds x 8 G x 14 primitive 32-bit ops; the kernel issues part of the "
                             "additions on the FMA pipe (IMAD), the XORs and rotations on the ALU pipe"},
        "int_peaks": peaks_int,
        "fft_plans": fft_plans,
        "wide_fib_prove": ({"workload": "Wide-Fibonacci 100 cols x 2^14 rows, blowup 2, 70 queries, pow 10, "
                                         "full prove (trace generated on device); native prover "
                                         "(cs_prove_wide_fib), restated prover beside it",
                            "proofs_per_s": ff(1e3 / statistics.median(wf_native)),
                            "p50_ms": ff(float(np.percentile(wf_native, 50))),
                            "p99_ms": ff(float(np.percentile(wf_native, 99))),
                            "native_plain": {"proofs_per_s": ff(1e3 / statistics.median(wf_plain)),
                                             "p50_ms": ff(float(np.percentile(wf_plain, 50))),
                                             "p99_ms": ff(float(np.percentile(wf_plain, 99)))},
                            "restated": {"proofs_per_s": ff(1e3 / statistics.median(wf_lat)),
                                         "p50_ms": ff(float(np.percentile(wf_lat, 50))),
                                         "p99_ms": ff(float(np.percentile(wf_lat, 99)))},
                            "generic": {"proofs_per_s": ff(1e3 / statistics.median(wf_generic)),
                                        "p50_ms": ff(float(np.percentile(wf_generic, 50))),
                                        "p99_ms": ff(float(np.percentile(wf_generic, 99))),
                                        "note": "air_prover over the NVRTC kernel of wide_fib_air; "
                                                "bytes checked against the restated prover"},
                            "generic_native": {"proofs_per_s": ff(1e3 / statistics.median(wf_generic_native)),
                                               "p50_ms": ff(float(np.percentile(wf_generic_native, 50))),
                                               "p99_ms": ff(float(np.percentile(wf_generic_native, 99))),
                                               "note": "cs_prove_air (air_prover.prove_native) over the same "
                                                       "kernel; bytes checked against the restated prover"}}
                           if wf_lat else None),
        "batched_vs_plain": bvp,
        "serving": serving_res,
        "poseidon_prove": poseidon_res,
        "mixed_prove": mixed_res,
        "gkr": gkr_res,
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
        "cpu_baseline": cpu,
    }
    print(json.dumps(res))
    if dist:
        dist.destroy_process_group()


# ----------------------------------------------------------------- CPU arm

class CpuCommitStage:
    """The commit-stage step on the oracle (the C restatement of the reference's CPU backend, run
    with OpenMP on every host core): the whole workload, no sampling. As the reference's
    interpolate consumes its evaluations, each step interpolates a fresh copy of the trace in
    place; the copy is made before the step's clock starts."""

    def __init__(self, seed: int = 11):
        from oracle import oracle as O
        from proving_gb300.synthetic import m31_columns, qm31_column, seeded_qm31
        self.O = O
        self.evals = m31_columns(seed, N_COLS, LOG_ROWS)
        self.work = np.empty_like(self.evals)
        self.ext = np.empty((N_COLS, 1 << LOG_EXT), np.uint32)
        self.tw, self.itw = O.canonic_twiddles(LOG_EXT + 1)
        self.fri = qm31_column(seed + 2, FRI_LOG)
        self.alphas = [seeded_qm31(k) for k in range(FRI_LOG)]
        vp = ctypes.c_void_p
        self.t_work = (vp * N_COLS)(*[self.work[i].ctypes.data for i in range(N_COLS)])
        self.t_ext = (vp * N_COLS)(*[self.ext[i].ctypes.data for i in range(N_COLS)])
        self.logs_in = np.full(N_COLS, LOG_ROWS, np.uint32)
        self.logs_ext = np.full(N_COLS, LOG_EXT, np.uint32)

    def step(self):
        """One step; returns (seconds per stage, Merkle root)."""
        O, lib, c32 = self.O, self.O.lib(), ctypes.c_uint32
        np.copyto(self.work, self.evals)
        t0 = time.perf_counter()
        lib.orc_interpolate_batch(self.t_work, O._p(self.logs_in), c32(N_COLS), O._p(self.itw),
                                  c32(self.itw.size.bit_length() - 1))
        t1 = time.perf_counter()
        lib.orc_evaluate_batch(self.t_work, O._p(self.logs_in), self.t_ext, O._p(self.logs_ext), c32(N_COLS),
                               O._p(self.tw), c32(self.tw.size.bit_length() - 1))
        t2 = time.perf_counter()
        root = O.merkle_commit(list(self.ext), LOG_EXT)  # leaves + node layers over 2^LOG_EXT leaves
        t3 = time.perf_counter()
        lay = O.fold_circle_into_line(self.fri, self.alphas[0])
        init = O.line_domain_initial_index(FRI_LOG - 1)
        for k in range(1, FRI_LOG):
            lay = O.fold_line(lay, init, self.alphas[k])
            init = O.double_index(init)
        t4 = time.perf_counter()
        return {"interpolate": t1 - t0, "evaluate": t2 - t1, "merkle": t3 - t2, "fri_folds": t4 - t3}, root


def cpu_proof_times(mixed: bool = True, poseidon_log_rows: int = 18):
    """Whole proofs on the oracle's own prover (oracle/oracle_prover.c, every host core):
    Wide-Fibonacci 100 x 2^14, Poseidon2 at 2^poseidon_log_rows rows and, when asked, the 600 +
    120-column mixed trace. The same proof bytes as the GPU provers (checked in
    tests/test_gpu_proof_parity_full.py). Returns proofs/s and latencies per workload."""
    from oracle import oracle as O
    from proving_gb300.synthetic import m31_column, mixed_trace_shape
    fri = (10, 1, 0, 70, 1)
    out = {}
    lat = []
    for k in range(6):
        tr = [O.wide_fib_trace(m31_column(100 + k, 14), m31_column(200 + k, 14), 100)]
        t0 = time.perf_counter()
        O.prove_fib_and_lookups(fri, tr, [14])
        if k:
            lat.append(time.perf_counter() - t0)
    out["wide_fib_100x2^14"] = {"proofs_per_s": round(1 / statistics.median(lat), 3),
                                "p50_ms": round(1e3 * statistics.median(lat), 2), "proofs": len(lat)}
    t0 = time.perf_counter()
    O.prove_poseidon(fri, poseidon_log_rows)
    dt = time.perf_counter() - t0
    out[f"poseidon_2^{poseidon_log_rows}_rows"] = {"proofs_per_s": round(1 / dt, 4), "ms": round(1e3 * dt, 1),
                                                   "proofs": 1}
    if mixed:
        comps, lookup_logs = mixed_trace_shape()
        traces = [O.wide_fib_trace(m31_column(300 + i, l), m31_column(400 + i, l), n) for i, (n, l) in enumerate(comps)]
        values = [m31_column(500 + k, l) for k, l in enumerate(lookup_logs)]
        t0 = time.perf_counter()
        O.prove_fib_and_lookups(fri, traces, [l for _, l in comps], values, lookup_logs)
        dt = time.perf_counter() - t0
        out["mixed_600+120_cols"] = {"proofs_per_s": round(1 / dt, 4), "ms": round(1e3 * dt, 1), "proofs": 1}
    return out


def cpu_baseline(args):
    """The reported CPU baseline of the GPU arm: two whole commit-stage steps of the oracle after one
    warm-up step (about 10 s on 16 cores), and the oracle prover's whole proofs."""
    from oracle import oracle as O
    st = CpuCommitStage()
    st.step()
    times = [st.step()[0] for _ in range(2)]
    total = statistics.mean(sum(t.values()) for t in times)
    stages = {k: statistics.mean(t[k] for t in times) for k in times[0]}
    res = {"value": float(f"{1.0 / total:.6g}"), "unit": UNIT, "cores": O.num_threads(), "kind": "port",
           "sample": f"2 whole steps ({N_COLS} x 2^{LOG_ROWS} interpolate, evaluate on 2^{LOG_EXT}, the full "
                     f"height-{LOG_EXT} tree, {FRI_LOG} folds) after 1 warm-up step; nothing extrapolated",
           "stages_s": {k: float(f"{v:.4g}") for k, v in stages.items()}}
    if not args.skip_cpu_proofs:
        res["proofs"] = cpu_proof_times(mixed=not args.skip_cpu_mixed_proof, poseidon_log_rows=args.poseidon_log_rows)
        res["proofs_unit"] = PROOF_UNIT
    return res


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle")], check=True)
    from oracle import oracle as O
    O.set_num_threads(os.cpu_count() or 1)  # this rank alone times the CPU arm: every host core
    st = CpuCommitStage()
    for _ in range(args.warmup):
        st.step()
    totals = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        stages, _ = st.step()
        totals.append(sum(stages.values()))
    wall = time.perf_counter() - t0
    value = args.steps / sum(totals)
    sample = (f"every step whole: {N_COLS} x 2^{LOG_ROWS} interpolate, evaluate on 2^{LOG_EXT}, the full height-"
              f"{LOG_EXT} tree, {FRI_LOG} folds; the oracle (C restatement of the reference CPU backend, OpenMP); "
              "the Rust reference cannot be built: no cargo on either machine")
    res = {
        "metric": METRIC, "value": float(f"{value:.6g}"), "unit": UNIT, "n_gpus": 0, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": float(f"{1e3 * sum(totals) / args.steps:.6g}"),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32 (M31 field words)",
        "data": "synthetic (seeded)", "impl": "reference",
        "config": {"workload": workload_name(), "n_cols": N_COLS, "log_rows": LOG_ROWS, "log_blowup": LOG_BLOWUP},
        "cpu_baseline": {"value": float(f"{value:.6g}"), "unit": UNIT, "cores": O.num_threads(), "kind": "port",
                         "sample": sample},
        "e2e": {"value": float(f"{value:.6g}"), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "wall_s": float(f"{wall:.4g}"),
    }
    print(json.dumps(res))


def case_mixed_kernels(torch):
    """Small cases of the mixed-size proof's kernels, for ncu (about 3 GB on the device): barycentric
    weights and partial sums (64 columns x 2^22), quotient numerators (64 x 2^22, one point), LogUp
    quotients (16 components x 2^22), LogUp running sums (8 x 2^22 and 8 x 2^16) and a lifted Merkle
    commit of 64 x 2^22, 64 x 2^18 and 64 x 2^14 columns (leaf launches at three sizes). Every kernel
    runs twice, the first run warming up."""
    from proving_gb300.backend import BaseColumn, CudaBackend as B, SecureColumnByCoords
    g = torch.Generator(device="cuda")
    g.manual_seed(1)
    P = (1 << 31) - 1

    def col(l):
        return BaseColumn(torch.randint(0, P, (1 << l,), generator=g, device="cuda", dtype=torch.int64)
                          .to(torch.int32))
    L = 22
    cols = [col(L) for _ in range(64)]
    pt = ((1, 2, 3, 4), (5, 6, 7, 8))
    for _ in range(2):
        B.barycentric_eval_at_point(cols, B.barycentric_weights(L, pt))
    coeffs = np.random.default_rng(0).integers(0, P, (64, 3, 4)).astype(np.uint32)
    for _ in range(2):
        B.accumulate_numerators(cols, coeffs, 1)
    vals = [col(L) for _ in range(16)]
    inters = [SecureColumnByCoords([col(L) for _ in range(4)]) for _ in range(16)]
    acc = SecureColumnByCoords.zeros(1 << L)
    rcs = [(k + 1, 2, 3, 4) for k in range(16)]
    claimed = [(5, k + 6, 7, 8) for k in range(16)]
    for _ in range(2):
        B.logup_compositions(vals, inters, L - 1, (9, 10, 11, 12), claimed, rcs, acc)
    del inters, acc
    values = vals[:8] + [col(16) for _ in range(8)]
    for _ in range(2):
        B.logup_running_sums(values, (9, 10, 11, 12))
    del values, vals
    mixed = cols + [col(18) for _ in range(64)] + [col(14) for _ in range(64)]
    for _ in range(2):
        B.merkle_commit(mixed, L)
    torch.cuda.synchronize()
    return {"case": "mixed-kernels", "ok": True}


def gkr_leg(torch, log_logup: int = 22, log_gp: int = 20, n_proofs: int = 3, kernel_log: int = 24):
    """GKR lookups (GkrOps / MleOps, crates/stwo/src/prover/lookups/): a batch proof of a generic
    LogUp instance of 2^log_logup fractions and a grand product of 2^log_gp values (seeded inputs on
    the device), and the streaming kernels alone at 2^kernel_log values (larger than L2) against
    HBM. Algorithmic bytes: next_layer reads 2 x 16 B and writes 2 x 16 B per output pair
    (numerators and denominators); fix_first_variable reads 2 x 16 B and writes 16 B per output;
    the sum-check sums read 4 x 16 B per term from each of the two columns plus 16 B of eq."""
    from proving_gb300 import gkr as G
    from proving_gb300 import prover as pr
    from proving_gb300.serving import collector_paused
    P = (1 << 31) - 1
    dev = G.DeviceGkrOps()
    gen = torch.Generator(device="cuda").manual_seed(11)
    rnd = lambda n: torch.randint(0, P, (4, n), dtype=torch.int32, device="cuda", generator=gen)
    layers = [G.Layer(G.LOGUP_GENERIC, [G.Mle(rnd(1 << log_logup), log_logup), G.Mle(rnd(1 << log_logup), log_logup)]),
              G.Layer(G.GRAND_PRODUCT, [G.Mle(rnd(1 << log_gp), log_gp)])]
    lat, lat_native = [], []
    with collector_paused():
        for i in range(n_proofs + 1):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            proof, _ = G.prove_batch(dev, pr.Blake2sChannel(), layers)
            torch.cuda.synchronize()
            if i:
                lat.append((time.perf_counter() - t0) * 1e3)
        for i in range(n_proofs + 1):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            native, _ = G.prove_batch_native(pr.Blake2sChannel(), layers)
            torch.cuda.synchronize()
            if i:
                lat_native.append((time.perf_counter() - t0) * 1e3)
    same = (native.sumcheck_proofs == proof.sumcheck_proofs
            and native.output_claims_by_instance == proof.output_claims_by_instance)
    n = 1 << kernel_log
    num, den = G.Mle(rnd(n), kernel_log), G.Mle(rnd(n), kernel_log)
    lay = G.Layer(G.LOGUP_GENERIC, [num, den])
    eqm = G.Mle(rnd(n // 4), kernel_log - 2)
    lam = (1, 2, 3, 4)
    hbm, _ = peaks()

    def timed(fn, reps=10):
        fn()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        for _ in range(reps):
            fn()
        e.record()
        torch.cuda.synchronize()
        return s.elapsed_time(e) / reps

    kernels = {}
    for name, fn, nbytes in (("next_layer", lambda: dev.next_layer(lay), 32 * n + 16 * n),
                             ("fix_first_variable", lambda: dev.fix_first_variable(den, lam), 16 * n + 8 * n),
                             ("sum_as_poly", lambda: dev.sum_as_poly_evals([(lay, eqm, lam)]), 32 * n + 4 * n),
                             ("gen_eq_evals", lambda: dev.gen_eq_evals([(i, 1, 2, 3) for i in range(kernel_log)], lam),
                              16 * n)):
        ms = timed(fn)
        gbs = nbytes / (ms / 1e3) / 1e9
        kernels[name] = {"ms": round(ms, 4), "gb_per_s": round(gbs, 1), "frac_of_hbm": round(gbs / hbm, 3)}
    return {"workload": f"GKR batch proof: generic LogUp 2^{log_logup} + grand product 2^{log_gp} (secure values); "
                        f"kernels alone at 2^{kernel_log} values",
            "layers": log_logup, "sumcheck_rounds": log_logup * (log_logup - 1) // 2,
            "native_prove_p50_ms": round(float(np.percentile(lat_native, 50)), 3),
            "prove_p50_ms": round(float(np.percentile(lat, 50)), 3), "prove_max_ms": round(max(lat), 3),
            "native_equals_driver": bool(same),
            "kernels": kernels,
            "note": "prove_p50_ms: the protocol in Python over the device ops (proving_gb300.gkr.prove_batch); "
                    "native_prove_p50_ms: the protocol in C++ (cs_gkr_prove_batch), one read-back per round"}


def run_case(args):
    import torch
    from proving_gb300 import build as cuda_build
    cuda_build.build()
    if args.case == "mixed-kernels":
        res = case_mixed_kernels(torch)
    elif args.case == "mixed-prove-native":  # one native proof after one warm-up proof
        res = mixed_prove_leg(torch, n_proofs=1, arms=("native",))
    elif args.case == "poseidon-native":  # one native Poseidon2 proof after one warm-up proof
        from proving_gb300 import poseidon as ps
        from proving_gb300 import prover as pr
        from proving_gb300.backend import CudaBackend
        log_n = args.poseidon_log_rows
        tw = pr.GpuOps().twiddles(log_n + ps.LOG_EXPAND + 1)
        lat = []
        for _ in range(2):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            CudaBackend.prove_poseidon_native(log_n, (10, 1, 0, 70), tw)
            torch.cuda.synchronize()
            lat.append((time.perf_counter() - t0) * 1e3)
        res = {"workload": f"native Poseidon2 proof, 2^{log_n} rows", "ms": [round(x, 3) for x in lat]}
    elif args.case == "poseidon-generic-native":
        # twice: a Poseidon2 proof through the native generic prover (the AIR recorded by the
        # constraint evaluator, its kernels compiled first), then one through cs_prove_poseidon
        from proving_gb300 import air_prover as ap
        from proving_gb300 import framework as fw
        from proving_gb300 import poseidon as ps
        from proving_gb300 import prover as pr
        from proving_gb300.backend import CudaBackend
        log_n = args.poseidon_log_rows
        ops = pr.GpuOps()
        fp = pr.FriParams(pow_bits=10, log_blowup_factor=1, log_last_layer_degree_bound=0, n_queries=70, fold_step=1)
        cfg = ps.poseidon_pcs_config(log_n + 3, fp)
        tw = ops.twiddles(log_n + ps.LOG_EXPAND + 1)
        air = fw.poseidon_air_recorded()
        fw.CompiledAir.get(air)
        comp = ap.FrameworkComponent(ap.TraceLocationAllocator(), air, log_n, constraint_log_degree=ps.LOG_EXPAND)
        same = []
        for _ in range(2):
            words = ap.prove_native([comp], CudaBackend.poseidon_trace(log_n), cfg, tw)
            same.append(words == CudaBackend.prove_poseidon_native(log_n, (10, 1, 0, 70), tw))
        res = {"workload": f"Poseidon2 at 2^{log_n} rows, generic native then hand-written native", "same": same}
    elif args.case == "wide-fib-native":  # two native 100 x 2^14 Wide-Fibonacci proofs after two warm-up proofs
        lat = wide_fib_prove_native(torch, n_proofs=2)
        res = {"workload": "native Wide-Fibonacci proof, 100 x 2^14", "ms": [round(x, 3) for x in lat]}
    elif args.case == "gkr":
        res = gkr_leg(torch, log_logup=args.gkr_log, log_gp=max(args.gkr_log - 2, 2), n_proofs=1,
                      kernel_log=args.gkr_log)
    else:  # one mixed-size proof after one warm-up proof, batched arm only
        res = mixed_prove_leg(torch, n_proofs=1, arms=("batched",))
    print(json.dumps(res))


def launch_replicas(n: int) -> int:
    """Starts this command as n ranks on this node (torch.distributed.run, rendezvous on 127.0.0.1 at a
    free port) and returns the launcher's exit status."""
    import socket
    with socket.socket() as so:
        so.bind(("127.0.0.1", 0))
        port = so.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={n}",
           "--master-addr=127.0.0.1", f"--master-port={port}", str(Path(__file__).resolve()), *sys.argv[1:]]
    return subprocess.call(cmd)


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--no-cpu-baseline", action="store_true", help="skip the timed oracle steps and proofs")
    ap.add_argument("--skip-cpu-proofs", action="store_true", help="skip the oracle's whole proofs in cpu_baseline")
    ap.add_argument("--skip-cpu-mixed-proof", action="store_true",
                    help="skip the oracle's mixed-size proof (about a minute) in cpu_baseline")
    ap.add_argument("--n-cols", type=int, default=N_COLS, help="trace columns (smaller cases for profiling)")
    ap.add_argument("--log-rows", type=int, default=LOG_ROWS, help="log2 rows per trace column")
    ap.add_argument("--skip-e2e", action="store_true", help="skip the host-buffer end-to-end leg")
    ap.add_argument("--skip-prove", action="store_true", help="skip the Wide-Fibonacci full-prove latency leg")
    ap.add_argument("--skip-plain", action="store_true", help="skip the batched-vs-plain comparison legs")
    ap.add_argument("--skip-serving", action="store_true", help="skip the proof-service leg")
    ap.add_argument("--skip-poseidon", action="store_true", help="skip the Poseidon2 prove leg")
    ap.add_argument("--poseidon-log-rows", type=int, default=18, help="log2 rows of the Poseidon2 prove leg")
    ap.add_argument("--skip-mixed-prove", action="store_true", help="skip the mixed-size full-proof leg")
    ap.add_argument("--skip-gkr", action="store_true", help="skip the GKR lookup leg")
    ap.add_argument("--skip-autotune", action="store_true",
                    help="keep the default FFT pass plans (no candidate sweep before timing; for profiling)")
    ap.add_argument("--gkr-log", type=int, default=22, help="log2 values of the --case gkr instance")
    ap.add_argument("--case", choices=["mixed-kernels", "mixed-prove", "mixed-prove-native", "poseidon-native",
                                       "poseidon-generic-native", "wide-fib-native", "gkr"],
                    help="run one small profiling case instead of the benchmark (for ncu)")
    args = ap.parse_args()
    set_shape(args.n_cols, args.log_rows)
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ and not args.case:
        # one process per GPU: re-run this command under torch.distributed.run (replicas, weak scaling)
        sys.exit(launch_replicas(args.gpus))
    if args.case:
        run_case(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
