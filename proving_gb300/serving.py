"""A continuous-batching proof service on one GPU.

Requests (Wide-Fibonacci proofs of different sizes) arrive over time. Each is
admitted as soon as a worker slot is free and its device-memory estimate fits
in the HBM budget left by the proofs in flight; admitted proofs run
concurrently, each on its own CUDA stream, so the device work of several
proofs and their host orchestration overlap. Traces are generated on the
device from the request's seeds, the twiddle tree for the largest size stays
resident and serves every smaller canonic domain. The service reports
proofs/s and per-request latency (arrival to proof) percentiles.
"""
from __future__ import annotations

import queue
import threading
import time
from dataclasses import dataclass, field

import numpy as np

from . import prover as pr
from .synthetic import m31_column

N_COLS = 100


@dataclass
class ProofRequest:
    request_id: int
    log_n_rows: int
    seed: int
    arrival: float = 0.0
    admitted: float = 0.0
    done: float = 0.0
    proof: object = None
    error: str | None = None

    @property
    def latency_ms(self) -> float:
        return (self.done - self.arrival) * 1e3


def hbm_estimate(log_n_rows: int, n_cols: int = N_COLS) -> int:
    """Device bytes a Wide-Fibonacci proof holds at its peak: the trace and its
    blown-up evaluation, the composition columns, the Merkle layers, the
    quotient and FRI columns and barycentric weights."""
    n, ext = 1 << log_n_rows, 1 << (log_n_rows + 1)
    trace = 4 * n_cols * (n + ext)
    comp = 4 * 8 * (n + ext) + 16 * ext
    merkle = 2 * 2 * 32 * ext
    fri = 4 * 16 * ext
    return trace + comp + merkle + fri + 16 * ext


def default_config(log_n_rows: int) -> pr.PcsConfig:
    fp = pr.FriParams(pow_bits=10, log_blowup_factor=1, log_last_layer_degree_bound=0, n_queries=70, fold_step=1)
    return pr.PcsConfig(fp, trace_lifting_log_size=log_n_rows + 1)


class ProverService:
    def __init__(self, n_workers: int = 4, hbm_budget: int = 64 << 30, max_log_n_rows: int = 20,
                 plain: bool = False):
        import torch
        from .backend import BaseColumn, CudaBackend
        self.torch = torch
        self.BaseColumn, self.B = BaseColumn, CudaBackend
        # plain: one launch per column per stage; otherwise the batched stage launches
        self.ops = pr.PlainGpuOps() if plain else pr.GpuOps()
        self.twiddles = self.ops.twiddles(max_log_n_rows + 2)
        torch.cuda.synchronize()
        self.n_workers = n_workers
        self.budget = hbm_budget
        self.in_flight = 0
        self.cv = threading.Condition()
        self.pending: queue.Queue = queue.Queue()
        self.finished: list[ProofRequest] = []
        self.threads = []
        self.stop = False

    # ---------------------------------------------------------------- workers
    def _prove(self, req: ProofRequest, stream):
        torch = self.torch
        with torch.cuda.stream(stream):
            a = self.BaseColumn.from_cpu(m31_column(req.seed, req.log_n_rows))
            b = self.BaseColumn.from_cpu(m31_column(req.seed + 1, req.log_n_rows))
            trace = self.B.wide_fib_trace(a, b, N_COLS)
            proof = pr.prove_wide_fib(self.ops, trace, req.log_n_rows, default_config(req.log_n_rows),
                                      pr.Blake2sChannel(), self.twiddles)
            stream.synchronize()
        return proof

    def _worker(self):
        stream = self.torch.cuda.Stream()
        while True:
            req = self.pending.get()
            if req is None:
                return
            need = hbm_estimate(req.log_n_rows)
            with self.cv:
                # admission: wait until the proof fits in the HBM budget left in flight
                while self.in_flight + need > self.budget and self.in_flight > 0:
                    self.cv.wait()
                self.in_flight += need
            req.admitted = time.perf_counter()
            try:
                req.proof = self._prove(req, stream)
            except Exception as e:  # one failed request does not stop the service
                req.error = repr(e)
            req.done = time.perf_counter()
            with self.cv:
                self.in_flight -= need
                self.finished.append(req)
                self.cv.notify_all()

    def start(self):
        for _ in range(self.n_workers):
            t = threading.Thread(target=self._worker, daemon=True)
            t.start()
            self.threads.append(t)

    def submit(self, req: ProofRequest):
        req.arrival = time.perf_counter()
        self.pending.put(req)

    def close(self):
        for _ in self.threads:
            self.pending.put(None)
        for t in self.threads:
            t.join()


def poisson_requests(n: int, rate_per_s: float, log_min: int, log_max: int, seed: int):
    """Seeded request stream: exponential inter-arrival gaps, sizes uniform in [log_min, log_max]."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate_per_s, n)
    sizes = rng.integers(log_min, log_max + 1, n)
    return [(float(g), ProofRequest(i, int(s), seed * 100003 + 2 * i)) for i, (g, s) in enumerate(zip(gaps, sizes))]


def run_stream(n_workers: int, requests, hbm_budget: int = 64 << 30, max_log: int = 20, plain: bool = False):
    """Serves a request stream; returns (finished requests, wall seconds)."""
    svc = ProverService(n_workers=n_workers, hbm_budget=hbm_budget, max_log_n_rows=max_log, plain=plain)
    svc.start()
    t0 = time.perf_counter()
    for gap, req in requests:
        time.sleep(gap)
        svc.submit(req)
    svc.close()
    wall = time.perf_counter() - t0
    return svc.finished, wall


def summarize(finished, wall: float) -> dict:
    lat = [r.latency_ms for r in finished if r.error is None]
    return {"proofs": len(lat), "errors": sum(r.error is not None for r in finished),
            "proofs_per_s": round(len(lat) / wall, 3),
            "p50_ms": round(float(np.percentile(lat, 50)), 3) if lat else None,
            "p99_ms": round(float(np.percentile(lat, 99)), 3) if lat else None}
