"""A continuous-batching proof service on one GPU.

Requests (Wide-Fibonacci or Poseidon2 proofs of different sizes) arrive over
time. Each is admitted as soon as a worker is free and its device-memory
estimate fits in the HBM budget left by the proofs in flight. Admitted proofs
run concurrently, so the device work of one proof overlaps the host
orchestration and device work of the others. Traces are generated on the
device from the request's seeds, and the twiddle tree for the largest size
stays resident and serves every smaller canonic domain. The service reports
proofs/s and per-request latency (arrival to proof) percentiles.

Two forms:
- `ProverService` runs its workers as threads of this process, each on its own
  CUDA stream. With the native provers (cs_prove_wide_fib, cs_prove_poseidon)
  a worker leaves the interpreter for the whole proof, so the workers' host
  code runs on separate cores and their kernels overlap in the one CUDA
  context. This is the faster form.
- `ProcessProverService` runs each worker as a spawned process with its own CUDA
  context and stream; the contexts time-slice the device instead of sharing it.

`plain=True` gives the plain form: one launch per column for every per-column
stage. With the native provers that is their CS_PROVE_PLAIN mode; with
`native=False` it is prover.PlainGpuOps under the restated (Python) prover.
Otherwise the workers prove requests with the native provers' batched stages.
Every form gives the same proof bytes for a request.
"""
from __future__ import annotations

import contextlib
import gc
import queue
import threading
import time
from collections import deque
from dataclasses import dataclass

import numpy as np

from . import prover as pr
from .synthetic import m31_column

N_COLS = 100  # Wide-Fibonacci columns (the 100 x 2^14 proof's width)


@dataclass
class ProofRequest:
    request_id: int
    log_n_rows: int
    seed: int
    kind: str = "wide_fib"  # or "poseidon"
    arrival: float = 0.0
    admitted: float = 0.0
    done: float = 0.0
    proof: object = None  # the proof (threads) or its bytes (processes)
    error: str | None = None

    @property
    def latency_ms(self) -> float:
        return (self.done - self.arrival) * 1e3

    def proof_bytes(self) -> bytes:
        return self.proof if isinstance(self.proof, bytes) else self.proof.to_bytes()


def hbm_estimate(log_n_rows: int, n_cols: int = N_COLS, kind: str = "wide_fib") -> int:
    """Device bytes a proof holds at its peak.
    Wide-Fibonacci: the trace and its blown-up evaluation, the composition columns, the Merkle
    layers, the quotient and FRI columns and barycentric weights. Poseidon2: the trace, its
    coefficients, blown-up evaluation and evaluation on the 4x domain, the same for the 32
    interaction columns, and the Merkle layers."""
    n, ext = 1 << log_n_rows, 1 << (log_n_rows + 1)
    if kind == "poseidon":
        cols = 1264 + 32
        return 4 * cols * (2 * n + ext + 4 * n) + 2 * 32 * (2 * ext) + 4 * 16 * (4 * n)
    trace = 4 * n_cols * (n + ext)
    comp = 4 * 8 * (n + ext) + 16 * ext
    merkle = 2 * 2 * 32 * ext
    fri = 4 * 16 * ext
    return trace + comp + merkle + fri + 16 * ext


def fri_params() -> pr.FriParams:
    return pr.FriParams(pow_bits=10, log_blowup_factor=1, log_last_layer_degree_bound=0, n_queries=70, fold_step=1)


def default_config(log_n_rows: int) -> pr.PcsConfig:
    return pr.PcsConfig(fri_params(), trace_lifting_log_size=log_n_rows + 1)


def twiddle_domain(max_log_n_rows: int) -> int:
    """The canonic domain whose twiddle tree serves both AIRs up to max_log_n_rows
    (Poseidon2 evaluates on log_n_rows + 2 with blowup 1)."""
    return max_log_n_rows + 3


def prove_request(ops, twiddles, req: ProofRequest, native: bool = False, plain: bool = False):
    """One proof on the current CUDA stream: the trace generated on the device from the request's
    seed, then the restated prover, or with native=True the native prover (cs_prove_wide_fib /
    cs_prove_poseidon, the same bytes; returned as bytes; plain=True: one launch per column per
    stage)."""
    from .backend import BaseColumn, CudaBackend
    if req.kind == "poseidon":
        from . import poseidon as ps
        if native:
            fp = fri_params()
            return CudaBackend.prove_poseidon_native(
                req.log_n_rows, (fp.pow_bits, fp.log_blowup_factor, fp.log_last_layer_degree_bound, fp.n_queries),
                twiddles, plain=plain)
        cfg = ps.poseidon_pcs_config(req.log_n_rows + 3, fri_params())
        # the reference's own sanity check fails for this AIR (lifted protocol): check=False
        return ps.prove_poseidon(ops, req.log_n_rows, cfg, pr.Blake2sChannel(), twiddles, check=False)
    a = BaseColumn.from_cpu(m31_column(req.seed, req.log_n_rows))
    b = BaseColumn.from_cpu(m31_column(req.seed + 1, req.log_n_rows))
    trace = CudaBackend.wide_fib_trace(a, b, N_COLS)
    if native:
        fp = fri_params()
        return CudaBackend.prove_wide_fib_native(
            [trace], [req.log_n_rows], (fp.pow_bits, fp.log_blowup_factor, fp.log_last_layer_degree_bound,
                                        fp.n_queries), twiddles, plain=plain)
    return pr.prove_wide_fib(ops, trace, req.log_n_rows, default_config(req.log_n_rows), pr.Blake2sChannel(),
                             twiddles)


@contextlib.contextmanager
def collector_paused():
    """Automatic garbage collection off while proofs run: a proof's objects are freed by reference
    counting, and a full collection in the middle of a proof (tens of ms with the prover's working
    set) would land in that proof's latency. A collection also leaves the next proof a few ms slower
    (its allocations start cold), so workers collect only when idle."""
    was = gc.isenabled()
    gc.disable()
    try:
        yield
    finally:
        if was:
            gc.enable()


def _ops(plain: bool):
    return pr.PlainGpuOps() if plain else pr.GpuOps()


# ------------------------------------------------------------ threads

class ProverService:
    def __init__(self, n_workers: int = 4, hbm_budget: int = 64 << 30, max_log_n_rows: int = 20,
                 plain: bool = False, native: bool | None = None):
        import torch
        self.torch = torch
        # the native provers release the interpreter for the whole proof, so worker threads prove
        # concurrently, each on its own stream of the one CUDA context
        self.native = (not plain) if native is None else native
        self.plain = plain
        self.ops = _ops(plain and not self.native)
        # the worker threads share one CUDA context: a graph capture in one of them would stop the
        # others' work, so the FRI layer loop runs eagerly here (worker processes replay graphs)
        self.ops.fri_graphs = False
        self.twiddles = self.ops.twiddles(twiddle_domain(max_log_n_rows))
        torch.cuda.synchronize()
        self.n_workers = n_workers
        self.budget = hbm_budget
        self.in_flight = 0
        self.cv = threading.Condition()
        self.pending: queue.Queue = queue.Queue()
        self.finished: list[ProofRequest] = []
        self.threads = []

    def _prove(self, req: ProofRequest, stream):
        with self.torch.cuda.stream(stream):
            proof = prove_request(self.ops, self.twiddles, req, native=self.native, plain=self.plain)
            stream.synchronize()
        return proof

    def _worker(self):
        stream = self.torch.cuda.Stream()
        while True:
            req = self.pending.get()
            if req is None:
                return
            need = hbm_estimate(req.log_n_rows, kind=req.kind)
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


def run_stream(n_workers: int, requests, hbm_budget: int = 64 << 30, max_log: int = 20, plain: bool = False,
               native: bool | None = None):
    """Serves a request stream with worker threads; returns (finished requests, wall seconds)."""
    svc = ProverService(n_workers=n_workers, hbm_budget=hbm_budget, max_log_n_rows=max_log, plain=plain,
                        native=native)
    svc.start()
    t0 = time.perf_counter()
    for gap, req in requests:
        time.sleep(gap)
        svc.submit(req)
    svc.close()
    wall = time.perf_counter() - t0
    return svc.finished, wall


# ------------------------------------------------------------ processes

def _process_worker(worker_id: int, plain: bool, max_log: int, warm_logs, tasks, results):
    """A worker process: its own CUDA context and stream; proves the requests it is sent and returns
    the proof bytes with its start and end times (time.perf_counter is the same monotonic clock in
    every process)."""
    import torch
    torch.cuda.set_device(0)
    ops = _ops(plain)
    twiddles = ops.twiddles(twiddle_domain(max_log))
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        for kind, log_n in warm_logs:
            prove_request(ops, twiddles, ProofRequest(-1, log_n, 1, kind), native=not plain)
        stream.synchronize()
    results.put(("ready", worker_id))
    gc.collect()
    gc.disable()  # collections run between requests (collector_paused)
    while True:
        try:
            msg = tasks.get(timeout=0.05)
        except queue.Empty:
            gc.collect()  # idle: collect off the latency path
            msg = tasks.get()
        if msg is None:
            break
        rid, kind, log_n, seed = msg
        t0 = time.perf_counter()
        out, err = None, None
        try:
            with torch.cuda.stream(stream):
                out = prove_request(ops, twiddles, ProofRequest(rid, log_n, seed, kind), native=not plain)
                out = out if isinstance(out, bytes) else out.to_bytes()
                stream.synchronize()
        except Exception as e:  # one failed request does not stop the worker
            err = repr(e)
        results.put(("done", worker_id, rid, out, t0, time.perf_counter(), err))
        if hbm_estimate(log_n, kind=kind) > (8 << 30):
            # return the blocks of a large proof to the device, so idle workers do not hold them
            torch.cuda.empty_cache()


class ProcessProverService:
    """Worker processes on one GPU with arrival-order admission under an HBM budget."""

    def __init__(self, n_workers: int = 4, hbm_budget: int = 160 << 30, max_log_n_rows: int = 20,
                 plain: bool = False, warm_logs=(("wide_fib", 10), ("poseidon", 5))):
        import multiprocessing as mp
        ctx = mp.get_context("spawn")
        self.n_workers = n_workers
        self.budget = hbm_budget
        self.tasks = [ctx.Queue() for _ in range(n_workers)]
        self.results = ctx.Queue()
        self.procs = [ctx.Process(target=_process_worker,
                                  args=(w, plain, max_log_n_rows, list(warm_logs), self.tasks[w], self.results),
                                  daemon=True) for w in range(n_workers)]
        for p in self.procs:
            p.start()
        ready = 0
        while ready < n_workers:
            if self.results.get(timeout=900)[0] == "ready":
                ready += 1

    def run(self, requests):
        """requests: [(gap seconds, ProofRequest)]. Returns (finished requests, wall seconds)."""
        t0 = time.perf_counter()
        arrivals, t = [], t0
        for gap, req in requests:
            t += gap
            arrivals.append((t, req))
        pending: deque = deque()
        idle = list(range(self.n_workers))
        running = {}  # request id -> (request, hbm estimate)
        in_flight = 0
        finished = []
        i = 0
        while len(finished) < len(arrivals):
            now = time.perf_counter()
            while i < len(arrivals) and arrivals[i][0] <= now:
                req = arrivals[i][1]
                req.arrival = arrivals[i][0]
                pending.append(req)
                i += 1
            # admission in arrival order: a free worker and room in the HBM budget
            while pending and idle:
                need = hbm_estimate(pending[0].log_n_rows, kind=pending[0].kind)
                if in_flight + need > self.budget and in_flight > 0:
                    break
                req = pending.popleft()
                w = idle.pop()
                req.admitted = time.perf_counter()
                running[req.request_id] = (req, need)
                in_flight += need
                self.tasks[w].put((req.request_id, req.kind, req.log_n_rows, req.seed))
            next_arrival = arrivals[i][0] - time.perf_counter() if i < len(arrivals) else 1.0
            try:
                msg = self.results.get(timeout=min(max(next_arrival, 1e-4), 1.0))
            except queue.Empty:
                continue
            _, w, rid, out, _t_start, t_end, err = msg
            req, need = running.pop(rid)
            req.proof, req.error, req.done = out, err, t_end
            in_flight -= need
            idle.append(w)
            finished.append(req)
        return finished, time.perf_counter() - t0

    def close(self):
        for q in self.tasks:
            q.put(None)
        for p in self.procs:
            p.join(timeout=60)


def poisson_requests(n: int, rate_per_s: float, log_min: int, log_max: int, seed: int, poseidon_share: float = 0.0):
    """Seeded request stream: exponential inter-arrival gaps, sizes uniform in [log_min, log_max], a
    share of the requests Poseidon2 proofs."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate_per_s, n)
    sizes = rng.integers(log_min, log_max + 1, n)
    kinds = np.where(rng.random(n) < poseidon_share, "poseidon", "wide_fib")
    return [(float(g), ProofRequest(i, int(s), seed * 100003 + 2 * i, str(k)))
            for i, (g, s, k) in enumerate(zip(gaps, sizes, kinds))]


def summarize(finished, wall: float) -> dict:
    lat = [r.latency_ms for r in finished if r.error is None]
    return {"proofs": len(lat), "errors": sum(r.error is not None for r in finished),
            "proofs_per_s": round(len(lat) / wall, 3),
            "p50_ms": round(float(np.percentile(lat, 50)), 3) if lat else None,
            "p99_ms": round(float(np.percentile(lat, 99)), 3) if lat else None}
