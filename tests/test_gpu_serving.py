"""The proof service: requests of different sizes proved concurrently on
separate streams give the same proof bytes as each request proved alone, and
admission keeps the in-flight HBM estimate within the budget."""
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from proving_gb300 import serving  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def built():
    from proving_gb300 import build
    build.build()


def test_results_alone_equal_results_in_the_mix():
    # worker threads prove with the native provers, concurrently on their own streams; each proof
    # equals the restated prover's through the plain one-launch-per-column path, proved alone
    spec = [(8, "wide_fib"), (11, "wide_fib"), (5, "poseidon"), (9, "wide_fib"), (12, "wide_fib"),
            (6, "poseidon"), (8, "wide_fib"), (10, "wide_fib")]
    reqs = [serving.ProofRequest(i, s, 1000 + 7 * i, k) for i, (s, k) in enumerate(spec)]
    mixed, _ = serving.run_stream(4, [(0.0, r) for r in reqs], max_log=12)
    assert all(r.error is None for r in mixed), [r.error for r in mixed]
    alone_reqs = [serving.ProofRequest(i, s, 1000 + 7 * i, k) for i, (s, k) in enumerate(spec)]
    alone, _ = serving.run_stream(1, [(0.0, r) for r in alone_reqs], max_log=12, plain=True)
    by_id = {r.request_id: r.proof_bytes() for r in alone}
    for r in mixed:
        assert r.proof_bytes() == by_id[r.request_id]


def test_admission_respects_the_budget():
    # a budget that fits one size-12 proof at a time still finishes every request
    budget = serving.hbm_estimate(12) + serving.hbm_estimate(8) // 2
    reqs = [serving.ProofRequest(i, 12, 50 + i) for i in range(3)]
    done, _ = serving.run_stream(3, [(0.0, r) for r in reqs], hbm_budget=budget, max_log=12)
    assert len(done) == 3 and all(r.error is None for r in done)
    # admitted one after another: each admission is after the previous completion
    done.sort(key=lambda r: r.admitted)
    for prev, nxt in zip(done, done[1:]):
        assert nxt.admitted >= prev.done - 1e-3


def test_worker_processes_give_the_same_proofs():
    # the process service (own CUDA context per worker) returns the bytes the in-process prover
    # gives alone, for both AIRs
    reqs = [serving.ProofRequest(0, 8, 11), serving.ProofRequest(1, 5, 12, "poseidon"),
            serving.ProofRequest(2, 9, 13), serving.ProofRequest(3, 4, 14, "poseidon")]
    svc = serving.ProcessProverService(n_workers=2, max_log_n_rows=10, warm_logs=(("wide_fib", 6),))
    try:
        done, _ = svc.run([(0.0, r) for r in reqs])
    finally:
        svc.close()
    assert all(r.error is None for r in done), [r.error for r in done]
    alone = [serving.ProofRequest(r.request_id, r.log_n_rows, r.seed, r.kind) for r in reqs]
    alone_done, _ = serving.run_stream(1, [(0.0, r) for r in alone], max_log=10)
    want = {r.request_id: r.proof_bytes() for r in alone_done}
    for r in done:
        assert r.proof_bytes() == want[r.request_id]


def test_native_plain_and_served_forms_agree():
    # the native provers' plain form (one launch per column per stage), one request at a time, gives
    # the bytes of the served form (worker threads, batched stages)
    spec = [(9, "wide_fib"), (5, "poseidon"), (12, "wide_fib"), (4, "poseidon")]
    reqs = [serving.ProofRequest(i, s, 2000 + 5 * i, k) for i, (s, k) in enumerate(spec)]
    served, _ = serving.run_stream(3, [(0.0, r) for r in reqs], max_log=12, native=True)
    plain_reqs = [serving.ProofRequest(i, s, 2000 + 5 * i, k) for i, (s, k) in enumerate(spec)]
    plain, _ = serving.run_stream(1, [(0.0, r) for r in plain_reqs], max_log=12, native=True, plain=True)
    assert all(r.error is None for r in served + plain), [r.error for r in served + plain]
    by_id = {r.request_id: r.proof_bytes() for r in plain}
    assert all(r.proof_bytes() == by_id[r.request_id] for r in served)
