"""GPU parity of the generic constraint path: kernels generated from AIRs written against the
framework's evaluator and compiled at run time with NVRTC give the same quotients as the
hand-written kernels and the oracle's CPU constraint evaluator, and the same proofs."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import oracle as O  # noqa: E402
from oracle.air_eval import air_composition  # noqa: E402
from proving_gb300 import framework as fw  # noqa: E402
from proving_gb300.synthetic import m31_column, seeded_qm31  # noqa: E402


@pytest.fixture(scope="module")
def B():
    from proving_gb300 import _lib, build
    build.build()
    from proving_gb300.backend import CudaBackend
    _lib.call("cs_rtc_available")
    return CudaBackend


def _acc(base):
    from proving_gb300.backend import BaseColumn, SecureColumnByCoords
    return SecureColumnByCoords([BaseColumn.from_cpu(c) for c in base])


@pytest.mark.parametrize("n_cols,trace_log,eval_log", [(3, 2, 3), (100, 10, 11), (50, 12, 14)])
def test_wide_fib_generated_equals_hand_written(B, n_cols, trace_log, eval_log):
    from proving_gb300.backend import BaseColumn
    air = fw.compile_air("wide_fib", fw.wide_fib_air, n_cols)
    host = [m31_column(200 + k, eval_log) for k in range(n_cols)]
    cols = [BaseColumn.from_cpu(c) for c in host]
    rc = np.stack([seeded_qm31(300 + k) for k in range(n_cols - 2)])
    base = [m31_column(400 + k, eval_log) for k in range(4)]
    gen, hand = _acc(base), _acc(base)
    fw.CompiledAir.get(air).composition({1: cols}, trace_log, {}, rc, gen)
    B.wide_fib_composition(cols, trace_log, rc, hand)
    g, h = gen.to_cpu(), hand.to_cpu()
    assert all(np.array_equal(a, b) for a, b in zip(g, h))
    if eval_log <= 11:
        want = air_composition(air, {1: host}, eval_log, trace_log, {}, rc, out=base)
        assert all(np.array_equal(a, b) for a, b in zip(g, want))


@pytest.mark.parametrize("trace_log,eval_log", [(1, 2), (5, 6), (12, 13)])
def test_single_lookup_generated_equals_hand_written(B, trace_log, eval_log):
    from proving_gb300.backend import BaseColumn, SecureColumnByCoords
    air = fw.compile_air("lookup", fw.single_lookup_air)
    v = m31_column(7, eval_log)
    inter = [m31_column(8 + k, eval_log) for k in range(4)]
    z, claimed, rc = seeded_qm31(11), seeded_qm31(12), seeded_qm31(13)
    shift = (np.asarray(claimed, np.int64) * pow(1 << trace_log, O.P - 2, O.P) % O.P).astype(np.uint32)
    vcol = BaseColumn.from_cpu(v)
    icols = [BaseColumn.from_cpu(c) for c in inter]
    base = [m31_column(20 + k, eval_log) for k in range(4)]
    gen, hand = _acc(base), _acc(base)
    fw.CompiledAir.get(air).composition({1: [vcol], 2: icols}, trace_log, {"z": z, "shift": shift}, [rc], gen)
    B.logup_compositions([vcol], [SecureColumnByCoords(icols)], trace_log, z, [claimed], [rc], hand)
    assert all(np.array_equal(a, b) for a, b in zip(gen.to_cpu(), hand.to_cpu()))


def test_generic_path_proof_equals_hand_written(B):
    # the mixed Wide-Fibonacci + LogUp proof with every constraint through generated kernels
    from proving_gb300 import prover as pr
    ops = pr.GpuOps()
    traces, lookups = [], []
    for n_cols, log_n in ((4, 9), (5, 3)):
        a, b = np.ones(1 << log_n, np.uint32), np.arange(1 << log_n, dtype=np.uint32)
        traces.append(O.wide_fib_trace(a, b, n_cols))
    rng = np.random.default_rng(7)
    vals = [rng.integers(0, O.P, 1 << n, dtype=np.uint32) for n in (8, 4)]
    fp = pr.FriParams(pow_bits=10, log_blowup_factor=1, log_last_layer_degree_bound=0, n_queries=3, fold_step=1)
    cfg = pr.PcsConfig(fp, trace_lifting_log_size=10)

    def prove(o, generic):
        return pr.prove_fib_and_lookups(o, [o.columns_from_host(t) for t in traces], [9, 3],
                                        [o.columns_from_host([v])[0] for v in vals], [8, 4], cfg,
                                        pr.Blake2sChannel(), o.twiddles(10), generic=generic)
    g = prove(ops, True)
    want, _ = O.prove_fib_and_lookups((10, 1, 0, 3, 1), traces, [9, 3], vals, [8, 4])
    assert g.to_bytes() == prove(ops, False).to_bytes() == want


@pytest.mark.parametrize("trace_log,eval_log", [(4, 6), (8, 10)])
def test_poseidon_generated_equals_hand_written(B, trace_log, eval_log):
    # eval_poseidon_constraints written against the evaluator (relation entries finalized in pairs),
    # compiled with NVRTC: the words of the hand-written Poseidon2 composition kernel
    from proving_gb300.backend import BaseColumn
    from proving_gb300.synthetic import m31_columns
    trace = [BaseColumn.from_cpu(c) for c in m31_columns(500 + eval_log, O.POSEIDON_COLS, eval_log)]
    inter = [BaseColumn.from_cpu(c) for c in m31_columns(600 + eval_log, O.POSEIDON_INTERACTION_COLS, eval_log)]
    lookup = list(seeded_qm31(41)) + list(seeded_qm31(42))
    claimed = list(seeded_qm31(43))
    rc = np.random.default_rng(eval_log).integers(0, O.P, (O.POSEIDON_CONSTRAINTS, 4)).astype(np.uint32)
    start = m31_columns(700 + eval_log, 4, eval_log)
    gen, hand = _acc(start), _acc(start)
    fw.CompiledAir.get(fw.poseidon_air_recorded()).composition(
        {1: trace, 2: inter}, trace_log, fw.poseidon_params(lookup, claimed, trace_log), rc, gen)
    B.poseidon_composition(trace, inter, trace_log, lookup, claimed, rc, hand)
    assert all(np.array_equal(a, b) for a, b in zip(gen.to_cpu(), hand.to_cpu()))


def test_generic_poseidon_proof_equals_oracle_prover(B):
    # the whole Poseidon2 proof with the constraints through the generated kernel: the oracle's words
    from proving_gb300 import poseidon as ps
    from proving_gb300 import prover as pr
    log_n = 4
    fp = pr.FriParams(pow_bits=10, log_blowup_factor=1, log_last_layer_degree_bound=0, n_queries=70, fold_step=1)
    ops = pr.GpuOps()
    tw = ops.twiddles(log_n + ps.LOG_EXPAND + fp.log_blowup_factor)
    proof = ps.prove_poseidon(ops, log_n, ps.poseidon_pcs_config(log_n + 3, fp), pr.Blake2sChannel(), tw, check=False,
                              generic=True)
    assert proof.to_bytes() == O.prove_poseidon((10, 1, 0, 70, 1), log_n)


@pytest.mark.parametrize("trace_log,eval_log,split", [(3, 5, False), (10, 12, False), (6, 8, True), (14, 16, True)])
def test_mask_offsets_generated_equal_oracle(B, monkeypatch, trace_log, eval_log, split):
    # masks at offsets -3, -1, 0, 1 and 2 (offset_row / prev_row in the kernel), in one body and
    # split into functions that take each offset's row as an argument
    from test_mask_offsets_cpu import window_air
    if split:
        monkeypatch.setattr(fw, "_SINGLE_LINES", 4)
        monkeypatch.setattr(fw, "_CHUNK_NODES", 2)
    air = fw.compile_air("window", window_air)
    assert ("cs_air_group1(" in air.source) == split
    host = [m31_column(500 + k, eval_log) for k in range(4)]
    from proving_gb300.backend import BaseColumn
    cols = [BaseColumn.from_cpu(c) for c in host]
    rc = np.stack([seeded_qm31(510 + k) for k in range(air.n_constraints)])
    base = [m31_column(520 + k, eval_log) for k in range(4)]
    gen = _acc(base)
    fw.CompiledAir.get(air).composition({1: cols}, trace_log, {}, rc, gen)
    want = air_composition(air, {1: host}, eval_log, trace_log, {}, rc, out=base)
    assert all(np.array_equal(a, b) for a, b in zip(gen.to_cpu(), want))
