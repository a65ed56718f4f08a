"""GPU parity of the generic prover: proofs of components written against the constraint evaluator,
their constraints run as kernels compiled at run time, equal the oracle's prover (the mixed
Wide-Fibonacci + LogUp trace) and the host prover on the oracle's operations (masks at several
offsets, preprocessed columns, components of several sizes, larger blowups, FRI fold steps above
one with packed leaves, last layers of higher degree), byte for byte."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from cpu_backend import CpuOps  # noqa: E402
from oracle import oracle as O  # noqa: E402
from proving_gb300 import air_prover as ap  # noqa: E402
from proving_gb300 import framework as fw  # noqa: E402
from proving_gb300 import prover as pr  # noqa: E402
from test_air_prover_cpu import (FRI, _relation_lookup_air, blowup_proof, fib_and_lookups_generic,  # noqa: E402
                                 poseidon_fully_generic, poseidon_generic, seq_air)
from test_mask_offsets_cpu import window_air, window_trace  # noqa: E402
from test_prove_cpu import fib_and_lookups_inputs  # noqa: E402


@pytest.fixture(scope="module")
def ops():
    from proving_gb300 import _lib, build
    build.build()
    _lib.call("cs_rtc_available")
    return pr.GpuOps()


def test_generic_fib_and_lookups_proof_equals_oracle(ops):
    proof, _, _, _ = fib_and_lookups_generic(ops)
    traces, logs, values, lookup_logs, fri = fib_and_lookups_inputs()
    want, _ = O.prove_fib_and_lookups(fri, traces, logs, values, lookup_logs)
    assert proof.to_bytes() == want


def _window_and_fib(o, log_w, log_f, n_fib):
    lifting = max(log_w, log_f) + 1
    cfg = pr.PcsConfig(FRI, trace_lifting_log_size=lifting)
    ch = pr.Blake2sChannel()
    scheme = ap.CommitmentSchemeProver(o, cfg, o.twiddles(lifting))
    scheme.commit([], ch)
    fib = O.wide_fib_trace(np.ones(1 << log_f, np.uint32), np.arange(1 << log_f, dtype=np.uint32), n_fib)
    scheme.commit(o.columns_from_host(window_trace(log_w, 9) + list(fib)), ch)
    alloc = ap.TraceLocationAllocator()
    comps = [ap.FrameworkComponent(alloc, fw.compile_air("window", window_air), log_w),
             ap.FrameworkComponent(alloc, fw.compile_air(f"wide_fib_{n_fib}", fw.wide_fib_air, n_fib), log_f)]
    return ap.prove(comps, ch, scheme).to_bytes()


@pytest.mark.parametrize("log_w,log_f,n_fib", [(4, 6, 6), (9, 5, 3), (12, 12, 20)])
def test_mask_offsets_proof_equals_host_prover_on_oracle_ops(ops, log_w, log_f, n_fib):
    assert _window_and_fib(ops, log_w, log_f, n_fib) == _window_and_fib(CpuOps(), log_w, log_f, n_fib)


def _seq_proof(o, log_n):
    n = 1 << log_n
    rng = np.random.default_rng(3)
    seq_c = rng.integers(0, O.P, n, dtype=np.int64)
    seq_c[-1] = (-seq_c[:-1].sum()) % O.P
    x_c = np.concatenate([[5], (5 + np.cumsum(seq_c[:-1])) % O.P])
    y_c = (x_c + seq_c * seq_c) % O.P
    k = np.arange(n)
    nat = np.where(k % 2 == 0, k // 2, n - 1 - (k - 1) // 2)
    rows = np.array([int(format(int(v), f"0{log_n}b")[::-1], 2) for v in nat])

    def lay(c):
        out = np.zeros(n, np.uint32)
        out[rows] = c
        return out
    cfg = pr.PcsConfig(FRI, trace_lifting_log_size=log_n + 1)
    ch = pr.Blake2sChannel()
    scheme = ap.CommitmentSchemeProver(o, cfg, o.twiddles(log_n + 1))
    scheme.commit(o.columns_from_host([lay(seq_c)]), ch)
    scheme.commit(o.columns_from_host([lay(x_c), lay(y_c)]), ch)
    comp = ap.FrameworkComponent(ap.TraceLocationAllocator(["seq"]), fw.compile_air("seq", seq_air), log_n)
    return ap.prove([comp], ch, scheme).to_bytes()


def test_preprocessed_column_proof_equals_host_prover_on_oracle_ops(ops):
    assert _seq_proof(ops, 10) == _seq_proof(CpuOps(), 10)


@pytest.mark.parametrize("log_n,log_blowup,fold_step,last_layer", [(6, 2, 1, 0), (8, 1, 3, 0), (10, 2, 2, 1),
                                                                     (12, 1, 4, 2), (9, 3, 2, 0)])
def test_blowup_and_fold_steps_equal_host_prover_on_oracle_ops(ops, log_n, log_blowup, fold_step, last_layer):
    kw = dict(fold_step=fold_step, last_layer=last_layer)
    got, _, _ = blowup_proof(ops, log_n, log_blowup, **kw)
    want, _, _ = blowup_proof(CpuOps(), log_n, log_blowup, **kw)
    assert got.to_bytes() == want.to_bytes()


@pytest.mark.parametrize("log_n", [4, 7])
def test_poseidon_through_the_generic_api_equals_oracle(ops, log_n):
    # Poseidon2's 1,144 constraints as the generated kernel, extended to CanonicCoset(n + 2): the
    # generic API's words equal prove_poseidon's and the oracle prover's
    proof, want = poseidon_generic(ops, log_n)
    assert proof.to_bytes() == want.to_bytes() == O.prove_poseidon((10, 1, 0, 70, 1), log_n)


def _native_against_python(o, specs, plain=False):
    """specs: (air, log size, host columns) per component, in trace order. Returns (native bytes,
    bytes of prove() for the same flow)."""
    lifting = max(n for _, n, _ in specs) + 1
    cfg = pr.PcsConfig(FRI, trace_lifting_log_size=lifting)
    tw = o.twiddles(lifting + 1)
    host = [c for _, _, cols in specs for c in cols]
    ch = pr.Blake2sChannel()
    scheme = ap.CommitmentSchemeProver(o, cfg, tw)
    scheme.commit([], ch)
    scheme.commit(o.columns_from_host(host), ch)
    alloc = ap.TraceLocationAllocator()
    comps = [ap.FrameworkComponent(alloc, air, n) for air, n, _ in specs]
    want = ap.prove(comps, ch, scheme).to_bytes()
    got = ap.prove_native(comps, o.columns_from_host(host), cfg, tw, plain=plain)
    return got, want


def _fib(log_n, n_cols):
    return list(O.wide_fib_trace(np.ones(1 << log_n, np.uint32), np.arange(1 << log_n, dtype=np.uint32), n_cols))


@pytest.mark.parametrize("plain", [False, True])
def test_native_generic_prover_equals_the_python_generic_prover(ops, plain):
    # masks at -3..2 and components of three sizes through cs_prove_air: the words of air_prover.prove
    window = fw.compile_air("window", window_air)
    fib = fw.compile_air("wide_fib_3", fw.wide_fib_air, 3)
    specs = [(window, 9, window_trace(9, 1)), (fib, 5, _fib(5, 3)), (window, 12, window_trace(12, 2))]
    got, want = _native_against_python(ops, specs, plain)
    assert got == want


@pytest.mark.parametrize("log_blowup,degrees,fold_step", [(2, (1, 1), 1), (3, (1, 1), 2), (2, (2, 2), 1),
                                                          (2, (1, 2), 3), (3, (1, 2), 1)])
def test_native_generic_prover_with_larger_blowups_equals_the_python_generic_prover(ops, log_blowup, degrees,
                                                                                    fold_step):
    # SubDomain evaluation (every constraint degree at most the blowup, by the same log_expansion)
    # and ExtendToEvalDomain (degrees that differ, or above the blowup), FRI with one or several
    # folds per layer, through cs_prove_air: the words of air_prover.prove for the same components
    log_n = 7
    want, comps, _ = blowup_proof(ops, log_n, log_blowup, degrees, fold_step=fold_step, check=max(degrees) == 1)
    lifting = log_n + max(degrees) - 1 + log_blowup
    fri = pr.FriParams(pow_bits=10, log_blowup_factor=log_blowup, log_last_layer_degree_bound=0, n_queries=3,
                       fold_step=fold_step)
    fib = O.wide_fib_trace(np.ones(1 << log_n, np.uint32), np.arange(1 << log_n, dtype=np.uint32), 5)
    trace = ops.columns_from_host(window_trace(log_n, 9) + list(fib))
    got = ap.prove_native(comps, trace, pr.PcsConfig(fri, trace_lifting_log_size=lifting), ops.twiddles(lifting + 1))
    assert got == want.to_bytes()


def test_native_generic_prover_single_component_equals_oracle(ops):
    # one Wide-Fibonacci component through cs_prove_air: the oracle prover's words
    fib = fw.compile_air("wide_fib_8", fw.wide_fib_air, 8)
    trace = _fib(10, 8)
    got, want = _native_against_python(ops, [(fib, 10, trace)])
    assert got == want == O.prove_fib_and_lookups((10, 1, 0, 3, 1), [trace], [10])[0]


@pytest.mark.parametrize("log_n", [1, 12])
def test_generic_interaction_on_gpu_equals_the_running_sum(ops, log_n):
    from proving_gb300.synthetic import seeded_qm31
    air = fw.compile_air("lookup_rel", _relation_lookup_air)
    v = np.random.default_rng(log_n).integers(0, O.P, 1 << log_n, dtype=np.uint32)
    z = tuple(int(x) for x in seeded_qm31(41))
    cols, claimed = ap.logup_interaction(ops, air, ops.columns_from_host([v]), log_n,
                                         {"lookup_z": z, "lookup_alpha0": (1, 0, 0, 0)})
    want, want_claimed = O.logup_running_sum(v, z)
    assert all(np.array_equal(c.to_cpu(), w) for c, w in zip(cols, want))
    assert claimed == tuple(int(x) for x in want_claimed)


def test_generic_poseidon_interaction_on_gpu_equals_the_hand_written_kernel(ops):
    from proving_gb300.synthetic import seeded_qm31
    log_n = 8
    air = fw.poseidon_air_recorded()
    trace = ops.poseidon_trace(log_n)
    z, alpha = seeded_qm31(42), seeded_qm31(43)
    params = fw.lookup_params("poseidon", z, alpha, fw.POSEIDON_STATE)
    cols, claimed = ap.logup_interaction(ops, air, trace, log_n, params)
    want, want_claimed = ops.poseidon_interaction(trace, [int(x) for x in z] + [int(x) for x in alpha])
    assert all(np.array_equal(c.to_cpu(), w.to_cpu()) for c, w in zip(cols, want))
    assert claimed == tuple(int(x) for x in want_claimed)


def test_poseidon_fully_through_the_generic_api_equals_oracle(ops):
    proof = poseidon_fully_generic(ops, 4)
    assert proof.to_bytes() == O.prove_poseidon((10, 1, 0, 70, 1), 4)


def test_native_generic_prover_with_relations_equals_oracle(ops):
    # two components of the relation entry -1 / (v - z) (sizes 2^8 and 2^4), their interaction tree
    # generated from their fraction kernels, the claimed sums mixed before its root: the oracle's
    # proof of two single-column LogUp components. The relation's parameters come from the draw.
    air = fw.compile_air("lookup_rel", _relation_lookup_air)
    rng = np.random.default_rng(7)
    vals = [rng.integers(0, O.P, 1 << n, dtype=np.uint32) for n in (8, 4)]
    cfg = pr.PcsConfig(FRI, trace_lifting_log_size=9)
    tw = ops.twiddles(10)
    alloc = ap.TraceLocationAllocator()
    comps = [ap.FrameworkComponent(alloc, air, n) for n in (8, 4)]
    got = ap.prove_native(comps, ops.columns_from_host(vals), cfg, tw, mix_claimed=True)
    want, _ = O.prove_fib_and_lookups((10, 1, 0, 3, 1), [], [], vals, [8, 4])
    assert got == want


@pytest.mark.parametrize("log_n", [4, 7])
def test_native_generic_poseidon_equals_the_hand_written_native_prover(ops, log_n):
    # Poseidon2 recorded by the evaluator through cs_prove_air: fraction kernel, generated
    # interaction, constraint log degree 2 (extended evaluation, no sanity check): the words of
    # cs_prove_poseidon and of the oracle prover
    from proving_gb300 import poseidon as ps
    from proving_gb300.backend import CudaBackend
    air = fw.poseidon_air_recorded()
    fp = pr.FriParams(pow_bits=10, log_blowup_factor=1, log_last_layer_degree_bound=0, n_queries=70, fold_step=1)
    cfg = ps.poseidon_pcs_config(log_n + 3, fp)
    tw = ops.twiddles(log_n + ps.LOG_EXPAND + 1)
    # z, the alpha powers and the shift come from the proof
    comp = ap.FrameworkComponent(ap.TraceLocationAllocator(), air, log_n, constraint_log_degree=ps.LOG_EXPAND)
    got = ap.prove_native([comp], ops.poseidon_trace(log_n), cfg, tw)
    want = CudaBackend.prove_poseidon_native(log_n, (10, 1, 0, 70), tw)
    assert got == want == O.prove_poseidon((10, 1, 0, 70, 1), log_n)


def test_native_generic_prover_rejects_inconsistent_components(ops):
    # every table is checked against the kernel and the program before any launch
    from proving_gb300._lib import CudaBackendError
    from proving_gb300.backend import CudaBackend
    from proving_gb300.framework import CompiledAir
    air = fw.compile_air("window", window_air)
    nodes, cons, offs, masks, inter_two = air.point_program()
    good = {"kernel": CompiledAir.get(air).handle, "log_size": 6, "degree": 1, "offsets": offs, "masks": masks,
            "nodes": nodes, "constraints": cons, "params": [], "kinds": [], "n_batches": 0, "frac_cols": [],
            "inter_two": []}
    tw = ops.twiddles(8)

    def attempt(**change):
        spec = dict(good, **change)
        trace = ops.columns_from_host(window_trace(6, 3))
        return CudaBackend.prove_air_native([spec], trace, 7, (10, 1, 0, 3), tw)
    assert len(attempt()) > 0
    bad_nodes = np.array(nodes, np.uint32)
    bad_nodes[len(bad_nodes) // 2, 1] = len(bad_nodes) - 1          # reads a later node
    for change in ({"nodes": bad_nodes}, {"masks": masks[:-1]}, {"constraints": cons[:-1]},
                   {"degree": 3}, {"masks": [(9, 1)] + masks[1:]}, {"offsets": offs[:-1]}):
        with pytest.raises(CudaBackendError):
            attempt(**change)
