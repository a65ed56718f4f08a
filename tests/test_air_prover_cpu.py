"""The generic prover on the CPU (the oracle's operations behind the host logic): components
written against the constraint evaluator, committed tree by tree and proved with prove(), give the
bytes of the AIR-specific prover and of the oracle's prover for the mixed Wide-Fibonacci + LogUp
trace; AIRs with masks at other offsets, preprocessed columns and components of several sizes give
proofs the oracle's restated verifier accepts, and rejects once tampered with."""
import copy

import numpy as np
import pytest

from cpu_backend import CpuOps
from oracle import oracle as O
from oracle.verifier import VerificationError, verify_components
from proving_gb300 import air_prover as ap
from proving_gb300 import framework as fw
from proving_gb300 import prover as pr
from proving_gb300.poseidon import ConstraintsNotSatisfied
from proving_gb300.synthetic import seeded_qm31
from test_mask_offsets_cpu import window_air, window_trace
from test_prove_cpu import fib_and_lookups_inputs, fib_and_lookups_proof

FRI = pr.FriParams(pow_bits=10, log_blowup_factor=1, log_last_layer_degree_bound=0, n_queries=3, fold_step=1)


def fib_and_lookups_generic(ops):
    """The flow of prove_fib_and_lookups through the generic API: the empty preprocessed tree, the
    trace tree, the lookup elements, the interaction tree after the claimed sums, then prove()."""
    traces, logs, values, lookup_logs, _ = fib_and_lookups_inputs()
    cfg = pr.PcsConfig(FRI, trace_lifting_log_size=10)
    ch = pr.Blake2sChannel()
    scheme = ap.CommitmentSchemeProver(ops, cfg, ops.twiddles(10))
    scheme.commit([], ch)
    vals = [ops.columns_from_host([v])[0] for v in values]
    scheme.commit([c for t in traces for c in ops.columns_from_host(t)] + vals, ch)
    z = ch.draw_secure_felt()
    ch.draw_secure_felt()  # alpha
    sums, claimed = ops.logup_running_sums(vals, z)
    ch.mix_felts(claimed)
    scheme.commit([c for s in sums for c in ops.secure_coords(s)], ch)
    alloc = ap.TraceLocationAllocator()
    comps = [ap.FrameworkComponent(alloc, fw.compile_air(f"wide_fib_{len(t)}", fw.wide_fib_air, len(t)), log_n)
             for t, log_n in zip(traces, logs)]
    lookup = fw.compile_air("single_lookup", fw.single_lookup_air)
    comps += [ap.FrameworkComponent(alloc, lookup, log_n, {"z": z}, claimed_sum=c)
              for log_n, c in zip(lookup_logs, claimed)]
    return ap.prove(comps, ch, scheme), comps, z, claimed


def test_generic_proof_equals_the_air_specific_and_oracle_proofs():
    ops = CpuOps()
    proof, comps, z, claimed = fib_and_lookups_generic(ops)
    assert proof.to_bytes() == fib_and_lookups_proof(ops).to_bytes()
    traces, logs, values, lookup_logs, fri = fib_and_lookups_inputs()
    want, _ = O.prove_fib_and_lookups(fri, traces, logs, values, lookup_logs)
    assert proof.to_bytes() == want
    # and the generic verifier accepts it, the statement's claimed sums giving the shifts
    ch = O.Blake2sChannel()
    ch.mix_root(proof.commitments[0])
    ch.mix_root(proof.commitments[1])
    ch.draw_secure_felt()
    ch.draw_secure_felt()
    ch.mix_felts(np.asarray([list(c) for c in claimed], np.uint32).reshape(-1, 4))
    ch.mix_root(proof.commitments[2])
    sizes = [[], [log_n for t, log_n in zip(traces, logs) for _ in t] + list(lookup_logs),
             [log_n for log_n in lookup_logs for _ in range(4)]]
    verify_components(proof, ch, [(c.air, c.log_size, c.params) for c in comps], sizes)


def window_proof(log_n, extra=None, bad=False, check=True):
    """The window AIR (masks at -3, -1, 0, 1, 2) over 2^log_n rows, with optional further
    (air, host columns, log size) components in the same trace tree."""
    ops = CpuOps()
    extra = extra or []
    lifting = max([log_n] + [e[2] for e in extra]) + 1
    cfg = pr.PcsConfig(FRI, trace_lifting_log_size=lifting)
    ch = pr.Blake2sChannel()
    scheme = ap.CommitmentSchemeProver(ops, cfg, ops.twiddles(lifting))
    scheme.commit([], ch)
    host = window_trace(log_n, 9, bad=bad)
    cols = host + [c for _, cs, _ in extra for c in cs]
    scheme.commit(ops.columns_from_host(cols), ch)
    alloc = ap.TraceLocationAllocator()
    comps = [ap.FrameworkComponent(alloc, fw.compile_air("window", window_air), log_n)]
    comps += [ap.FrameworkComponent(alloc, air, n) for air, _, n in extra]
    proof = ap.prove(comps, ch, scheme, check=check)
    sizes = [[], [log_n] * 4 + [n for _, cs, n in extra for _ in cs]]
    return proof, comps, sizes


def verify_window(proof, comps, sizes):
    ch = O.Blake2sChannel()
    ch.mix_root(proof.commitments[0])
    ch.mix_root(proof.commitments[1])
    verify_components(proof, ch, [(c.air, c.log_size, c.params) for c in comps], sizes)


@pytest.mark.parametrize("log_n", [3, 5, 7])
def test_mask_offsets_prove_then_verify(log_n):
    proof, comps, sizes = window_proof(log_n)
    # x is sampled at its five offsets, y, z and w at the row; the x column has five samples, so
    # it takes no periodicity sample
    assert [len(c) for c in proof.sampled_values[1]] == [5, 1, 1, 1]
    verify_window(proof, comps, sizes)
    bad = copy.deepcopy(proof)
    bad.sampled_values[1][0][0] = tuple((v + 1) % O.P for v in bad.sampled_values[1][0][0])
    with pytest.raises(VerificationError):
        verify_window(bad, comps, sizes)


def test_unsatisfied_window_constraints_are_caught():
    with pytest.raises(ConstraintsNotSatisfied):
        window_proof(5, bad=True)
    proof, comps, sizes = window_proof(5, bad=True, check=False)
    assert not proof.constraints_satisfied
    with pytest.raises(VerificationError):
        verify_window(proof, comps, sizes)


def test_components_of_several_sizes_in_one_proof():
    # the window AIR at 2^4 rows beside a Wide-Fibonacci component of 6 columns x 2^6
    log_f = 6
    fib = O.wide_fib_trace(np.ones(1 << log_f, np.uint32), np.arange(1 << log_f, dtype=np.uint32), 6)
    extra = [(fw.compile_air("wide_fib_6", fw.wide_fib_air, 6), list(fib), log_f)]
    proof, comps, sizes = window_proof(4, extra=extra)
    assert comps[1].trace_locations == {1: (4, 10)}
    verify_window(proof, comps, sizes)


def seq_air(e):
    """y = x + seq^2 with seq a preprocessed column and x read at the next row too:
    x[1] - x[0] = seq (the preprocessed column steps x)."""
    seq = e.get_preprocessed_column("seq")
    x0, x1 = e.next_interaction_mask(1, (0, 1))
    y = e.next_trace_mask()
    e.add_constraint(y - x0 - seq * seq)
    e.add_constraint(x1 - x0 - seq)


def test_preprocessed_columns_prove_then_verify():
    log_n = 5
    n = 1 << log_n
    ops = CpuOps()
    cfg = pr.PcsConfig(FRI, trace_lifting_log_size=log_n + 1)
    # x steps by seq along the trace's coset order and wraps: seq sums to zero over the cycle
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
    ch = pr.Blake2sChannel()
    scheme = ap.CommitmentSchemeProver(ops, cfg, ops.twiddles(log_n + 1))
    scheme.commit(ops.columns_from_host([lay(seq_c)]), ch)
    scheme.commit(ops.columns_from_host([lay(x_c), lay(y_c)]), ch)
    alloc = ap.TraceLocationAllocator(preprocessed_columns=["seq"])
    air = fw.compile_air("seq", seq_air)
    assert air.preprocessed == ["seq"] and air.mask_offsets == {1: [(0, 1), (0,)]}
    comp = ap.FrameworkComponent(alloc, air, log_n)
    assert comp.preprocessed_column_indices == [0]
    proof = ap.prove([comp], ch, scheme)
    ch = O.Blake2sChannel()
    ch.mix_root(proof.commitments[0])
    ch.mix_root(proof.commitments[1])
    verify_components(proof, ch, [(air, log_n, {})], [[log_n], [log_n, log_n]], preprocessed_columns=["seq"])
    with pytest.raises(KeyError):
        ap.FrameworkComponent(ap.TraceLocationAllocator(preprocessed_columns=["other"]), air, log_n)


def test_preprocessed_columns_nobody_reads():
    # a second preprocessed column no component reads: sampled only with
    # include_all_preprocessed_columns (prove_ex's flag), decommitted either way
    log_n = 4
    ops = CpuOps()
    cfg = pr.PcsConfig(FRI, trace_lifting_log_size=log_n + 1)
    air = fw.compile_air("window", window_air)
    extra = np.arange(1 << log_n, dtype=np.uint32)
    for include_all in (False, True):
        ch = pr.Blake2sChannel()
        scheme = ap.CommitmentSchemeProver(ops, cfg, ops.twiddles(log_n + 1))
        scheme.commit(ops.columns_from_host([extra]), ch)
        scheme.commit(ops.columns_from_host(window_trace(log_n, 9)), ch)
        comp = ap.FrameworkComponent(ap.TraceLocationAllocator(["unused"]), air, log_n)
        proof = ap.prove([comp], ch, scheme, include_all_preprocessed_columns=include_all)
        assert [len(c) for c in proof.sampled_values[0]] == [1 if include_all else 0]
        assert len(proof.queried_values[0]) == 1
        v = O.Blake2sChannel()
        v.mix_root(proof.commitments[0])
        v.mix_root(proof.commitments[1])
        verify_components(proof, v, [(air, log_n, {})], [[log_n], [log_n] * 4], preprocessed_columns=["unused"],
                          include_all_preprocessed_columns=include_all)


def test_component_arguments_are_checked():
    with pytest.raises(ValueError):
        fw.compile_air("p", lambda e: e.next_interaction_mask(0))
    with pytest.raises(ValueError):
        ap.TraceLocationAllocator(preprocessed_columns=["a", "a"])
    lookup = fw.compile_air("single_lookup", fw.single_lookup_air)
    with pytest.raises(KeyError):
        ap.FrameworkComponent(ap.TraceLocationAllocator(), lookup, 4)   # no z (not a relation's parameter)
    # a relation's parameters may come later; prove() asks for them
    rel = fw.compile_air("lookup_rel", _relation_lookup_air)
    late = ap.FrameworkComponent(ap.TraceLocationAllocator(), rel, 4)
    assert "lookup_z" not in late.params and late.params["shift"] == (0, 0, 0, 0)
    scheme = ap.CommitmentSchemeProver(CpuOps(), pr.PcsConfig(FRI, trace_lifting_log_size=5), None)
    with pytest.raises(KeyError):
        ap.prove([late], pr.Blake2sChannel(), scheme)
    c = ap.FrameworkComponent(ap.TraceLocationAllocator(), lookup, 4, {"z": (1, 2, 3, 4)}, claimed_sum=(16, 0, 0, 0))
    assert c.params["shift"] == (1, 0, 0, 0)
    with pytest.raises(ValueError):
        ap.FrameworkComponent(ap.TraceLocationAllocator(), lookup, 4, {"z": (1, 2, 3, 4)}, constraint_log_degree=0)


def test_evaluation_mode_is_inferred_like_the_reference():
    # EvaluationMode::infer (crates/stwo/src/prover/air/accumulation.rs:42-62)
    air = fw.compile_air("window", window_air)

    def comps(*degrees):
        alloc = ap.TraceLocationAllocator()
        return [ap.FrameworkComponent(alloc, air, 4, constraint_log_degree=d) for d in degrees]
    assert ap.evaluation_mode(comps(1, 1), 1) == 0
    assert ap.evaluation_mode(comps(1, 1), 3) == 2
    assert ap.evaluation_mode(comps(2), 1) is None        # degree above the blowup
    assert ap.evaluation_mode(comps(1, 2), 2) is None     # expansions differ
    assert ap.evaluation_mode(comps(2, 2), 2) == 0


def blowup_proof(ops, log_n, log_blowup, degrees=(1, 1), fold_step=1, last_layer=0, check=True):
    """The window AIR and a Wide-Fibonacci component of 2^log_n rows with the given constraint
    log degrees, committed at log blowup log_blowup (as test_wide_fib_prove_with_larger_blowup,
    crates/examples/src/wide_fibonacci/mod.rs:311-370). The trees are lifted to the composition
    halves' domain, log_n + max degree - 1 + log_blowup (as poseidon_pcs_config)."""
    fri = pr.FriParams(pow_bits=10, log_blowup_factor=log_blowup, log_last_layer_degree_bound=last_layer,
                       n_queries=3, fold_step=fold_step)
    lifting = log_n + max(degrees) - 1 + log_blowup
    cfg = pr.PcsConfig(fri, trace_lifting_log_size=lifting)
    ch = pr.Blake2sChannel()
    scheme = ap.CommitmentSchemeProver(ops, cfg, ops.twiddles(lifting + 1))
    scheme.commit([], ch)
    fib = O.wide_fib_trace(np.ones(1 << log_n, np.uint32), np.arange(1 << log_n, dtype=np.uint32), 5)
    scheme.commit(ops.columns_from_host(window_trace(log_n, 9) + list(fib)), ch)
    alloc = ap.TraceLocationAllocator()
    comps = [ap.FrameworkComponent(alloc, fw.compile_air("window", window_air), log_n,
                                   constraint_log_degree=degrees[0]),
             ap.FrameworkComponent(alloc, fw.compile_air("wide_fib_5", fw.wide_fib_air, 5), log_n,
                                   constraint_log_degree=degrees[1])]
    proof = ap.prove(comps, ch, scheme, check=check)
    return proof, comps, [[], [log_n] * 9]


@pytest.mark.parametrize("log_n,log_blowup", [(4, 2), (5, 2), (6, 2), (7, 2), (5, 3), (4, 4)])
def test_larger_blowup_prove_then_verify(log_n, log_blowup):
    # log blowup b over constraints of log degree 1: SubDomain with log_expansion b - 1, the
    # composition interpolated on the committed domain's subdomain
    proof, comps, sizes = blowup_proof(CpuOps(), log_n, log_blowup)
    verify_window(proof, comps, sizes)
    bad = copy.deepcopy(proof)
    bad.sampled_values[1][4][0] = tuple((v + 1) % O.P for v in bad.sampled_values[1][4][0])
    with pytest.raises(VerificationError):
        verify_window(bad, comps, sizes)


@pytest.mark.parametrize("log_blowup,degrees", [(1, (2, 2)), (2, (1, 2)), (3, (2, 2))])
def test_constraint_degree_two_fails_the_sanity_check_like_the_reference(log_blowup, degrees):
    # "AIRs with constraint degree >= 2 are not supported yet in the lifted protocol"
    # (crates/examples/src/poseidon/mod.rs:467): the trace is committed below the trees' height and
    # lifted, the composition is not, so prove_ex's check compares values at different points
    with pytest.raises(ConstraintsNotSatisfied):
        blowup_proof(CpuOps(), 5, log_blowup, degrees)
    proof, _, _ = blowup_proof(CpuOps(), 5, log_blowup, degrees, check=False)
    assert not proof.constraints_satisfied


@pytest.mark.parametrize("log_n", [4, 5, 6, 7, 8])
def test_fri_fold_steps_prove_then_verify(log_n):
    # fold_step 2 for 2^4 and 2^5 rows, else 3, as test_wide_fib_prove_with_blake_with_fri_jumps
    # (crates/examples/src/wide_fibonacci/mod.rs:372-420): packed FRI leaves, a first layer of a
    # circle fold and line folds, a shorter last step
    k = 2 if log_n in (4, 5) else 3
    proof, comps, sizes = blowup_proof(CpuOps(), log_n, 1, fold_step=k)
    verify_window(proof, comps, sizes)
    # the tree height is log_n + 1; after the first layer's k folds, layers of k folds down to the
    # last layer's 2 values, the last step shorter
    assert len(proof.fri_inner_layers) == -(-(log_n + 1 - k - 1) // k)
    bad = copy.deepcopy(proof)
    w = bad.fri_first_layer["fri_witness"]
    w[0] = tuple((v + 1) % O.P for v in w[0])
    with pytest.raises(VerificationError):
        verify_window(bad, comps, sizes)


@pytest.mark.parametrize("log_n,log_blowup,fold_step,last_layer", [(6, 2, 2, 1), (7, 1, 4, 2), (5, 3, 3, 0),
                                                                     (8, 1, 2, 3)])
def test_fri_parameters_combined_prove_then_verify(log_n, log_blowup, fold_step, last_layer):
    # larger blowups, fold steps and last-layer degree bounds together
    proof, comps, sizes = blowup_proof(CpuOps(), log_n, log_blowup, fold_step=fold_step, last_layer=last_layer)
    assert len(proof.fri_last_layer_poly) == 1 << last_layer
    verify_window(proof, comps, sizes)
    bad = copy.deepcopy(proof)
    bad.fri_last_layer_poly[-1] = tuple((v + 1) % O.P for v in bad.fri_last_layer_poly[-1])
    with pytest.raises(VerificationError):
        verify_window(bad, comps, sizes)


def poseidon_generic(ops, log_n):
    """prove_poseidon's flow (crates/examples/src/poseidon/mod.rs:320-379) through the generic API:
    the AIR recorded by the evaluator, LOG_EXPAND 2 over a log blowup of 1 (ExtendToEvalDomain),
    the lifted configuration whose sanity check the reference itself fails (check=False)."""
    from proving_gb300 import poseidon as ps
    fp = pr.FriParams(pow_bits=10, log_blowup_factor=1, log_last_layer_degree_bound=0, n_queries=70, fold_step=1)
    cfg = ps.poseidon_pcs_config(log_n + 3, fp)
    tw = ops.twiddles(log_n + ps.LOG_EXPAND + 1)
    ch = pr.Blake2sChannel()
    scheme = ap.CommitmentSchemeProver(ops, cfg, tw)
    scheme.commit([], ch)
    trace = ops.poseidon_trace(log_n)
    scheme.commit(trace, ch)
    lookup = list(ch.draw_secure_felt()) + list(ch.draw_secure_felt())
    inter, claimed = ops.poseidon_interaction(trace, lookup)
    claimed = tuple(int(x) for x in claimed)
    scheme.commit(inter, ch)
    comp = ap.FrameworkComponent(ap.TraceLocationAllocator(), fw.poseidon_air_recorded(), log_n,
                                 fw.poseidon_params(lookup, claimed, log_n), constraint_log_degree=ps.LOG_EXPAND)
    proof = ap.prove([comp], ch, scheme, check=False)
    want = ps.prove_poseidon(ops, log_n, cfg, pr.Blake2sChannel(), tw, check=False, generic=True)
    return proof, want


def test_poseidon_through_the_generic_api_equals_prove_poseidon():
    proof, want = poseidon_generic(CpuOps(), 4)
    assert not proof.constraints_satisfied and not want.constraints_satisfied
    assert proof.to_bytes() == want.to_bytes()


def test_larger_blowup_with_components_of_several_sizes():
    # SubDomain with log_expansion 1 for a 2^4-row and a 2^6-row component: each accumulates on its
    # own committed domain's subdomain, the two lifted together before the composition is
    # interpolated on the largest one's subdomain
    fri = pr.FriParams(pow_bits=10, log_blowup_factor=2, log_last_layer_degree_bound=0, n_queries=3, fold_step=1)
    log_w, log_f = 4, 6
    lifting = log_f + 2
    ops = CpuOps()
    cfg = pr.PcsConfig(fri, trace_lifting_log_size=lifting)
    ch = pr.Blake2sChannel()
    scheme = ap.CommitmentSchemeProver(ops, cfg, ops.twiddles(lifting + 1))
    scheme.commit([], ch)
    fib = O.wide_fib_trace(np.ones(1 << log_f, np.uint32), np.arange(1 << log_f, dtype=np.uint32), 6)
    scheme.commit(ops.columns_from_host(window_trace(log_w, 9) + list(fib)), ch)
    alloc = ap.TraceLocationAllocator()
    comps = [ap.FrameworkComponent(alloc, fw.compile_air("window", window_air), log_w),
             ap.FrameworkComponent(alloc, fw.compile_air("wide_fib_6", fw.wide_fib_air, 6), log_f)]
    proof = ap.prove(comps, ch, scheme)
    verify_window(proof, comps, [[], [log_w] * 4 + [log_f] * 6])


def _run_program(nodes, cons, offs, mask, params):
    """The node program of cs_prove_air read back in Python (the semantics of include/stwo_cuda.h)."""
    v = []
    for op, a0, a1, a2, a3 in np.asarray(nodes, np.int64).tolist():
        if op == 0:
            v.append(tuple(mask[(a2, a0, offs[a0][a1])]))
        elif op == 1:
            v.append(pr.qm(a0))
        elif op == 2:
            v.append(tuple(params[a0]))
        elif op == 3:
            v.append(pr.from_partial_evals([v[a0], v[a1], v[a2], v[a3]]))
        elif op == 4:
            v.append(pr.qm_sub(pr.qm(0), v[a0]))
        else:
            v.append({5: pr.qm_add, 6: pr.qm_sub, 7: pr.qm_mul}[op](v[a0], v[a1]))
    return [v[c] for c in cons]


@pytest.mark.parametrize("make", [lambda: fw.compile_air("window", window_air),
                                  lambda: fw.compile_air("wide_fib_7", fw.wide_fib_air, 7)])
def test_point_program_equals_the_point_evaluation(make):
    air = make()
    nodes, cons, offs, masks, inter_two = air.point_program()
    assert len(cons) == air.n_constraints and len(masks) == len(air.masks) and inter_two == []
    assert all(offs[m.column][0] is not None and m.offset in offs[m.column] for m in air.masks)
    rng = np.random.default_rng(5)
    mask = {(1, c, o): tuple(int(x) for x in rng.integers(0, O.P, 4)) for c, os in enumerate(offs) for o in os}
    assert _run_program(nodes, cons, offs, mask, []) == ap.constraints_at_point(air, mask, {})


def test_point_program_reads_trace_and_interaction_columns_only():
    nodes, _, _, masks, inter_two = fw.compile_air("single_lookup", fw.single_lookup_air).point_program()
    assert inter_two == [True] * 4 and {t for _, t in masks} == {1, 2}
    with pytest.raises(NotImplementedError):
        fw.compile_air("seq", seq_air).point_program()


def _relation_lookup_air(e):
    e.add_to_relation("lookup", -1, [e.next_trace_mask()])
    e.finalize_logup()


@pytest.mark.parametrize("log_n", [1, 4, 9])
def test_generic_interaction_equals_the_single_column_running_sum(log_n):
    # the relation of multiplicity -1 and values [v]: fractions -1 / (v - z), the running sum of
    # logup_running_sum (the reference's LogupTraceGenerator for one batch)
    air = fw.compile_air("lookup_rel", _relation_lookup_air)
    ops = CpuOps()
    v = np.random.default_rng(log_n).integers(0, O.P, 1 << log_n, dtype=np.uint32)
    z = tuple(int(x) for x in seeded_qm31(41))
    cols, claimed = ap.logup_interaction(ops, air, ops.columns_from_host([v]), log_n,
                                         {"lookup_z": z, "lookup_alpha0": (1, 0, 0, 0)})
    want, want_claimed = O.logup_running_sum(v, z)
    assert all(np.array_equal(c.v, w) for c, w in zip(cols, want))
    assert claimed == tuple(int(x) for x in want_claimed)


@pytest.mark.parametrize("log_n", [2, 4])
def test_generic_interaction_equals_the_poseidon_interaction(log_n):
    # Poseidon2's two relation entries per instance finalized in pairs: the oracle's hand-written
    # interaction generator (gen_interaction_trace, crates/examples/src/poseidon/mod.rs:277-303)
    air = fw.poseidon_air_recorded()
    assert len(air.logup) == 8
    ops = CpuOps()
    trace = O.poseidon_trace(log_n)
    z, alpha = seeded_qm31(42), seeded_qm31(43)
    params = fw.lookup_params("poseidon", z, alpha, fw.POSEIDON_STATE)
    cols, claimed = ap.logup_interaction(ops, air, ops.columns_from_host(trace), log_n, params)
    want, want_claimed = O.poseidon_interaction(trace, z, alpha)
    assert all(np.array_equal(c.v, w) for c, w in zip(cols, want))
    assert claimed == tuple(int(x) for x in want_claimed)


def poseidon_fully_generic(ops, log_n):
    """prove_poseidon's flow with the interaction trace from the AIR's own fractions too."""
    from proving_gb300 import poseidon as ps
    fp = pr.FriParams(pow_bits=10, log_blowup_factor=1, log_last_layer_degree_bound=0, n_queries=70, fold_step=1)
    cfg = ps.poseidon_pcs_config(log_n + 3, fp)
    tw = ops.twiddles(log_n + ps.LOG_EXPAND + 1)
    ch = pr.Blake2sChannel()
    scheme = ap.CommitmentSchemeProver(ops, cfg, tw)
    scheme.commit([], ch)
    trace = ops.poseidon_trace(log_n)
    scheme.commit(trace, ch)
    z, alpha = ch.draw_secure_felt(), ch.draw_secure_felt()
    air = fw.poseidon_air_recorded()
    params = fw.lookup_params("poseidon", z, alpha, fw.POSEIDON_STATE)
    inter, claimed = ap.logup_interaction(ops, air, trace, log_n, params)
    scheme.commit(inter, ch)
    comp = ap.FrameworkComponent(ap.TraceLocationAllocator(), air, log_n, params, claimed_sum=claimed,
                                 constraint_log_degree=ps.LOG_EXPAND)
    return ap.prove([comp], ch, scheme, check=False)


def test_poseidon_fully_through_the_generic_api_equals_prove_poseidon():
    proof = poseidon_fully_generic(CpuOps(), 4)
    _, want = poseidon_generic(CpuOps(), 4)
    assert proof.to_bytes() == want.to_bytes()


def test_everything_in_one_proof_verifies():
    # a window AIR (offset masks), a relation entry with its interaction generated from the AIR's
    # fractions, and an AIR over a preprocessed column, in one proof: the restated verifier accepts
    # it after replaying the same commitments and draws, and rejects a wrong claimed sum
    log_n = 5
    n = 1 << log_n
    ops = CpuOps()
    cfg = pr.PcsConfig(FRI, trace_lifting_log_size=log_n + 1)
    rng = np.random.default_rng(11)
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
    window, rel, seq = (fw.compile_air("window", window_air), fw.compile_air("lookup_rel", _relation_lookup_air),
                        fw.compile_air("seq", seq_air))
    values = rng.integers(0, O.P, n, dtype=np.uint32)
    trace = window_trace(log_n, 4) + [values, lay(x_c), lay(y_c)]
    ch = pr.Blake2sChannel()
    scheme = ap.CommitmentSchemeProver(ops, cfg, ops.twiddles(log_n + 1))
    scheme.commit(ops.columns_from_host([lay(seq_c)]), ch)
    trace_cols = ops.columns_from_host(trace)
    scheme.commit(trace_cols, ch)
    z, alpha = ch.draw_secure_felt(), ch.draw_secure_felt()
    params = fw.lookup_params("lookup", z, alpha, 1)
    inter, claimed = ap.logup_interaction(ops, rel, [trace_cols[4]], log_n, params)
    ch.mix_felts([claimed])
    scheme.commit(inter, ch)
    alloc = ap.TraceLocationAllocator(preprocessed_columns=["seq"])
    comps = [ap.FrameworkComponent(alloc, window, log_n), ap.FrameworkComponent(alloc, rel, log_n, params, claimed),
             ap.FrameworkComponent(alloc, seq, log_n)]
    assert [c.trace_locations[1] for c in comps] == [(0, 4), (4, 5), (5, 7)]
    proof = ap.prove(comps, ch, scheme)

    def verify(claimed_sum):
        v = O.Blake2sChannel()
        v.mix_root(proof.commitments[0])
        v.mix_root(proof.commitments[1])
        vz, va = v.draw_secure_felt(), v.draw_secure_felt()
        vp = fw.lookup_params("lookup", vz, va, 1)
        vp["shift"] = fw.logup_shift(claimed_sum, log_n)
        v.mix_felts(np.asarray([list(claimed_sum)], np.uint32))
        v.mix_root(proof.commitments[2])
        verify_components(proof, v, [(window, log_n, {}), (rel, log_n, vp), (seq, log_n, {})],
                          [[log_n], [log_n] * 7, [log_n] * 4], preprocessed_columns=["seq"])
    verify(claimed)
    with pytest.raises(VerificationError):
        verify(tuple((c + 1) % O.P for c in claimed))
