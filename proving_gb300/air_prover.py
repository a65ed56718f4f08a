"""The generic prover: components whose constraints are written against the constraint evaluator
(proving_gb300.framework), committed tree by tree and proved by prove(), as with the reference's
constraint framework and prover:

- TraceLocationAllocator and FrameworkComponent (crates/constraint-framework/src/component.rs):
  each component's columns in each tree, its mask points, its constraints at the OODS point;
- CommitmentSchemeProver (crates/stwo/src/prover/pcs/mod.rs:76-110): one tree per commit, the
  columns' trace-domain evaluations interpolated, evaluated on the blown-up domain, committed by
  the lifted Merkle tree, the root mixed into the channel;
- prove (prove_ex, crates/stwo/src/prover/mod.rs:39-138): the composition polynomial from every
  component's generated kernel, its commitment, the OODS proof of work and point, the sampled
  values, the FRI quotients, FRI, the proof of work and the decommitments.

The device work goes through the same operations object as the AIR-specific provers
(proving_gb300.prover.GpuOps); an AIR's constraints run as the kernel NVRTC compiled from it.

    scheme = CommitmentSchemeProver(ops, config, twiddles)
    scheme.commit([], channel)                 # the preprocessed tree
    scheme.commit(trace, channel)              # bit-reversed trace-domain evaluations
    alloc = TraceLocationAllocator()
    proof = prove([FrameworkComponent(alloc, air, log_size)], channel, scheme)
"""
from __future__ import annotations

import hashlib

from . import prover as pr
from .framework import Air
from .poseidon import ConstraintsNotSatisfied
from .prover import P, PcsConfig, m_inv, qm, qm_add, qm_inv, qm_mul, qm_sub


class TraceLocationAllocator:
    """Hands each component, in the order they are made, the next columns of every tree it reads
    (TraceLocationAllocator::next_for_structure), and the preprocessed columns by id: in order of
    first use, or from a fixed list (new_with_preprocessed_columns), where an id outside the list
    is an error."""

    def __init__(self, preprocessed_columns=None):
        self.next_offsets: dict[int, int] = {}
        self.static = preprocessed_columns is not None
        self.preprocessed_columns = list(preprocessed_columns or [])
        if len(set(self.preprocessed_columns)) != len(self.preprocessed_columns):
            raise ValueError("Duplicate preprocessed columns are not allowed!")

    def next_for_structure(self, mask_offsets: dict) -> dict:
        """tree -> (first column, end) for the columns mask_offsets lists per tree (trees 1..)."""
        spans = {}
        for tree in range(1, max(mask_offsets, default=0) + 1):
            start = self.next_offsets.get(tree, 0)
            end = start + len(mask_offsets.get(tree, []))
            self.next_offsets[tree] = end
            spans[tree] = (start, end)
        return spans

    def preprocessed_index(self, name: str) -> int:
        if name not in self.preprocessed_columns:
            if self.static:
                raise KeyError(f"preprocessed column {name!r} is not in the fixed set")
            self.preprocessed_columns.append(name)
        return self.preprocessed_columns.index(name)


class FrameworkComponent:
    """An AIR over a trace of 2^log_size rows with its columns' places in the trees
    (FrameworkComponent::new). params: the AIR's QM31 parameters by name. claimed_sum: the
    component's LogUp claimed sum; when the AIR reads the parameter `shift` and params do not give
    it, it is claimed_sum / 2^log_size (LogupAtRow::new). constraint_log_degree: log2 of the
    constraints' degree bound over the trace's, so that max_constraint_log_degree_bound is
    log_size + constraint_log_degree (the examples' LOG_EXPAND)."""

    def __init__(self, allocator: TraceLocationAllocator, air: Air, log_size: int, params=None,
                 claimed_sum=None, constraint_log_degree: int = 1):
        if constraint_log_degree < 1:
            raise ValueError("the composition polynomial is split in two: constraint_log_degree >= 1")
        self.air = air
        self.log_size = log_size
        self.constraint_log_degree = constraint_log_degree
        self.trace_locations = allocator.next_for_structure(air.mask_offsets)
        self.preprocessed_column_indices = [allocator.preprocessed_index(n) for n in air.preprocessed]
        self.claimed_sum = qm(0) if claimed_sum is None else tuple(int(x) % P for x in claimed_sum)
        params = {k: tuple(int(x) % P for x in v) for k, v in (params or {}).items()}
        if "shift" in air.params and "shift" not in params:
            inv = m_inv(1 << log_size)
            params["shift"] = tuple(c * inv % P for c in self.claimed_sum)
        # a relation's z and alpha powers may come later (prove() needs them; prove_native draws them)
        missing = [n for n in air.params if n not in params and _param_kind(air, n) == 0]
        if missing:
            raise KeyError(f"{air.name}: no value for the parameters {missing}")
        self.params = params

    @property
    def n_constraints(self) -> int:
        return self.air.n_constraints

    def max_constraint_log_degree_bound(self) -> int:
        return self.log_size + self.constraint_log_degree

    def mask_points(self, point, max_log_degree_bound: int) -> dict:
        """(tree, column) -> the points its values are sampled at: the point plus offset steps of
        CanonicCoset(max_log_degree_bound) (component.rs:202-214); a preprocessed column at the
        point."""
        out = {}
        for tree, (start, _) in self.trace_locations.items():
            for k, offsets in enumerate(self.air.mask_offsets.get(tree, [])):
                out[(tree, start + k)] = [point_at_offset(point, o, max_log_degree_bound) for o in offsets]
        for idx in self.preprocessed_column_indices:
            out[(0, idx)] = [point]
        return out

    def mask_values(self, sampled) -> dict:
        """(interaction, column, offset) -> the sampled value the AIR's mask reads."""
        mask = {}
        for tree, (start, _) in self.trace_locations.items():
            for k, offsets in enumerate(self.air.mask_offsets.get(tree, [])):
                for j, o in enumerate(offsets):
                    mask[(tree, k, o)] = sampled[tree][start + k][j]
        for k, idx in enumerate(self.preprocessed_column_indices):
            mask[(0, k, 0)] = sampled[0][idx][0]
        return mask


def point_at_offset(point, offset: int, log_size: int):
    """point + offset G_log_size (the generator of CanonicCoset(log_size)'s subgroup)."""
    g = pr.index_to_point((offset << (31 - log_size)) % (1 << 31))
    return pr.qpoint_add_m31(point, g)


def constraints_at_point(air: Air, mask: dict, params: dict) -> list:
    """The AIR's constraints at a point from its mask values (PointEvaluator,
    crates/constraint-framework/src/point.rs:12-64): every value is a QM31, four base values
    combine as SecureField::from_partial_evals."""
    memo = {}
    stack = list(air.constraints)
    while stack:
        x = stack[-1]
        if x.key in memo:
            stack.pop()
            continue
        kids = [a for a in x.args if hasattr(a, "key")]
        todo = [a for a in kids if a.key not in memo]
        if todo:
            stack.extend(todo)
            continue
        stack.pop()
        if x.op == "mask":
            v = tuple(mask[x.args])
        elif x.op == "const":
            v = qm(x.args[0])
        elif x.op == "param":
            v = tuple(params[x.args[0]])
        elif x.op == "secure":
            v = pr.from_partial_evals([memo[a.key] for a in x.args])
        elif x.op == "neg":
            v = qm_sub(qm(0), memo[x.args[0].key])
        else:
            a, b = memo[x.args[0].key], memo[x.args[1].key]
            v = {"add": qm_add, "sub": qm_sub, "mul": qm_mul}[x.op](a, b)
        memo[x.key] = v
    return [memo[c.key] for c in air.constraints]


class _Tree:
    def __init__(self, evals, coeffs, log_sizes, merkle, root):
        self.evals, self.coeffs, self.log_sizes, self.merkle, self.root = evals, coeffs, log_sizes, merkle, root


def evaluation_mode(components, log_blowup_factor: int):
    """EvaluationMode::infer (crates/stwo/src/prover/air/accumulation.rs:42-62): the common
    log_expansion = log_blowup_factor - constraint log degree of every component (SubDomain: the
    constraints are evaluated on a subdomain of the committed evaluations), or None when a
    component's constraint degree exceeds the blowup or two components differ
    (ExtendToEvalDomain: the columns are evaluated anew on CanonicCoset(max constraint bound))."""
    common = None
    for c in components:
        if c.constraint_log_degree > log_blowup_factor:
            return None
        e = log_blowup_factor - c.constraint_log_degree
        if common is not None and common != e:
            return None
        common = e
    return 0 if common is None else common


class CommitmentSchemeProver:
    """The committed trees of one proof (CommitmentSchemeProver). twiddles: for the largest
    evaluation domain the proof uses."""

    def __init__(self, ops, config: PcsConfig, twiddles):
        self.ops, self.config, self.twiddles = ops, config, twiddles
        self.trees: list[_Tree] = []

    def commit(self, columns, channel: pr.Blake2sChannel) -> bytes:
        """tree_builder().extend_evals(columns) and commit(channel): columns are device columns of
        bit-reversed trace-domain evaluations (kept), any sizes; the first tree is the
        preprocessed one. Returns the root."""
        ops, b = self.ops, self.config.fri_params.log_blowup_factor
        columns = list(columns)
        if not columns:
            tree = _Tree([], [], [], None, hashlib.blake2s(b"").digest())
        else:
            height = self.config.trace_lifting_log_size
            if not self.trees and self.config.preprocessed_lifting_log_size not in (0, height):
                raise NotImplementedError("a preprocessed tree lifted to the trace trees' height")
            logs = [ops.log_size(c) for c in columns]
            coeffs = [None] * len(columns)
            for _, idx in pr._size_groups(logs).items():
                for i, c in zip(idx, ops.interpolate_into([columns[i] for i in idx], self.twiddles)):
                    coeffs[i] = c
            evals = pr._evaluate_grouped(ops, coeffs, logs, b, self.twiddles)
            merkle = ops.merkle_commit(evals, height)
            tree = _Tree(evals, coeffs, logs, merkle, merkle.root)
        self.trees.append(tree)
        channel.mix_root(tree.root)
        return tree.root

    def component_columns(self, comp: FrameworkComponent, eval_log: int, subdomain: bool) -> dict:
        """interaction -> the component's columns for its constraint evaluation
        (get_trace_columns, crates/constraint-framework/src/prover/component_prover.rs:29-56): in
        SubDomain mode the committed evaluations, whose first 2^eval_log rows are the evaluation
        domain; in ExtendToEvalDomain mode the columns on CanonicCoset(eval_log), the committed
        evaluations when that is their domain, else the coefficients evaluated there."""
        b = self.config.fri_params.log_blowup_factor
        picks = {t: list(range(s, e)) for t, (s, e) in comp.trace_locations.items()}
        if comp.preprocessed_column_indices:
            picks[0] = comp.preprocessed_column_indices
        out = {}
        for t, idx in picks.items():
            if t >= len(self.trees) or (idx and idx[-1] >= len(self.trees[t].evals)):
                raise ValueError(f"{comp.air.name}: tree {t} has no column {idx[-1] if idx else 0}")
            tree = self.trees[t]
            if any(tree.log_sizes[i] != comp.log_size for i in idx):
                raise ValueError(f"{comp.air.name}: a column of tree {t} is not 2^{comp.log_size} rows")
            if subdomain or eval_log == comp.log_size + b:
                out[t] = [tree.evals[i] for i in idx]
            else:
                out[t] = self.ops.evaluate([tree.coeffs[i] for i in idx], eval_log, self.twiddles) if idx else []
        return out


def prove(components, channel: pr.Blake2sChannel, scheme: CommitmentSchemeProver, check: bool = True,
          include_all_preprocessed_columns: bool = False):
    """prove_ex: with include_all_preprocessed_columns every preprocessed column is sampled at the
    OODS point, else only those the components read (Components::mask_points,
    crates/stwo/src/core/air/components.rs:27-51; prove() passes false). Raises
    ConstraintsNotSatisfied when the composition polynomial's OODS value differs from the
    components' constraints at the point (check=False returns the proof with constraints_satisfied
    set instead)."""
    ops, cfg, tw = scheme.ops, scheme.config, scheme.twiddles
    fp = cfg.fri_params
    b = fp.log_blowup_factor
    L = cfg.trace_lifting_log_size
    if not components:
        raise ValueError("no components")

    # --- composition polynomial (ComponentProvers::compute_composition_polynomial): components in
    # order take the highest powers of the random coefficient, each constraint the next lower one
    for comp in components:
        missing = [n for n in comp.air.params if n not in comp.params]
        if missing:
            raise KeyError(f"{comp.air.name}: no value for the parameters {missing}")
    random_coeff = channel.draw_secure_felt()
    log_expansion = evaluation_mode(components, b)
    total = sum(c.n_constraints for c in components)
    powers = ops.secure_powers(random_coeff, total)
    sub_acc, start = {}, 0
    for comp in components:
        n = comp.n_constraints
        rc = list(reversed(powers[total - start - n:total - start]))
        eval_log = comp.max_constraint_log_degree_bound()
        if eval_log not in sub_acc:
            sub_acc[eval_log] = ops.secure_zeros(1 << eval_log)
        cols = scheme.component_columns(comp, eval_log, log_expansion is not None)
        ops.air_composition(comp.air, cols, comp.log_size, comp.params, rc, sub_acc[eval_log], log_expansion or 0)
        start += n
    accs = [sub_acc[k] for k in sorted(sub_acc)]
    accum = accs[0] if len(accs) == 1 else ops.lift_and_accumulate(accs)
    comp_log = max(sub_acc)
    # DomainEvaluationAccumulator::finalize (accumulation.rs:136-180): on the subdomain of
    # CanonicCoset(comp_log + log_expansion) in SubDomain mode, else on CanonicCoset(comp_log)
    if log_expansion:
        comp_coeffs = ops.interpolate_secure_on_subdomain(accum, comp_log + log_expansion, tw)
    else:
        comp_coeffs = ops.interpolate_secure(accum, tw)
    left, right = ops.split_at_mid(comp_coeffs)
    comp_evals = ops.evaluate(left + right, (comp_log - 1) + b, tw)
    comp_tree = ops.merkle_commit(comp_evals, L)
    channel.mix_root(comp_tree.root)

    # --- OODS proof of work and point, the mask points of every component
    oods_pow = ops.grind(channel.digest, pr.OODS_POW_BITS)
    channel.mix_u64(oods_pow)
    oods = pr.random_point(channel.draw_secure_felt())
    mldb = L - b
    sample_points = [[[] for _ in t.evals] for t in scheme.trees]
    for comp in components:
        for (t, c), pts in comp.mask_points(oods, mldb).items():
            sample_points[t][c] = pts
    if include_all_preprocessed_columns and scheme.trees:
        sample_points[0] = [[oods] for _ in scheme.trees[0].evals]
    sample_points.append([[oods]] * 8)
    columns = [t.evals for t in scheme.trees] + [comp_evals]
    sampled = pr.sample_values(ops, columns, sample_points, L)
    channel.mix_felts([v for tree in sampled for col in tree for v in col])
    quotient_coeff = channel.draw_secure_felt()
    quotients = pr.compute_fri_quotients(ops, columns, sample_points, sampled, quotient_coeff, L, b, tw)
    fri = pr.fri_commit(ops, channel, fp, quotients, L, tw)

    # --- proof of work, queries, decommitments
    fri_pow = ops.grind(channel.digest, fp.pow_bits)
    channel.mix_u64(fri_pow)
    queries = sorted(set(channel.draw_queries(L, fp.n_queries)))
    reads = pr.Reads()
    first = pr.FriLayerDecommit(reads, quotients, fri["first"]["tree"], queries, fp.fold_step, ops)
    inner = []
    layer_queries = pr.fold_queries(queries, fp.fold_step)
    for layer in fri["inner"]:
        inner.append(pr.FriLayerDecommit(reads, layer["eval"], layer["tree"], layer_queries, layer["fold_step"], ops))
        layer_queries = pr.fold_queries(layer_queries, layer["fold_step"])
    trees = [(t.merkle, t.evals) for t in scheme.trees] + [(comp_tree, comp_evals)]
    decommits = [pr.MerkleDecommit(reads, m, queries, cols, ops) if cols else None for m, cols in trees]
    reads.run(ops)

    proof = pr.StarkProof(config=cfg)
    proof.fri_first_layer = first.result()
    proof.fri_inner_layers = [d.result() for d in inner]
    proof.fri_last_layer_poly = fri["last_poly"]
    proof.fri_proof_of_work = fri_pow
    proof.commitments = [t.root for t in scheme.trees] + [comp_tree.root]
    proof.oods_proof_of_work = oods_pow
    proof.sampled_values = sampled
    for d in decommits:
        qv, wit = d.result() if d is not None else ([], [])
        proof.queried_values.append(qv)
        proof.decommitments.append(wit)
    proof.claimed_sums = [c.claimed_sum for c in components]

    # --- sanity check (mod.rs:121-132): the composition's OODS value against the constraints
    comp_s = sampled[-1]
    left_v = pr.from_partial_evals([comp_s[k][0] for k in range(4)])
    right_v = pr.from_partial_evals([comp_s[k][0] for k in range(4, 8)])
    x = oods[0]
    for _ in range(mldb - 1):
        x = pr.q_double_x(x)
    composition_oods = qm_add(left_v, qm_mul(x, right_v))
    den_inv = qm_inv(x)  # 1 / V(CanonicCoset(mldb)) at the point
    acc = qm(0)
    for comp in components:
        for c in constraints_at_point(comp.air, comp.mask_values(sampled), comp.params):
            acc = qm_add(qm_mul(acc, random_coeff), qm_mul(den_inv, c))
    proof.constraints_satisfied = composition_oods == acc
    if check and not proof.constraints_satisfied:
        raise ConstraintsNotSatisfied("Constraints not satisfied.")
    return proof


def logup_interaction(ops, air: Air, trace, log_size: int, params) -> tuple:
    """The interaction columns of an AIR's LogUp relations from its trace columns on the trace
    domain, as the reference's LogupTraceGenerator writes them (crates/constraint-framework/src/
    prover/logup.rs:22-130): per batch of finalize_logup_batched its combined fraction at every row
    (from the AIR's fraction kernel), added to the previous batch's column; the last column turned
    into the shifted running sum. params: the relation's parameters (`{relation}_z`,
    `{relation}_alpha{i}`). Returns (4 coordinate columns per batch, in interaction order, and the
    claimed sum)."""
    if not air.logup:
        raise ValueError(f"{air.name} has no LogUp relation")
    gen = ops.logup_generator(log_size)
    for num, den in ops.air_fractions(air, {1: list(trace)}, log_size, params):
        gen.col_from_fractions([(num, den)])
    return gen.finalize_last()


def _param_kind(air: Air, name: str) -> int:
    """cs_air_component's parameter kinds: 0 a given value, 1 a relation's z, 2 the shift, 3 + i
    a relation's alpha^i (every relation uses the one lookup-element draw of the proof)."""
    if name == "shift":
        return 2
    for rel in air.relations:
        if name == f"{rel}_z":
            return 1
        if name.startswith(f"{rel}_alpha") and name[len(rel) + 6:].isdigit():
            return 3 + int(name[len(rel) + 6:])
    return 0


def prove_native(components, trace, config: PcsConfig, twiddles, plain: bool = False,
                 mix_claimed: bool = False) -> bytes:
    """The same proof in native code (cs_prove_air): the empty preprocessed tree, `trace` (device
    columns on their trace domains, every component's in allocation order) as the trace tree; when
    components have LogUp relations, the lookup elements (z, alpha) drawn, the interaction tree of
    their columns generated from their fraction kernels (the claimed sums mixed first with
    mix_claimed), then prove() with the relations' parameters filled from the draw and the shift
    from each claimed sum. The trace columns of components without relations are interpolated in
    place (consumed). Constraint log degree 1 or 2 (degree 2 without the sanity check, as in the
    reference's lifted protocol), any log blowup up to 16 (the evaluation mode inferred as
    evaluation_mode does), any fold_step up to 8. Returns the proof bytes, equal to prove()'s for
    the same flow."""
    from .backend import CudaBackend
    from .framework import CompiledAir
    fp = config.fri_params
    specs, col = [], 0
    for c in components:
        if c.constraint_log_degree not in (1, 2):
            raise NotImplementedError("the native prover: constraint log degree 1 or 2")
        nodes, cons, offs, masks, inter_two = c.air.point_program()
        if c.trace_locations.get(1, (col, col))[0] != col:
            raise ValueError("components' trace columns must follow one another in component order")
        col += len(offs)
        kinds = [_param_kind(c.air, p) for p in c.air.params]
        params = [c.params[p] if k == 0 else (0, 0, 0, 0) for p, k in zip(c.air.params, kinds)]
        specs.append({"kernel": CompiledAir.get(c.air).handle, "log_size": c.log_size,
                      "degree": c.constraint_log_degree, "offsets": offs, "masks": masks, "nodes": nodes,
                      "constraints": cons, "params": params, "kinds": kinds, "n_batches": len(c.air.logup),
                      "frac_cols": [m.column for m in c.air.fraction_masks], "inter_two": inter_two})
    return CudaBackend.prove_air_native(specs, trace, config.trace_lifting_log_size,
                                        (fp.pow_bits, fp.log_blowup_factor, fp.log_last_layer_degree_bound,
                                         fp.n_queries, fp.fold_step), twiddles, plain, mix_claimed)


__all__ = ["TraceLocationAllocator", "FrameworkComponent", "CommitmentSchemeProver", "prove",
           "constraints_at_point", "point_at_offset", "evaluation_mode", "prove_native",
           "logup_interaction"]
