"""The Poseidon2 prover restatement on the CPU oracle backend.

The reference's own prove test for this AIR is ignored upstream (the lifted
protocol does not support constraint degree >= 2): its prove_ex sanity check
fails. These tests pin the pieces that decide that outcome: the point
evaluation of the constraints agrees with the domain evaluation when nothing
is lifted, and with poseidon_pcs_config the check fails exactly as the
reference's does."""
import numpy as np
import pytest

from oracle import oracle as O
from cpu_backend import CpuOps
from proving_gb300 import poseidon as ps
from proving_gb300 import prover as pr
from proving_gb300.synthetic import seeded_qm31

P = O.P


def _point(seed):
    ch = pr.Blake2sChannel()
    ch.mix_u64(seed)
    return pr.random_point(ch.draw_secure_felt())


@pytest.mark.parametrize("log_n", [4, 5])
def test_point_evaluation_matches_the_composition_polynomial(log_n):
    # Q = interpolate(sum_k rc_k C_k / V_trace) on CanonicCoset(n + 2); at a random point q the
    # constraints evaluated from the trace polynomials at q and q - G_n give Q(q)
    eval_log = log_n + ps.LOG_EXPAND
    lookup = [int(x) for x in seeded_qm31(31)] + [int(x) for x in seeded_qm31(32)]
    random_coeff = tuple(int(x) for x in seeded_qm31(33))
    trace = O.poseidon_trace(log_n)
    inter, claimed = O.poseidon_interaction(trace, lookup[:4], lookup[4:])
    tw, itw = O.canonic_twiddles(eval_log)
    t_coeffs = [O.interpolate(c, itw) for c in trace]
    i_coeffs = [O.interpolate(c, itw) for c in inter]
    t_eval = [O.evaluate(c, eval_log, tw) for c in t_coeffs]
    i_eval = [O.evaluate(c, eval_log, tw) for c in i_coeffs]
    rc = np.asarray(list(reversed(pr.secure_powers(random_coeff, ps.N_CONSTRAINTS))), np.uint32)
    accum = O.poseidon_composition(t_eval, i_eval, log_n, lookup, claimed, rc)
    q_coeffs = [O.interpolate(a, itw) for a in accum]

    q = _point(log_n)
    g = pr.m31_subgroup_generator(log_n)
    q_prev = pr.qpoint_add_m31(q, (g[0], (-g[1]) % P))

    def at(coeffs, pt):
        return tuple(int(v) for v in O.eval_at_point(coeffs, pt[0], pt[1]))

    trace_mask = [at(c, q) for c in t_coeffs]
    inter_mask = [[at(c, q)] for c in i_coeffs[:28]] + [[at(c, q_prev), at(c, q)] for c in i_coeffs[28:]]
    expected = ps.composition_at_point(q, trace_mask, inter_mask, lookup, claimed, random_coeff, log_n, log_n)
    got = pr.from_partial_evals([at(c, q) for c in q_coeffs])
    assert got == expected


def _prove(log_n, check=False):
    ops = CpuOps()
    fp = pr.FriParams(pow_bits=10, log_blowup_factor=1, log_last_layer_degree_bound=0, n_queries=70, fold_step=1)
    cfg = ps.poseidon_pcs_config(log_n + 3, fp)
    tw = ops.twiddles(log_n + ps.LOG_EXPAND + fp.log_blowup_factor)
    return ps.prove_poseidon(ops, log_n, cfg, pr.Blake2sChannel(), tw, check=check)


def test_lifted_config_fails_the_sanity_check_like_the_reference():
    # prove_poseidon with poseidon_pcs_config: ProvingError::ConstraintsNotSatisfied
    with pytest.raises(ps.ConstraintsNotSatisfied):
        _prove(4, check=True)


def test_proof_words_are_deterministic_and_well_formed():
    a, b = _prove(4), _prove(4)
    assert a.to_bytes() == b.to_bytes()
    assert len(a.commitments) == 4 and len(a.sampled_values) == 4
    # 1264 trace columns, 32 interaction columns (the last four with two samples), 8 composition
    assert len(a.sampled_values[1]) == 1264 and len(a.sampled_values[2]) == 32
    assert [len(c) for c in a.sampled_values[2][27:]] == [1, 2, 2, 2, 2]
    assert len(a.queried_values[1]) == 1264 and len(a.queried_values[3]) == 8
