"""Oracle checks for the Poseidon2 AIR (crates/examples/src/poseidon/mod.rs),
restating the reference's own tests of it (CPU only)."""
import numpy as np
import pytest

from oracle import oracle as O

P = O.P

# PoseidonElements::dummy() (crates/constraint-framework/src/logup.rs:95-105)
DUMMY_Z = [1, 2, 3, 4]
DUMMY_ALPHA = [4, 3, 2, 1]


def test_apply_m4():
    # test_apply_m4 (mod.rs:411-425): apply_m4 is the product with this matrix
    m4 = np.array([[5, 7, 1, 3], [4, 6, 1, 1], [1, 3, 5, 7], [1, 1, 4, 6]], np.int64)
    state = np.array([0, 1, 2, 3], np.int64)
    assert list(O.poseidon_m4(state)) == list((m4 @ state) % P)


def test_apply_internal():
    # test_apply_internal (mod.rs:427-441): all-ones matrix plus 2^(i+1) on the diagonal
    state = np.array([i * 3 + 187 for i in range(16)], np.int64)
    mat = np.ones((16, 16), np.int64) + np.diag([1 << (i + 1) for i in range(16)])
    assert list(O.poseidon_internal(state)) == list((mat @ state) % P)


def test_external_is_circulant_of_m4():
    # circ(2 M4, M4, M4, M4) (mod.rs:91-113)
    m4 = np.array([[5, 7, 1, 3], [4, 6, 1, 1], [1, 3, 5, 7], [1, 1, 4, 6]], np.int64)
    big = np.block([[2 * m4 if i == j else m4 for j in range(4)] for i in range(4)])
    state = np.arange(100, 116, dtype=np.int64)
    assert list(O.poseidon_external(state)) == list((big @ state) % P)


def test_trace_layout():
    log_n = 5
    cols = O.poseidon_trace(log_n)
    assert len(cols) == 1264
    r = np.arange(1 << log_n)
    for k in range(8):
        for i in range(16):
            # gen_trace's inputs: row r, instance k, state word i -> r + i + k (mod.rs:215-219)
            assert np.array_equal(cols[158 * k + i], (r + i + k).astype(np.uint32))


def _rc(n, seed=3):
    return np.random.default_rng(seed).integers(0, P, (n, 4)).astype(np.uint32)


@pytest.mark.parametrize("log_n", [4, 8])
def test_constraints_vanish_on_the_trace_domain(log_n):
    # test_poseidon_constraints (mod.rs:443-464): every constraint is zero on every row of the
    # trace domain; with random weights the weighted row sums are all zero
    trace = O.poseidon_trace(log_n)
    inter, claimed = O.poseidon_interaction(trace, DUMMY_Z, DUMMY_ALPHA)
    out = O.poseidon_composition(trace, inter, log_n, DUMMY_Z + DUMMY_ALPHA, claimed, _rc(O.POSEIDON_CONSTRAINTS))
    assert all(not o.any() for o in out)


@pytest.mark.parametrize("col", [0, 17, 158 * 3 + 90, 1263])
def test_tampered_trace_violates_a_constraint(col):
    log_n = 4
    trace = O.poseidon_trace(log_n)
    inter, claimed = O.poseidon_interaction(trace, DUMMY_Z, DUMMY_ALPHA)
    trace[col] = trace[col].copy()
    trace[col][5] = (int(trace[col][5]) + 1) % P
    out = O.poseidon_composition(trace, inter, log_n, DUMMY_Z + DUMMY_ALPHA, claimed, _rc(O.POSEIDON_CONSTRAINTS))
    assert any(o.any() for o in out)


def test_interaction_running_sum_ends_at_zero():
    log_n = 6
    n = 1 << log_n
    trace = O.poseidon_trace(log_n)
    inter, claimed = O.poseidon_interaction(trace, DUMMY_Z, DUMMY_ALPHA)
    br = O.bit_reverse(np.arange(n))
    last_coset = int(br[n // 2])  # coset index n - 1 lives at circle-domain index n / 2
    assert [int(inter[28 + c][last_coset]) for c in range(4)] == [0, 0, 0, 0]
    assert any(int(x) for x in claimed)
