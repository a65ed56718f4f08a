"""Oracle checks for the accumulation / sampling / quotient ops, restating the
reference's own CPU tests as properties (CPU only)."""
import numpy as np
import pytest

from oracle import oracle as O
from proving_gb300.synthetic import m31_column, qm31_column, seeded_qm31

P = O.P


def _random_point(seed):
    ch = O.Blake2sChannel()
    ch.mix_u64(seed)
    return O.random_point_from_t(ch.draw_secure_felt())


def test_random_point_on_circle():
    x, y = _random_point(1)
    # x^2 + y^2 = 1
    s = [(a + b) % P for a, b in zip(O.qm31_mul(x, x), O.qm31_mul(y, y))]
    assert s == [1, 0, 0, 0]


@pytest.mark.parametrize("log_n", [2, 5, 9])
def test_barycentric_matches_eval_at_point(log_n):
    # crates/stwo/src/prover/backend/simd/circle.rs:786-870: barycentric value = direct value
    tw, _ = O.canonic_twiddles(log_n)
    coeffs = m31_column(log_n, log_n)
    ev = O.evaluate(coeffs, log_n, tw)
    x, y = _random_point(log_n)
    w = O.barycentric_weights(log_n, x, y)
    assert list(O.barycentric_eval(ev, w)) == list(O.eval_at_point(coeffs, x, y))


def test_lift_and_accumulate_matches_naive():
    cols = [qm31_column(s, l) for s, l in [(1, 2), (2, 4), (3, 7)]]
    got = O.lift_and_accumulate(cols)
    want = [np.zeros(1 << 7, np.int64) for _ in range(4)]
    for col in cols:
        l = col[0].size.bit_length() - 1
        i = np.arange(1 << 7)
        idx = ((i >> (7 - l + 1)) << 1) + (i & 1)
        for k in range(4):
            want[k] = (want[k] + col[k][idx].astype(np.int64)) % P
    for k in range(4):
        assert np.array_equal(got[k], want[k].astype(np.uint32))


def test_secure_powers():
    f = seeded_qm31(3)
    pw = O.generate_secure_powers(f, 5)
    acc = np.array([1, 0, 0, 0], np.uint32)
    for k in range(5):
        assert list(pw[k]) == list(acc)
        acc = O.qm31_mul(acc, f)


def test_decompose_of_fft_space_poly_is_exact():
    # crates/stwo/src/prover/backend/simd/fri.rs:315-389 decompose: a polynomial in the
    # FFT space has lambda = 0 and g = f.
    log_n = 6
    tw, _ = O.canonic_twiddles(log_n)
    coords = [O.evaluate(m31_column(40 + k, log_n - 1), log_n, tw) for k in range(4)]
    g, lam = O.decompose(coords)
    assert list(lam) == [0, 0, 0, 0]
    for a, b in zip(g, coords):
        assert np.array_equal(a, b)


def test_line_coeffs_vanish_on_sample():
    # c * value - (a * y + b) = 0 at the sample point itself (constraints.rs:119-135)
    x, y = _random_point(9)
    v = seeded_qm31(4)
    alpha = seeded_qm31(5)
    a, b, c = O.line_coeffs(y, v, alpha)
    lhs = O.qm31_mul(c, v)
    rhs = [(p + q) % P for p, q in zip(O.qm31_mul(a, y), b)]
    assert list(lhs) == rhs


def test_extract_subdomain_twiddles_matches_direct():
    # crates/stwo/src/prover/poly/twiddles.rs:85-107
    committed, sub = 6, 4
    tw, _ = O.canonic_twiddles(committed)
    extracted = O.extract_subdomain_twiddles(tw, committed, sub)
    init = O.canonic_half_coset_initial_index(committed)
    direct, _ = O.precompute_twiddles(init, sub - 1)
    assert np.array_equal(extracted[:-1], direct[:-1])


def test_logup_running_sum_ends_at_zero_and_steps_by_fractions():
    # the shifted running sum ends at 0 and its coset-order differences are the
    # fractions minus claimed/n (crates/constraint-framework/src/prover/logup.rs:96-130)
    log_n, n = 6, 64
    v = m31_column(5, log_n)
    z = seeded_qm31(6)
    out, claimed = O.logup_running_sum(v, z)
    br = O.bit_reverse(np.arange(n))
    pos = [int(br[(k // 2) if k % 2 == 0 else n // 2 + (n - 1 - k) // 2]) for k in range(n)]
    assert [int(o[pos[-1]]) for o in out] == [0, 0, 0, 0]
    shift = O.qm31_mul(claimed, [pow(n, P - 2, P), 0, 0, 0])
    for k in range(1, n):
        cur = np.array([o[pos[k]] for o in out], np.int64)
        prev = np.array([o[pos[k - 1]] for o in out], np.int64)
        frac = O.qm31_inv([(int(z[0]) - int(v[pos[k]])) % P, z[1], z[2], z[3]])
        want = (frac.astype(np.int64) - shift.astype(np.int64)) % P
        assert list((cur - prev) % P) == list(want)
