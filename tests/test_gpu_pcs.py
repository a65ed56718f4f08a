"""GPU parity for accumulation, out-of-domain sampling, DEEP quotients and
decompose, through the C ABI, against the oracle (raw u32 words)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import oracle as O  # noqa: E402
from proving_gb300.synthetic import m31_column, m31_columns, qm31_column, seeded_qm31  # noqa: E402


@pytest.fixture(scope="module")
def B():
    from proving_gb300 import build
    build.build()
    from proving_gb300.backend import CudaBackend
    return CudaBackend


def _sc(coords):
    from proving_gb300.backend import SecureColumnByCoords
    return SecureColumnByCoords.from_cpu(coords)


def _col(v):
    from proving_gb300.backend import BaseColumn
    return BaseColumn.from_cpu(v)


def _tree(B, log):
    from proving_gb300.backend import canonic_half_coset
    return B.precompute_twiddles(canonic_half_coset(log))


def _point(seed):
    ch = O.Blake2sChannel()
    ch.mix_u64(seed)
    return O.random_point_from_t(ch.draw_secure_felt())


def _eq(got_sc, want):
    return all(np.array_equal(g, w) for g, w in zip(got_sc.to_cpu(), want))


def test_accumulate(B):
    a, b = qm31_column(1, 10), qm31_column(2, 10)
    col = _sc(a)
    B.accumulate(col, _sc(b))
    assert _eq(col, O.accumulate(a, b))


def test_secure_powers(B):
    f = seeded_qm31(8)
    assert np.array_equal(B.generate_secure_powers(f, 9), O.generate_secure_powers(f, 9))


@pytest.mark.parametrize("logs", [[5], [1, 3], [2, 4, 9, 12]])
def test_lift_and_accumulate(B, logs):
    cols = [qm31_column(10 + i, l) for i, l in enumerate(logs)]
    got = B.lift_and_accumulate([_sc(c) for c in cols])
    assert _eq(got, O.lift_and_accumulate(cols))


@pytest.mark.parametrize("log_n", [1, 3, 8, 15, 18])
def test_barycentric_weights_and_eval(B, log_n):
    x, y = _point(log_n)
    w = B.barycentric_weights(log_n, (x, y))
    want_w = O.barycentric_weights(log_n, x, y)
    assert _eq(w, want_w)
    cols = m31_columns(log_n, 5, log_n)
    got = B.barycentric_eval_at_point([_col(c) for c in cols], w).cpu().numpy().view(np.uint32)
    for i in range(5):
        assert list(got[i]) == list(O.barycentric_eval(cols[i], want_w))


@pytest.mark.parametrize("log_n", [0, 1, 5, 8, 9, 14, 20])
def test_eval_at_point(B, log_n):
    x, y = _point(100 + log_n)
    cols = m31_columns(log_n + 3, 3, log_n)
    got = B.eval_at_point([_col(c) for c in cols], (x, y)).cpu().numpy().view(np.uint32)
    for i in range(3):
        assert list(got[i]) == list(O.eval_at_point(cols[i], x, y))


@pytest.mark.parametrize("n_terms,log_n,blowup", [(1, 6, 1), (7, 10, 1), (108, 15, 1), (600, 12, 2)])
def test_accumulate_numerators(B, n_terms, log_n, blowup):
    cols = m31_columns(n_terms, n_terms, log_n)
    x, y = _point(n_terms)
    coeffs = np.stack([O.line_coeffs(y, seeded_qm31(t), seeded_qm31(1000 + t)) for t in range(n_terms)])
    got, fl = B.accumulate_numerators([_col(c) for c in cols], coeffs, blowup)
    want, wfl = O.accumulate_numerators(list(cols), blowup, coeffs)
    assert _eq(got, want)
    assert list(fl) == list(wfl)


@pytest.mark.parametrize("L,b,acc_logs", [(8, 1, [7]), (12, 1, [5, 11]), (15, 2, [13, 9, 13])])
def test_quotients_and_combine(B, L, b, acc_logs):
    accs = [qm31_column(20 + i, l) for i, l in enumerate(acc_logs)]
    pts = [_point(50 + i) for i in range(len(acc_logs))]
    fls = [seeded_qm31(60 + i) for i in range(len(acc_logs))]
    got_sub = B.quotients_on_subdomain([_sc(a) for a in accs], pts, fls, L, b)
    want_sub = O.quotients_on_subdomain(accs, pts, fls, L, b)
    assert _eq(got_sub, want_sub)
    # combine: interpolate on the subdomain (extracted twiddles), evaluate on CanonicCoset(L)
    tree = _tree(B, L + 1)
    tw, itw = O.canonic_twiddles(L + 1)
    got = B.compute_quotients_and_combine([_sc(a) for a in accs], pts, fls, L, b, tree)
    sub_itw = O.extract_subdomain_twiddles(itw, L, L - b)
    want = [O.evaluate(O.interpolate(c, sub_itw), L, tw) for c in want_sub]
    assert _eq(got, want)


@pytest.mark.parametrize("log_n", [1, 4, 13])
def test_decompose(B, log_n):
    coords = qm31_column(7, log_n)
    g, lam = B.decompose(_sc(coords))
    wg, wl = O.decompose(coords)
    assert list(lam) == list(wl)
    assert _eq(g, wg)


def test_interpolate_on_subdomain_small_sizes(B):
    # subdomains of log 1..3 of CanonicCoset(8) against the oracle with extracted twiddles
    tree = _tree(B, 9)
    _, itw = O.canonic_twiddles(9)
    for sub in (3, 5):
        v = m31_column(sub, sub)
        c = _col(v)
        B.interpolate_on_subdomain([c], 8, tree)
        assert np.array_equal(c.to_cpu(), O.interpolate(v, O.extract_subdomain_twiddles(itw, 8, sub)))
