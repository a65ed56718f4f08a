"""GPU parity at sizes beyond the benchmark's 2^22: FFT pass plans of 25-28 layers, a 2^26-leaf
tree whose layer buffer passes 4 GiB (64-bit byte offsets), 26 folds of a 2^26 layer in one call,
a 2^24-row LogUp running sum. Inputs come from numpy's seeded generator (uniform in [0, P)); results
are compared with the oracle where it finishes in seconds, and the 2^28 evaluation through its
interpolation round trip."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import oracle as O  # noqa: E402
from proving_gb300.synthetic import seeded_qm31  # noqa: E402

P = O.P


@pytest.fixture(scope="module")
def B():
    from proving_gb300 import build
    build.build()
    from proving_gb300.backend import CudaBackend
    return CudaBackend


def _rand(seed, n):
    return np.random.default_rng(seed).integers(0, P, n, dtype=np.uint32)


def _tree(B, domain_log):
    from proving_gb300.backend import canonic_half_coset
    return B.precompute_twiddles(canonic_half_coset(domain_log))


def _col(values):
    from proving_gb300.backend import BaseColumn
    return BaseColumn.from_cpu(values)


def test_evaluate_2e24_on_2e26_matches_oracle(B):
    tree = _tree(B, 27)
    tw, _ = O.canonic_twiddles(27)
    c = _rand(1, 1 << 24)
    out = B.evaluate_polynomials([_col(c)], 26, tree)
    assert np.array_equal(out[0].to_cpu(), O.evaluate(c, 26, tw))


def test_fft_round_trip_at_2e28(B):
    # 2^26 coefficients evaluated on 2^28 points (1 GiB) and interpolated back: the coefficients,
    # then zeros
    from proving_gb300.backend import BaseColumn
    tree = _tree(B, 29)
    g = torch.Generator(device="cuda")
    g.manual_seed(2028)
    c = torch.randint(0, P, (1 << 26,), generator=g, device="cuda", dtype=torch.int64).to(torch.int32)
    ext = B.evaluate_polynomials([BaseColumn(c)], 28, tree)
    back = B.interpolate_columns_into(ext, tree)
    del ext
    assert torch.equal(back[0].data[: 1 << 26], c)
    assert not back[0].data[1 << 26:].any()


def test_merkle_height_26_matches_oracle(B):
    col = _rand(3, 1 << 26)
    tree = B.merkle_commit([_col(col)], 26)
    assert tree.root() == O.merkle_commit([col], 26)


def test_fold_line_26_challenges_at_2e26_matches_oracle(B):
    from proving_gb300.backend import SecureColumnByCoords
    log_n = 26
    tree = _tree(B, log_n + 1)
    coords = [_rand(10 + k, 1 << log_n) for k in range(4)]
    alphas = [seeded_qm31(3000 + j) for j in range(log_n)]
    got = B.fold_line(SecureColumnByCoords.from_cpu(coords), alphas, tree).to_cpu()
    w, init = coords, O.line_domain_initial_index(log_n)
    for a in alphas:
        w = O.fold_line(w, init, a)
        init = O.double_index(init)
    assert all(np.array_equal(a, b) for a, b in zip(got, w))


def test_logup_running_sum_at_2e24_matches_oracle(B):
    v, z = _rand(4, 1 << 24), seeded_qm31(5)
    got, claimed = B.logup_running_sum(_col(v), z)
    want, want_claimed = O.logup_running_sum(v, z)
    assert list(claimed) == list(want_claimed)
    assert all(np.array_equal(a, b) for a, b in zip(got.to_cpu(), want))
