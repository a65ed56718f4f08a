"""The commit-stage workload at its full size (256 columns x 2^20 rows, blowup
4, Merkle height 22) on the GPU against the oracle: same extended evaluations
(sampled rows) and the same Merkle root; plus the size-independent property
that interpolating the extension returns the zero-padded coefficients."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import oracle as O  # noqa: E402
from proving_gb300.synthetic import m31_columns  # noqa: E402

N_COLS, LOG_ROWS, LOG_EXT = 256, 20, 22


@pytest.fixture(scope="module")
def run():
    from proving_gb300 import build
    build.build()
    from proving_gb300.backend import BaseColumn, CudaBackend as B, canonic_half_coset
    evals = m31_columns(2026, N_COLS, LOG_ROWS)
    tree = B.precompute_twiddles(canonic_half_coset(LOG_EXT + 1))
    cols = [BaseColumn(torch.from_numpy(evals[i].view(np.int32)).cuda()) for i in range(N_COLS)]
    B.interpolate_columns(cols, tree)
    ext = B.evaluate_polynomials(cols, LOG_EXT, tree)
    merkle = B.merkle_commit(ext, LOG_EXT)
    torch.cuda.synchronize()
    return dict(B=B, tree=tree, evals=evals, coeffs=cols, ext=ext, merkle=merkle)


def test_full_size_root_matches_oracle(run):
    tw, itw = O.canonic_twiddles(LOG_EXT + 1)
    coeffs = O.interpolate_batch(list(run["evals"]), itw)
    for i in (0, 77, 255):
        assert np.array_equal(run["coeffs"][i].to_cpu(), coeffs[i])
    ext = O.evaluate_batch(coeffs, [LOG_EXT] * N_COLS, tw)
    rows = np.random.default_rng(0).integers(0, 1 << LOG_EXT, 4096)
    for i in (0, 128, 255):
        assert np.array_equal(run["ext"][i].data[torch.from_numpy(rows).cuda()].cpu().numpy().view(np.uint32),
                              ext[i][rows])
    assert run["merkle"].root() == O.merkle_commit(ext, LOG_EXT)


def test_full_size_extension_round_trip(run):
    # interpolate(evaluate(c)) on the 4x domain is c followed by zeros
    B = run["B"]
    from proving_gb300.backend import BaseColumn
    for i in (3, 200):
        e = BaseColumn(run["ext"][i].data.clone())
        B.interpolate_columns([e], run["tree"])
        back = e.data
        assert torch.equal(back[: 1 << LOG_ROWS], run["coeffs"][i].data)
        assert int(back[1 << LOG_ROWS:].abs().sum().item()) == 0
