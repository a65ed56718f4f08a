"""GPU parity: every CUDA op, called through the C ABI, against the CPU oracle
on the same seeded inputs. All values are compared as raw u32 words (the
reference hashes raw words, so canonical representatives must match too)."""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import oracle as O  # noqa: E402
from proving_gb300.synthetic import m31_column, m31_columns, qm31_column, seeded_qm31  # noqa: E402

KATS = json.loads((Path(__file__).parent / "golden" / "reference_kats.json").read_text())


@pytest.fixture(scope="module")
def B():
    from proving_gb300 import build
    build.build()
    from proving_gb300.backend import CudaBackend
    assert torch.cuda.is_available()
    return CudaBackend


def _tree(B, domain_log):
    from proving_gb300.backend import canonic_half_coset
    return B.precompute_twiddles(canonic_half_coset(domain_log))


def _col(values):
    from proving_gb300.backend import BaseColumn
    return BaseColumn.from_cpu(values)


# ------------------------------------------------------------------ twiddles

@pytest.mark.parametrize("domain_log", [2, 3, 8, 13, 20, 23])
def test_twiddles_match_oracle(B, domain_log):
    t = _tree(B, domain_log)
    tw, itw = O.canonic_twiddles(domain_log)
    assert np.array_equal(t.twiddles.cpu().numpy().view(np.uint32), tw)
    assert np.array_equal(t.itwiddles.cpu().numpy().view(np.uint32), itw)


@pytest.mark.parametrize("log_n", [1, 3, 10, 17])
def test_bit_reverse(B, log_n):
    v = m31_column(9, log_n)
    c = _col(v)
    B.bit_reverse_column(c)
    assert np.array_equal(c.to_cpu(), O.bit_reverse(v))


# ------------------------------------------------------------------ FFT

@pytest.mark.parametrize("log_n", list(range(1, 15)) + [16, 19, 20, 22])
def test_interpolate_matches_oracle(B, log_n):
    tree = _tree(B, log_n + 1)
    _, itw = O.canonic_twiddles(log_n + 1)
    cols_np = m31_columns(log_n, 3, log_n)
    cols = [_col(c) for c in cols_np]
    B.interpolate_columns(cols, tree)
    want = O.interpolate_batch(list(cols_np), itw)
    for c, w in zip(cols, want):
        assert np.array_equal(c.to_cpu(), w)


@pytest.mark.parametrize("log_c,log_n", [(0, 3), (1, 1), (1, 2), (2, 2), (2, 5), (3, 3), (3, 4), (5, 7), (8, 10),
                                         (11, 12), (12, 14), (13, 13), (14, 15), (16, 18), (18, 20), (20, 22),
                                         (20, 20), (21, 22)])
def test_evaluate_matches_oracle(B, log_c, log_n):
    tree = _tree(B, log_n + 1)
    tw, _ = O.canonic_twiddles(log_n + 1)
    coeffs_np = m31_columns(100 + log_c, 2, log_c)
    coeffs = [_col(c) for c in coeffs_np]
    out = B.evaluate_polynomials(coeffs, log_n, tree)
    want = O.evaluate_batch(list(coeffs_np), [log_n] * 2, tw)
    for o, w in zip(out, want):
        assert np.array_equal(o.to_cpu(), w)


@pytest.mark.parametrize("logs", [[1, 2, 3, 4, 5, 10, 12, 13, 16, 17, 20, 22], [7] * 5 + [9] * 3 + [3] * 7, [14]])
def test_mixed_size_interpolate_and_evaluate(B, logs):
    # cs_interpolate_columns_multi / cs_evaluate_columns_multi: every size of a mixed batch in one call
    # (size groups on side streams joined back into the caller's stream), out of place and in place
    from proving_gb300 import _lib
    from proving_gb300.backend import _ptr_table, _stream, _u32_table
    top = max(logs) + 1
    tree = _tree(B, top + 1)
    tw, itw = O.canonic_twiddles(top + 1)
    evals_np = [m31_column(700 + i, l) for i, l in enumerate(logs)]
    src = [_col(e) for e in evals_np]
    coeffs = [_col(np.zeros(1 << l, np.uint32)) for l in logs]
    _lib.call("cs_interpolate_columns_multi", _ptr_table([c.data for c in src]), _ptr_table([c.data for c in coeffs]),
              _u32_table(logs), len(logs), tree.itwiddles.data_ptr(), tree.log_size, _stream())
    inplace = [_col(e) for e in evals_np]
    _lib.call("cs_interpolate_columns_multi", _ptr_table([c.data for c in inplace]),
              _ptr_table([c.data for c in inplace]), _u32_table(logs), len(logs), tree.itwiddles.data_ptr(),
              tree.log_size, _stream())
    want_c = O.interpolate_batch(evals_np, itw)
    for c, ip, w, e in zip(coeffs, inplace, want_c, src):
        assert np.array_equal(c.to_cpu(), w) and np.array_equal(ip.to_cpu(), w)
    assert all(np.array_equal(e.to_cpu(), v) for e, v in zip(src, evals_np))  # out of place: sources kept
    ext = [_col(np.zeros(1 << (l + 1), np.uint32)) for l in logs]
    _lib.call("cs_evaluate_columns_multi", _ptr_table([c.data for c in coeffs]), _ptr_table([c.data for c in ext]),
              _u32_table(logs), 1, len(logs), tree.twiddles.data_ptr(), tree.log_size, _stream())
    want_e = O.evaluate_batch(want_c, [l + 1 for l in logs], tw)
    for x, w in zip(ext, want_e):
        assert np.array_equal(x.to_cpu(), w)


def test_twiddle_tree_larger_than_domain(B):
    # A tree for a bigger root coset serves every smaller canonic domain.
    tree = _tree(B, 16)
    _, itw = O.canonic_twiddles(16)
    v = m31_column(3, 11)
    c = _col(v)
    B.interpolate_columns([c], tree)
    assert np.array_equal(c.to_cpu(), O.interpolate(v, itw))


def test_batch_over_256_columns(B):
    # more columns than one launch's pointer table
    tree = _tree(B, 9)
    _, itw = O.canonic_twiddles(9)
    cols_np = m31_columns(5, 300, 8)
    cols = [_col(c) for c in cols_np]
    B.interpolate_columns(cols, tree)
    want = O.interpolate_batch(list(cols_np), itw)
    assert all(np.array_equal(c.to_cpu(), w) for c, w in zip(cols, want))


# ------------------------------------------------------------------ Merkle

def _digests(t):
    from proving_gb300.backend import digests_to_bytes
    return digests_to_bytes(t)


def test_merkle_leaves_kat(B):
    k = KATS["lifted_merkle_leaves"]
    cols = [_col(np.arange(1 << l, dtype=np.uint32)) for l in k["column_log_sizes"]]
    leaves = _digests(B.build_leaves(cols, k["lifting_log_size"]))
    for idx, hexd in k["leaves"].items():
        assert leaves[int(idx)].tobytes().hex() == hexd


@pytest.mark.parametrize("log_sizes,L", [([4], 4), ([3, 5, 5, 9], 9), ([1, 2], 6), ([6] * 16, 6), ([6] * 17, 6),
                                         ([7] * 33, 10), (list(range(1, 13)) * 3, 14),
                                         # prefix chaining values handed up through several sizes
                                         ([3] * 20 + [5] * 20 + [8] * 40, 9), ([2] * 16 + [4] * 16 + [6] * 16, 6),
                                         ([5] * 10 + [7] * 40, 7), ([1] * 16 + [3] * 15 + [9] * 2, 9),
                                         ([4] * 48 + [6] * 16 + [10] * 17, 11)])
def test_merkle_commit_matches_oracle(B, log_sizes, L):
    cols_np = [m31_column(i * 31 + l, l) for i, l in enumerate(log_sizes)]
    perm = np.random.default_rng(0).permutation(len(cols_np))  # commit sorts (stably) by length
    cols_np = [cols_np[i] for i in perm]
    tree = B.merkle_commit([_col(c) for c in cols_np], L)
    root, layers = O.merkle_commit(cols_np, L, with_layers=True)
    assert tree.root() == root
    for k, want in zip(range(L, -1, -1), layers):
        assert np.array_equal(_digests(tree.layer(k)), want)


def test_merkle_empty(B):
    tree = B.merkle_commit([], 0)
    assert tree.root() == hashlib.blake2s(b"").digest()


@pytest.mark.parametrize("L", [0, 1, 10, 11, 12])
def test_merkle_build_layers_above_caller_leaves(B, L):
    # cs_merkle_build_leaves into a caller-owned layer buffer, then cs_merkle_build_layers on it:
    # L = 11 and 12 take per-layer launches below the single top launch (layers of up to 2^10
    # nodes), L <= 10 the top launch alone, L = 0 an empty tree whose root is the leaf
    from proving_gb300 import _lib
    from proving_gb300.backend import _ptr, _ptr_table, _stream, _u32_table
    logs = [] if L == 0 else sorted([max(1, L - k % 3) for k in range(20)])
    cols_np = [m31_column(300 + i, l) for i, l in enumerate(logs)]
    cols = [_col(c) for c in cols_np]
    layers = torch.empty(((1 << (L + 1)) - 1, 8), dtype=torch.int32, device="cuda")
    _lib.call("cs_merkle_build_leaves", _ptr_table([c.data for c in cols]), _u32_table(logs), len(cols), L,
              _ptr(layers), _stream())
    _lib.call("cs_merkle_build_layers", _ptr(layers), L, _stream())
    torch.cuda.synchronize()
    root, want = O.merkle_commit(cols_np, L, with_layers=True)
    off = 0
    for k, w in zip(range(L, -1, -1), want):
        assert np.array_equal(_digests(layers[off:off + (1 << k)]), w), f"layer {k}"
        off += 1 << k
    assert _digests(layers[-1:]).tobytes() == root


def test_merkle_next_layer(B):
    prev = np.frombuffer(np.random.default_rng(3).bytes(32 * 64), np.uint8).reshape(64, 32)
    t = torch.from_numpy(prev.copy().view(np.int32).reshape(64, 8)).cuda()
    got = _digests(B.build_next_layer(t))
    assert np.array_equal(got, O.merkle_build_next_layer(prev))


def test_pack_leaves_input(B):
    coords = qm31_column(4, 6)
    from proving_gb300.backend import BaseColumn
    outs = B.pack_leaves_input([BaseColumn.from_cpu(c) for c in coords])
    for coord in range(4):
        for off in range(4):
            assert np.array_equal(outs[coord + 4 * off].to_cpu(), coords[coord][off::4])


# ------------------------------------------------------------------ FRI

@pytest.mark.parametrize("log_n", [3, 4, 10, 16, 22])
def test_fold_circle_into_line(B, log_n):
    from proving_gb300.backend import SecureColumnByCoords
    tree = _tree(B, log_n)
    coords = qm31_column(log_n, log_n)
    alpha = seeded_qm31(log_n)
    got = B.fold_circle_into_line(SecureColumnByCoords.from_cpu(coords), alpha, tree).to_cpu()
    want = O.fold_circle_into_line(coords, alpha)
    for g, w in zip(got, want):
        assert np.array_equal(g, w)


@pytest.mark.parametrize("log_n", [1, 2, 5, 12, 21])
def test_fold_line(B, log_n):
    from proving_gb300.backend import SecureColumnByCoords
    tree = _tree(B, log_n + 1)
    coords = qm31_column(50 + log_n, log_n)
    alpha = seeded_qm31(log_n + 7)
    got = B.fold_line(SecureColumnByCoords.from_cpu(coords), [alpha], tree).to_cpu()
    want = O.fold_line(coords, O.line_domain_initial_index(log_n), alpha)
    for g, w in zip(got, want):
        assert np.array_equal(g, w)


def test_fri_fold_chain_22(B):
    # The commit stage's FRI: one QM31 column of log 22, fold_circle_into_line, then 21
    # fold_line steps with seeded challenges, bit-exact at every layer.
    from proving_gb300.backend import SecureColumnByCoords
    log_n = 22
    tree = _tree(B, log_n)
    coords = qm31_column(22, log_n)
    alphas = [seeded_qm31(1000 + k) for k in range(22)]
    g = B.fold_circle_into_line(SecureColumnByCoords.from_cpu(coords), alphas[0], tree)
    w = O.fold_circle_into_line(coords, alphas[0])
    init = O.line_domain_initial_index(log_n - 1)
    for k in range(1, 22):
        g = B.fold_line(g, [alphas[k]], tree)
        w = O.fold_line(w, init, alphas[k])
        init = O.double_index(init)
        if k % 5 == 0 or k == 21:
            assert all(np.array_equal(a, b) for a, b in zip(g.to_cpu(), w))
    assert len(g) == 1


@pytest.fixture(params=[3, 4], ids=["8_per_thread", "16_per_thread"])
def fold_plan(B, request):
    old = B.get_fold_plan()
    B.set_fold_plan(request.param)
    yield request.param
    B.set_fold_plan(old)


@pytest.mark.parametrize("log_n,k", [(1, 1), (3, 3), (4, 2), (4, 4), (5, 5), (8, 8), (9, 4), (9, 9), (10, 10),
                                     (11, 11), (12, 3), (12, 12), (13, 6), (13, 12), (15, 1), (16, 7), (17, 15),
                                     (20, 13), (21, 10), (21, 20), (21, 21)])
def test_fold_line_with_several_alphas(B, fold_plan, log_n, k):
    # FriOps::fold_line with k challenges (launches of up to 11 or 12 folds in registers, shuffles
    # and shared memory, with 8 or 16 values a thread, or of up to 10 folds through shared-memory
    # tiles) equals k single folds of the oracle; only the last layer is returned.
    from proving_gb300.backend import SecureColumnByCoords
    tree = _tree(B, log_n + 1)
    coords = qm31_column(300 + log_n, log_n)
    alphas = [seeded_qm31(2000 + 31 * log_n + j) for j in range(k)]
    got = B.fold_line(SecureColumnByCoords.from_cpu(coords), alphas, tree)
    assert len(got) == 1 << (log_n - k)
    w, init = coords, O.line_domain_initial_index(log_n)
    for a in alphas:
        w = O.fold_line(w, init, a)
        init = O.double_index(init)
    assert all(np.array_equal(a, b) for a, b in zip(got.to_cpu(), w))


def test_fold_line_unaligned_source_takes_scalar_loads(B):
    # coordinates offset by 8 bytes (not 16): the tile kernel stages them with 4-byte loads
    import torch
    from proving_gb300.backend import BaseColumn, SecureColumnByCoords
    log_n = 9
    tree = _tree(B, log_n + 1)
    coords = qm31_column(77, log_n)
    block = torch.zeros((4, (1 << log_n) + 2), dtype=torch.int32, device="cuda")
    for c in range(4):
        block[c, 2:] = torch.from_numpy(np.asarray(coords[c], np.uint32).view(np.int32)).cuda()
    src = SecureColumnByCoords([BaseColumn(block[c, 2:]) for c in range(4)])
    alphas = [seeded_qm31(5000 + j) for j in range(4)]
    got = B.fold_line(src, alphas, tree).to_cpu()
    w, init = coords, O.line_domain_initial_index(log_n)
    for a in alphas:
        w = O.fold_line(w, init, a)
        init = O.double_index(init)
    assert all(np.array_equal(a, b) for a, b in zip(got, w))


# ------------------------------------------------------------------ grind

def test_grind_pow_kat(B):
    k = KATS["verify_pow_nonce"]
    digest = b"".join(int(w).to_bytes(4, "little") for w in k["digest_words"])
    nonce = B.grind(digest, 10)
    assert nonce == O.grind(digest, 10)
    assert nonce <= 649  # 649 passes at 10 bits (blake2s.rs:234)


@pytest.mark.parametrize("bits", [0, 1, 5, 12, 16, 20, 21])
def test_grind_smallest_nonce(B, bits):
    # 20 and 21 bits usually need several launches (the first tries 2^18.2 nonces, each next one
    # twice as many as the one before)
    ch = O.Blake2sChannel()
    ch.mix_u64(0x1111222233334344 + bits)
    assert B.grind(ch.digest, bits) == O.grind(ch.digest, bits)


def test_grind_gives_up(B):
    from proving_gb300._lib import CudaBackendError
    ch = O.Blake2sChannel()
    with pytest.raises(CudaBackendError) as e:
        B.grind(ch.digest, 32, max_nonce=1000)
    assert "TIMEOUT" in str(e.value)


@pytest.mark.parametrize("log_size,n_layers", [(1, 1), (3, 3), (6, 2), (10, 10), (10, 9)])
def test_fri_commit_fold_tail_equals_layer_by_layer(B, log_size, n_layers):
    # cs_fri_commit_fold_tail writes the trees, challenges, folded layers and channel state that
    # cs_merkle_commit, cs_channel_mix_root, cs_channel_draw_secure_felt and cs_fold_line_device_alpha
    # write layer by layer (FriProver::commit's loop, fri.rs:113-207); the folds also equal the oracle's
    import ctypes
    from proving_gb300 import _lib
    from proving_gb300.backend import _stream
    tree = _tree(B, log_size + 1)
    itw, tw_log = tree.itwiddles.data_ptr(), tree.log_size
    layer0 = np.stack([np.asarray(c, np.uint32) for c in qm31_column(800 + log_size, log_size)])
    rng = np.random.default_rng(log_size)
    state0 = np.concatenate([rng.integers(0, 1 << 32, 8, dtype=np.uint64).astype(np.uint32), [7]]).astype(np.uint32)
    vp = ctypes.c_void_p

    def buffers():
        evals = [torch.tensor(layer0.view(np.int32), device="cuda")]
        evals += [torch.zeros((4, 1 << (log_size - j - 1)), dtype=torch.int32, device="cuda") for j in range(n_layers)]
        trees = [torch.zeros(((2 << (log_size - j)) - 1) * 8, dtype=torch.int32, device="cuda") for j in range(n_layers)]
        state = torch.tensor(state0.view(np.int32), device="cuda")
        alphas = torch.zeros(4 * n_layers, dtype=torch.int32, device="cuda")
        return evals, trees, state, alphas

    def tab(t):
        return (vp * 4)(*[t[k].data_ptr() for k in range(4)])

    ev_a, tr_a, st_a, al_a = buffers()
    for j in range(n_layers):
        m = log_size - j
        logs = (ctypes.c_uint32 * 4)(*([m] * 4))
        _lib.call("cs_merkle_commit", tab(ev_a[j]), logs, 4, m, tr_a[j].data_ptr(), _stream())
        _lib.call("cs_channel_mix_root", st_a.data_ptr(), tr_a[j].data_ptr() + 4 * (tr_a[j].numel() - 8), _stream())
        _lib.call("cs_channel_draw_secure_felt", st_a.data_ptr(), al_a.data_ptr() + 16 * j, _stream())
        _lib.call("cs_fold_line_device_alpha", tab(ev_a[j]), m, al_a.data_ptr() + 16 * j, tab(ev_a[j + 1]), itw, tw_log,
                  _stream())
    ev_b, tr_b, st_b, al_b = buffers()
    ev_tab = (vp * (4 * (n_layers + 1)))(*[e[k].data_ptr() for e in ev_b for k in range(4)])
    tr_tab = (vp * n_layers)(*[t.data_ptr() for t in tr_b])
    _lib.call("cs_fri_commit_fold_tail", st_b.data_ptr(), al_b.data_ptr(), ev_tab, tr_tab, log_size, n_layers, itw,
              tw_log, _stream())
    assert torch.equal(st_a, st_b) and torch.equal(al_a, al_b)
    for j in range(n_layers):
        assert torch.equal(tr_a[j], tr_b[j]), j
        assert torch.equal(ev_a[j + 1], ev_b[j + 1]), j
    w, init = [layer0[k] for k in range(4)], O.line_domain_initial_index(log_size)
    alphas = al_b.cpu().numpy().view(np.uint32).reshape(n_layers, 4)
    for j in range(n_layers):
        w = O.fold_line(w, init, tuple(int(x) for x in alphas[j]))
        init = O.double_index(init)
    assert all(np.array_equal(a, b) for a, b in zip(ev_b[n_layers].cpu().numpy().view(np.uint32), w))


# ------------------------------------------------------------------ decommitment reads

def test_gather_words_matches_indexing(B):
    cols = [_col(m31_column(70 + k, 6 + k)) for k in range(3)]
    digests = torch.arange(64 * 8, dtype=torch.int32, device="cuda").reshape(64, 8)
    tensors = [c.data for c in cols] + [digests]
    rng = np.random.default_rng(5)
    slots = rng.integers(0, 4, 500).astype(np.uint32)
    lens = [t.numel() for t in tensors]
    idx = np.array([rng.integers(0, lens[s]) for s in slots], np.uint32)
    got = B.gather_words(tensors, slots, idx)
    host = [t.reshape(-1).cpu().numpy().view(np.uint32) for t in tensors]
    want = np.array([host[s][i] for s, i in zip(slots, idx)], np.uint32)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("inverse,log_n,n_layers,plan", [(True, 12, 12, (3, 4, 5)), (True, 13, 13, (7, 6)),
                                                        (False, 12, 10, (4, 6)), (False, 14, 12, (5, 3, 4))])
def test_fft_results_do_not_depend_on_the_pass_plan(B, inverse, log_n, n_layers, plan):
    from proving_gb300 import autotune
    tree = _tree(B, log_n + 1)
    tw, itw = O.canonic_twiddles(log_n + 1)
    vals = m31_column(90 + log_n, log_n if inverse else n_layers)
    autotune.set_plan(inverse, log_n, n_layers, plan)
    try:
        assert autotune.get_plan(inverse, log_n, n_layers) == plan
        col = _col(vals)
        if inverse:
            B.interpolate_columns([col], tree)
            got, want = col.to_cpu(), O.interpolate(vals, itw)
        else:
            got = B.evaluate_polynomials([col], log_n, tree)[0].to_cpu()
            want = O.evaluate(vals, log_n, tw)
    finally:
        autotune.set_plan(inverse, log_n, n_layers, [])
    assert np.array_equal(got, want)


# ------------------------------------------------------------------ device channel

def test_device_channel_matches_host_channel(B):
    # mix_root and draw_secure_felt on the device state equal Blake2sChannel's, draw counter included
    import struct
    from proving_gb300 import _lib
    from proving_gb300.backend import _stream
    from proving_gb300.prover import Blake2sChannel
    host = Blake2sChannel(bytes(range(32)))
    host.n_draws = 5
    state = torch.tensor(np.array(list(struct.unpack("<8I", host.digest)) + [5], np.uint32).view(np.int32),
                         device="cuda")
    felt = torch.empty(4, dtype=torch.int32, device="cuda")
    want = [host.draw_secure_felt()]
    _lib.call("cs_channel_draw_secure_felt", state.data_ptr(), felt.data_ptr(), _stream())
    got = [tuple(felt.cpu().numpy().view(np.uint32).tolist())]
    for k in range(3):
        root = np.random.default_rng(k).integers(0, 1 << 32, 8, dtype=np.uint64).astype(np.uint32)
        host.mix_root(root.astype("<u4").tobytes())
        d_root = torch.tensor(root.view(np.int32), device="cuda")
        _lib.call("cs_channel_mix_root", state.data_ptr(), d_root.data_ptr(), _stream())
        for _ in range(2):
            want.append(host.draw_secure_felt())
            _lib.call("cs_channel_draw_secure_felt", state.data_ptr(), felt.data_ptr(), _stream())
            got.append(tuple(felt.cpu().numpy().view(np.uint32).tolist()))
    assert got == want
    words = state.cpu().numpy().view(np.uint32)
    assert words[:8].astype("<u4").tobytes() == host.digest and int(words[8]) == host.n_draws
