"""Pins the CPU oracle to the reference: known-answer vectors from the
reference's unit tests (tests/golden/reference_kats.json) and the structural
tests the reference runs on its CpuBackend, restated. CPU only."""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O
from proving_gb300.synthetic import m31_column, qm31_column, seeded_qm31

KATS = json.loads((Path(__file__).parent / "golden" / "reference_kats.json").read_text())
P = O.P


def le_bytes(words):
    return b"".join(int(w).to_bytes(4, "little") for w in words)


# ------------------------------------------------------------------ KATs

def test_blake2s_kat():
    k = KATS["blake2s_a"]
    assert O.blake2s(bytes.fromhex(k["input_hex"])).hex() == k["digest_hex"]


def test_hash_u32s_kat():
    k = KATS["hash_u32s"]
    assert O.blake2s(le_bytes(k["words"])).hex() == k["digest_hex"]
    k = KATS["hash_u32s_followed_by_digest"]
    assert O.blake2s(le_bytes(k["words"]) + bytes.fromhex(k["digest_in_hex"])).hex() == k["digest_hex"]


@pytest.mark.parametrize("n", [0, 1, 31, 32, 55, 63, 64, 65, 127, 128, 129, 1000])
def test_blake2s_matches_hashlib(n):
    data = bytes((i * 37 + 11) & 0xFF for i in range(n))
    assert O.blake2s(data) == hashlib.blake2s(data).digest()


def test_channel_kats():
    k = KATS["channel_mix_u64"]
    ch = O.Blake2sChannel()
    ch.mix_u64(k["value"])
    assert list(ch.digest) == k["digest"]
    ch2 = O.Blake2sChannel()
    ch2.mix_u32s(k["equivalent_u32s"])
    assert ch2.digest == ch.digest
    k = KATS["channel_mix_u32s"]
    ch = O.Blake2sChannel()
    ch.mix_u32s(k["words"])
    assert list(ch.digest) == k["digest"]


def test_channel_draw_counts():
    # crates/stwo/src/core/channel/blake2s.rs:130-141
    ch = O.Blake2sChannel()
    ch.draw_u32s()
    assert ch.n_draws == 1
    for _ in range(9):
        ch.draw_secure_felt()
    assert ch.n_draws == 10
    ch.mix_u64(5)
    assert ch.n_draws == 0


def test_pow_kat():
    k = KATS["verify_pow_nonce"]
    digest = le_bytes(k["digest_words"])
    ch = O.Blake2sChannel(digest)
    for bits, nonce, ok in k["cases"]:
        assert ch.verify_pow_nonce(bits, nonce) == ok


@pytest.mark.parametrize("bits", [1, 4, 8, 10])
def test_grind_is_smallest(bits):
    ch = O.Blake2sChannel()
    ch.mix_u64(0x1111222233334344)
    nonce = O.grind(ch.digest, bits)
    assert ch.verify_pow_nonce(bits, nonce)
    assert not any(ch.verify_pow_nonce(bits, n) for n in range(nonce))


def test_bit_reverse_kat():
    k = KATS["bit_reverse"]
    assert list(O.bit_reverse(k["input"])) == k["output"]


def test_circle_gen_order():
    k = KATS["m31_circle_gen"]
    assert O.circle_index_to_point(1) == (k["x"], k["y"])
    # 2^30 * G is not the identity, 2^31 * G is.
    assert O.circle_index_to_point(1 << 30) != (1, 0)
    assert O.circle_index_to_point(0) == (1, 0)


def test_lifted_merkle_leaves_kat():
    k = KATS["lifted_merkle_leaves"]
    cols = [np.arange(1 << l, dtype=np.uint32) for l in k["column_log_sizes"]]
    leaves = O.merkle_build_leaves(cols, k["lifting_log_size"])
    for idx, hexd in k["leaves"].items():
        assert leaves[int(idx)].tobytes().hex() == hexd


def test_merkle_empty():
    # An empty tree is one hash of no data (prover.rs:41-50, merkle_lifted.rs:48-50).
    root = O.merkle_commit([], 0)
    assert root == hashlib.blake2s(b"").digest()


# ------------------------------------------------------------ fields

def test_qm31_inverse():
    rng = np.random.default_rng(1)
    for _ in range(20):
        a = rng.integers(0, P, 4, dtype=np.uint32)
        assert list(O.qm31_mul(a, O.qm31_inv(a))) == [1, 0, 0, 0]


def test_m31_mul_matches_python():
    rng = np.random.default_rng(2)
    a = rng.integers(0, P, 10000, dtype=np.uint32)
    b = rng.integers(0, P, 10000, dtype=np.uint32)
    ref = (a.astype(object) * b.astype(object)) % P
    assert np.array_equal(O.m31_mul(a, b), np.array(ref, dtype=np.uint32))


# ------------------------------------------------------------ polys

@pytest.mark.parametrize("log_n", [1, 2, 3, 4, 5, 8, 11])
def test_fft_roundtrip(log_n):
    tw, itw = O.canonic_twiddles(log_n + 2)
    coeffs = m31_column(seed=log_n, log_size=log_n)
    ev = O.evaluate(coeffs, log_n, tw)
    assert np.array_equal(O.interpolate(ev, itw), coeffs)


@pytest.mark.parametrize("log_n,blowup", [(3, 1), (5, 2), (8, 1), (10, 3)])
def test_extend_then_interpolate(log_n, blowup):
    # Evaluating on a blown-up domain and interpolating there gives the
    # zero-padded coefficients (crates/stwo/src/prover/backend/simd/circle.rs:606-640).
    tw, itw = O.canonic_twiddles(log_n + blowup + 1)
    coeffs = m31_column(seed=7, log_size=log_n)
    ev = O.evaluate(coeffs, log_n + blowup, tw)
    back = O.interpolate(ev, itw)
    assert np.array_equal(back[: 1 << log_n], coeffs)
    assert not back[1 << log_n:].any()


@pytest.mark.parametrize("log_n", [3, 6])
def test_evaluate_matches_eval_at_point(log_n):
    tw, _ = O.canonic_twiddles(log_n)
    coeffs = m31_column(seed=3, log_size=log_n)
    ev = O.evaluate(coeffs, log_n, tw)
    half_init = O.canonic_half_coset_initial_index(log_n)
    half_step = O.subgroup_gen(log_n - 1)
    for i in [0, 1, 5, (1 << log_n) - 1]:
        j = int(O.bit_reverse(np.arange(1 << log_n))[i])
        hs = 1 << (log_n - 1)
        idx = (half_init + half_step * j) % (1 << 31) if j < hs else \
            (-(half_init + half_step * (j - hs))) % (1 << 31)
        x, y = O.circle_index_to_point(idx)
        v = O.eval_at_point(coeffs, [x, 0, 0, 0], [y, 0, 0, 0])
        assert list(v) == [int(ev[i]), 0, 0, 0]


def test_twiddle_subtree_is_suffix():
    # A tree for a smaller canonic domain is the tail of a bigger tree's layers
    # (crates/stwo/src/prover/poly/twiddles.rs:85-134 and utils.rs:98-111).
    big, _ = O.canonic_twiddles(10)
    small, _ = O.canonic_twiddles(6)
    assert np.array_equal(big[-(1 << 5):-1], small[:-1])


def test_lifted_merkle_equals_explicit_lift():
    # crates/stwo/src/prover/vcs_lifted/prover.rs:238-266: committing a small
    # column lifted to a big tree equals committing its explicit lifted evaluation.
    log_n, lifted = 3, 9
    tw, itw = O.canonic_twiddles(lifted + 1)
    coeffs = np.arange(1 << log_n, dtype=np.uint32)
    small_ev = O.evaluate(coeffs, log_n, tw)
    # Lifted polynomial p(pi^k(P)) evaluated on the big domain.
    hs = 1 << (lifted - 1)
    half_init = O.canonic_half_coset_initial_index(lifted)
    half_step = O.subgroup_gen(lifted - 1)
    vals = []
    for j in range(1 << lifted):
        idx = (half_init + half_step * j) % (1 << 31) if j < hs else \
            (-(half_init + half_step * (j - hs))) % (1 << 31)
        idx = (idx << (lifted - log_n)) % (1 << 31)       # repeated doubling
        x, y = O.circle_index_to_point(idx)
        vals.append(int(O.eval_at_point(coeffs, [x, 0, 0, 0], [y, 0, 0, 0])[0]))
    lifted_ev = O.bit_reverse(np.array(vals, np.uint32))
    zeros = np.zeros(1 << lifted, np.uint32)
    r1 = O.merkle_commit([lifted_ev, zeros], lifted)
    r2 = O.merkle_commit([small_ev, zeros], lifted)
    assert r1 == r2


# ------------------------------------------------------------ FRI

@pytest.mark.parametrize("log_n", [3, 6, 9])
def test_fri_folds_reach_constant(log_n):
    # A polynomial of degree < 2^(log_n-1) on a domain of 2^log_n (blowup 1)
    # folds to a constant line polynomial: the last 2-point layer is equal.
    tw, itw = O.canonic_twiddles(log_n)
    coords = []
    for k in range(4):
        c = m31_column(seed=100 + k, log_size=log_n - 1)
        coords.append(O.evaluate(c, log_n, tw))
    alpha = seeded_qm31(5)
    layer = O.fold_circle_into_line(coords, alpha)
    init = O.line_domain_initial_index(log_n - 1)
    while layer[0].size > 2:
        layer = O.fold_line(layer, init, seeded_qm31(layer[0].size))
        init = O.double_index(init)
    for k in range(4):
        assert layer[k][0] == layer[k][1]
