"""Writes tests/golden/reference_kats.json.

Two kinds of entries:

* Known-answer values transcribed from the reference's own unit tests (each
  entry names the test file and lines it comes from). They pin the Blake2s
  hash, the Blake2s channel, proof-of-work verification and bit reversal.
* Lifted-Merkle leaf digests for the reference test
  `test_lifted_merkle_leaves` (crates/stwo/src/prover/vcs_lifted/prover.rs:207-236):
  columns of log sizes 2, 3, 4 holding 0..2^k, lifted to log size 4. The
  reference asserts leaf 0 = H(12 zero bytes), leaf 4 = H(le(0,2,4)) and
  leaf 15 = H(le(3,7,15)); those digests are computed here with Python's
  hashlib.blake2s, which is independent of the oracle's own Blake2s.

Run: python tests/golden/make_golden.py
"""
import hashlib
import json
import struct
from pathlib import Path


def h(data: bytes) -> str:
    return hashlib.blake2s(data, digest_size=32).hexdigest()


def le(*words) -> bytes:
    return b"".join(struct.pack("<I", w) for w in words)


WORDS = [0, 1, 2, 3, 0x12345678, 0xFFFFFFFF, 7, 8, 9]
DIGEST_HEX = "efee1538e0216d3a09ce742ce768c44a7db004d801c40f66040994353f55fe85"

kats = {
    "blake2s_a": {
        "source": "crates/stwo/src/core/vcs/blake2_hash.rs:126-132",
        "input_hex": b"a".hex(),
        "digest_hex": "4a0d129873403037c2cd9b9048203687f6233fb6738956e0349bd4320fec3e90",
    },
    "hash_u32s": {
        "source": "crates/stwo/src/core/vcs_lifted/hasher_test.rs:10-19",
        "words": WORDS,
        "digest_hex": "efee1538e0216d3a09ce742ce768c44a7db004d801c40f66040994353f55fe85",
    },
    "hash_u32s_followed_by_digest": {
        "source": "crates/stwo/src/core/vcs_lifted/hasher_test.rs:47-63",
        "words": WORDS,
        "digest_in_hex": DIGEST_HEX,
        "digest_hex": "18a60268d189dccf5065ddd361d280474fbc2b08d75a7e4e1c20e57a67f2f7fa",
    },
    "channel_mix_u64": {
        "source": "crates/stwo/src/core/channel/blake2s.rs:185-204",
        "value": 0x1111222233334444,
        "equivalent_u32s": [0x33334444, 0x11112222],
        "digest": [0xbc, 0x9e, 0x3f, 0xc1, 0xd2, 0x4e, 0x88, 0x97, 0x95, 0x6d, 0x33, 0x59, 0x32, 0x73,
                   0x97, 0x24, 0x9d, 0x6b, 0xca, 0xcd, 0x22, 0x4d, 0x92, 0x74, 0x4, 0xe7, 0xba, 0x4a,
                   0x77, 0xdc, 0x6e, 0xce],
    },
    "channel_mix_u32s": {
        "source": "crates/stwo/src/core/channel/blake2s.rs:206-219",
        "words": [1, 2, 3, 4, 5, 6, 7, 8, 9],
        "digest": [0x70, 0x91, 0x76, 0x83, 0x57, 0xbb, 0x1b, 0xb3, 0x34, 0x6f, 0xda, 0xb6, 0xb3, 0x57,
                   0xd7, 0xfa, 0x46, 0xb8, 0xfb, 0xe3, 0x2c, 0x2e, 0x43, 0x24, 0xa0, 0xff, 0xc2, 0x94,
                   0xcb, 0xf9, 0xa1, 0xc7],
    },
    "verify_pow_nonce": {
        "source": "crates/stwo/src/core/channel/blake2s.rs:221-239",
        "digest_words": [968886948, 725376924, 836084817, 484428276, 1805658819, 300032261, 172116750,
                         994058243],
        "cases": [[10, 649, True], [11, 649, False], [9, 649, False], [10, 648, False], [10, 650, False]],
    },
    "bit_reverse": {
        "source": "crates/stwo/src/prover/backend/cpu/mod.rs:86-91",
        "input": [0, 1, 2, 3, 4, 5, 6, 7],
        "output": [0, 4, 2, 6, 1, 5, 3, 7],
    },
    "lifted_merkle_leaves": {
        "source": "crates/stwo/src/prover/vcs_lifted/prover.rs:194-236",
        "column_log_sizes": [2, 3, 4],
        "column_values": "column k holds 0..2^log_size",
        "lifting_log_size": 4,
        "leaves": {
            "0": h(bytes(12)),
            "4": h(le(0, 2, 4)),
            "15": h(le(3, 7, 15)),
        },
    },
    "m31_circle_gen": {
        "source": "crates/stwo/src/core/circle.rs:181-185",
        "x": 2,
        "y": 1268011823,
        "log_order": 31,
    },
}

if __name__ == "__main__":
    out = Path(__file__).with_name("reference_kats.json")
    out.write_text(json.dumps(kats, indent=1) + "\n")
    print("wrote", out)
