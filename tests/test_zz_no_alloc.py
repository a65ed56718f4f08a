"""The allocation-free grind entry point against the allocating one.

cs_grind_blake2s_noalloc serves callers that cannot allocate device memory
(a fixed device-memory arena, or a stream they do not own): its best-nonce
slots live in a static device array of 64 slots instead of a per-call
allocation. Collected last so that a run stopping at the first failure has
already run every other test; it also passes alone in a fresh process.
"""
import ctypes

import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def lib():
    from proving_gb300 import build, _lib
    build.build()
    assert torch.cuda.is_available()
    torch.cuda.init()
    L = _lib.load()
    L.cs_grind_blake2s_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64,
                                           ctypes.c_void_p, ctypes.c_void_p]
    L.cs_grind_blake2s_noalloc.restype = ctypes.c_int
    return L


def _digests(n, salt):
    import hashlib
    return b"".join(hashlib.blake2s(f"{salt}-{i}".encode()).digest() for i in range(n))


def _grind_alloc(L, digest: bytes, bits: int) -> int:
    d = (ctypes.c_uint8 * 32).from_buffer_copy(digest)
    out = ctypes.c_uint64(0)
    assert L.cs_grind_blake2s(d, bits, 1 << 40, ctypes.byref(out), None) == 0, L.cs_last_error()
    return out.value


def _grind_noalloc(L, digests: bytes, bits: int):
    n = len(digests) // 32
    buf = (ctypes.c_uint8 * len(digests)).from_buffer_copy(digests)
    out = (ctypes.c_uint64 * n)()
    st = L.cs_grind_blake2s_noalloc(buf, n, bits, 1 << 40, out, None)
    assert st == 0, L.cs_last_error()
    return list(out)


@pytest.mark.parametrize("bits", [10, 16])
def test_noalloc_matches_allocating_entry_point_twice(lib, bits):
    # two calls in a row: the second must not see the first call's slot contents
    for salt in ("first", "second"):
        digests = _digests(5, f"{salt}-{bits}")
        got = _grind_noalloc(lib, digests, bits)
        want = [_grind_alloc(lib, digests[32 * i:32 * i + 32], bits) for i in range(5)]
        assert got == want


def test_noalloc_rejects_more_digests_than_the_static_scratch(lib):
    digests = _digests(65, "too-many")
    buf = (ctypes.c_uint8 * len(digests)).from_buffer_copy(digests)
    out = (ctypes.c_uint64 * 65)()
    assert lib.cs_grind_blake2s_noalloc(buf, 65, 8, 1 << 20, out, None) == 1  # CS_ERR_INVALID_ARG
    assert b"at most 64" in lib.cs_last_error()
