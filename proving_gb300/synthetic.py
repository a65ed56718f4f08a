"""Seeded synthetic inputs shared by the tests and the benchmark.

The reference seeds `SmallRng`; its stream is not reproduced. Instead every
input here comes from SplitMix64 (Steele, Lea, Flood 2014), two u32 words per
64-bit output, mapped to M31 by taking the low 31 bits and rejecting the
single value P, so each value is uniform in [0, P). The same arrays are fed to
the oracle and to the CUDA path.
"""
from __future__ import annotations

import numpy as np

P = (1 << 31) - 1
_GAMMA = np.uint64(0x9E3779B97F4A7C15)
_C1 = np.uint64(0xBF58476D1CE4E5B9)
_C2 = np.uint64(0x94D049BB133111EB)


def _splitmix64(seed: int, n: int) -> np.ndarray:
    with np.errstate(over="ignore"):
        i = np.arange(1, n + 1, dtype=np.uint64)
        z = np.uint64(seed & 0xFFFFFFFFFFFFFFFF) + i * _GAMMA
        z = (z ^ (z >> np.uint64(30))) * _C1
        z = (z ^ (z >> np.uint64(27))) * _C2
        return z ^ (z >> np.uint64(31))


def _mix_seed(seed: int, stream: int) -> int:
    return int(_splitmix64((seed * 0x100000001B3 + stream) & 0xFFFFFFFFFFFFFFFF, 1)[0])


def m31_values(seed: int, n: int) -> np.ndarray:
    """n uniform M31 values from one seeded stream."""
    extra = 64
    words = _splitmix64(seed, (n + extra + 1) // 2).view(np.uint32)
    vals = words & np.uint32(P)
    vals = vals[vals != P]
    assert vals.size >= n
    return np.ascontiguousarray(vals[:n])


def m31_column(seed: int, log_size: int) -> np.ndarray:
    return m31_values(_mix_seed(seed, 0), 1 << log_size)


def m31_columns(seed: int, n_cols: int, log_size: int) -> np.ndarray:
    """(n_cols, 2^log_size) uint32, column c drawn from stream (seed, c)."""
    out = np.empty((n_cols, 1 << log_size), dtype=np.uint32)
    for c in range(n_cols):
        out[c] = m31_values(_mix_seed(seed, c), 1 << log_size)
    return out


def qm31_column(seed: int, log_size: int) -> list[np.ndarray]:
    """A QM31 column as 4 coordinate arrays (SoA)."""
    return [m31_values(_mix_seed(seed, 1000 + k), 1 << log_size) for k in range(4)]


def seeded_qm31(seed: int) -> np.ndarray:
    return m31_values(_mix_seed(seed, 7777), 4)


def seeded_log_sizes(seed: int, n: int, lo: int, hi: int, mean: float) -> np.ndarray:
    """Log sizes lo + min(hi-lo, G), G geometric on {0,1,..} with the given mean of the result."""
    rng = np.random.default_rng(seed)
    target = mean - lo
    # Solve for the success probability p of a truncated geometric with the given mean.
    cap = hi - lo

    def trunc_mean(p):
        k = np.arange(cap + 1)
        pmf = p * (1 - p) ** k
        pmf[-1] = (1 - p) ** cap
        return float((k * pmf).sum())

    lo_p, hi_p = 1e-6, 1 - 1e-6
    for _ in range(100):
        mid = (lo_p + hi_p) / 2
        if trunc_mean(mid) > target:
            lo_p = mid
        else:
            hi_p = mid
    p = (lo_p + hi_p) / 2
    g = rng.geometric(p, n) - 1
    return (lo + np.minimum(cap, g)).astype(np.uint32)


def mixed_trace_shape(seed: int = 7, n_base: int = 600, n_interaction: int = 120, lo: int = 10, hi: int = 22,
                      mean: float = 16.0):
    """The batched mixed-size trace as components: n_interaction single-column LogUp components
    (one value column and one QM31 running-sum column each) and Wide-Fibonacci components holding
    the other n_base - n_interaction base columns, all log sizes drawn by seeded_log_sizes. The
    Wide-Fibonacci columns of one size form one component; a size drawn fewer than 3 times still
    gets a 3-column component (the AIR's minimum). Returns ([(n_cols, log_n)], [lookup log_n])."""
    fib_logs = seeded_log_sizes(seed, n_base - n_interaction, lo, hi, mean)
    lookup_logs = [int(v) for v in seeded_log_sizes(seed + 1, n_interaction, lo, hi, mean)]
    counts = {}
    for v in fib_logs:
        counts[int(v)] = counts.get(int(v), 0) + 1
    comps = [(max(3, counts[k]), k) for k in sorted(counts)]
    return comps, lookup_logs
