"""Seeded synthetic inputs for the CellFlow step.

Random numbers come from Philox4x32-10 (Salmon, Moraes, Dror, Shaw,
"Parallel random numbers: as easy as 1, 2, 3", SC'11), written here in numpy
integer arithmetic, so a seed gives the same integers on every machine; the
device spawn kernel (init.cu) uses the same generator with counter (i,0,0,0).

Domain convention: the reference simulates in [0, W)^3 with an fmodf wrap
(cuda-native/src/ParticleSimulation.cu:159-161).  Configurations quoted on
[-1, 1]^3 are drawn there and shifted by +1 in float32 into W = H = D = 2.
Uniform coordinates are multiples of 2^-23, so the shift is exact.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

_M0 = np.uint64(0xD2511F53)
_M1 = np.uint64(0xCD9E8D57)
_W0 = np.uint32(0x9E3779B9)
_W1 = np.uint32(0xBB67AE85)
_MASK = np.uint64(0xFFFFFFFF)


def philox4x32(counter: np.ndarray, stream: int, seed: int) -> np.ndarray:
    """Philox4x32-10 of counters (counter, stream, 0, 0) under a 64-bit seed.

    Returns uint32 of shape (len(counter), 4).
    """
    c0 = np.asarray(counter, dtype=np.uint64) & _MASK
    c1 = np.full_like(c0, np.uint64(stream) & _MASK)
    c2 = np.zeros_like(c0)
    c3 = np.zeros_like(c0)
    k0 = np.uint32(seed & 0xFFFFFFFF)
    k1 = np.uint32((seed >> 32) & 0xFFFFFFFF)
    for r in range(10):
        if r:
            k0 = np.uint32((int(k0) + int(_W0)) & 0xFFFFFFFF)
            k1 = np.uint32((int(k1) + int(_W1)) & 0xFFFFFFFF)
        p0 = _M0 * c0
        p1 = _M1 * c2
        hi0, lo0 = p0 >> np.uint64(32), p0 & _MASK
        hi1, lo1 = p1 >> np.uint64(32), p1 & _MASK
        c0, c1, c2, c3 = (hi1 ^ c1 ^ np.uint64(k0)), lo1, (hi0 ^ c3 ^ np.uint64(k1)), lo0
    return np.stack([c0, c1, c2, c3], axis=1).astype(np.uint32)


def _words(n: int, stream: int, seed: int) -> np.ndarray:
    """n uint32 words from one stream."""
    blocks = (n + 3) // 4
    return philox4x32(np.arange(blocks, dtype=np.uint64), stream, seed).reshape(-1)[:n]


def unit24(words: np.ndarray) -> np.ndarray:
    """Uniform float32 in [0, 1): multiples of 2^-24."""
    return ((words >> np.uint32(8)).astype(np.float32) * np.float32(1.0 / 16777216.0)).astype(np.float32)


def normal(n: int, stream: int, seed: int) -> np.ndarray:
    """Standard normal float64 by Box-Muller from two uniforms."""
    w = _words(2 * n, stream, seed).astype(np.float64)
    u1 = (w[0::2] + 0.5) * 2.0**-32
    u2 = w[1::2] * 2.0**-32
    return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)


def uniform_positions(n: int, seed: int) -> np.ndarray:
    """n x 3 float32 positions uniform in [-1, 1)^3, shifted into [0, 2)^3."""
    u = unit24(_words(3 * n, 1, seed)).reshape(n, 3)
    x = (u * np.float32(2.0) - np.float32(1.0)).astype(np.float32)
    return (x + np.float32(1.0)).astype(np.float32)


def uniform_types(n: int, num_types: int, seed: int) -> np.ndarray:
    w = _words(n, 2, seed).astype(np.uint64)
    return ((w * np.uint64(num_types)) >> np.uint64(32)).astype(np.uint32)


def gaussian_table(num_types: int, mean: float, sigma: float, seed: int, offset: float = 0.0) -> np.ndarray:
    """T x T force table drawn from N(mean, sigma) plus an additive offset, unclamped, float32."""
    z = normal(num_types * num_types, 3, seed)
    return (mean + sigma * z + offset).astype(np.float32).reshape(num_types, num_types)


def blob_positions(n: int, blobs: int, sigma: float, seed: int) -> np.ndarray:
    """n x 3 float32 positions in `blobs` Gaussian blobs (equal counts, centres uniform in
    [-1, 1)^3), wrapped into the periodic box and shifted into [0, 2)^3."""
    centres = unit24(_words(3 * blobs, 4, seed)).reshape(blobs, 3).astype(np.float64) * 2.0 - 1.0
    z = normal(3 * n, 5, seed).reshape(n, 3)
    owner = np.arange(n) % blobs
    x = centres[owner] + sigma * z
    x = np.mod(x + 1.0, 2.0)  # wrap into [0, 2)
    x = x.astype(np.float32)
    x[x >= np.float32(2.0)] = np.float32(0.0)
    return x


@dataclass
class Workload:
    """A synthetic configuration of the step."""

    name: str
    n: int
    num_types: int
    radius: float
    steps: int
    table_mean: float = 0.0
    table_sigma: float = 0.5
    blobs: int = 0
    blob_sigma: float = 0.0
    seed: int = 0
    extent: float = 2.0
    delta_t: float = 0.01
    prox_distance: float | None = None
    prox_max_conn: int = 5
    extra: dict = field(default_factory=dict)

    def params(self):
        from .world import SimulationParams

        return SimulationParams(
            radius=self.radius, delta_t=self.delta_t, friction=0.51, repulsion=64.83, attraction=3.06, k=29.45,
            balance=0.79, canvas_width=self.extent, canvas_height=self.extent, canvas_depth=self.extent,
            num_particle_types=self.num_types, ratio_with_lfo=0.0, force_multiplier=2.33,
            max_expected_neighbors=400,
        )

    def positions(self) -> np.ndarray:
        if self.blobs:
            return blob_positions(self.n, self.blobs, self.blob_sigma, self.seed)
        return uniform_positions(self.n, self.seed)

    def types(self) -> np.ndarray:
        return uniform_types(self.n, self.num_types, self.seed)

    def table(self) -> np.ndarray:
        return gaussian_table(self.num_types, self.table_mean, self.table_sigma, self.seed)


@dataclass
class BatchedWorkload:
    """Independent worlds of log-uniform size, each with its own seeded inputs."""

    name: str
    worlds: int
    n_min: int
    n_max: int
    num_types: int
    radius: float
    graph_steps: int
    seed: int
    table_sigma: float = 0.5
    extent: float = 2.0
    delta_t: float = 0.01

    def sizes(self) -> np.ndarray:
        u = unit24(_words(self.worlds, 7, self.seed)).astype(np.float64)
        lo, hi = np.log(self.n_min), np.log(self.n_max)
        return np.rint(np.exp(lo + u * (hi - lo))).astype(np.int32)

    def world(self, k: int, n: int):
        """Positions, types and force table of world k (seeded seed + k)."""
        s = self.seed + k
        return uniform_positions(n, s), uniform_types(n, self.num_types, s), gaussian_table(
            self.num_types, 0.0, self.table_sigma, s)

    def params(self):
        return Workload(self.name, n=1, num_types=self.num_types, radius=self.radius, steps=self.graph_steps,
                        extent=self.extent, delta_t=self.delta_t).params()


# The configurations of the benchmark suite (W = H = D = 2 after the shift).
PLAIN_SMALL = Workload("plain_n4096_t6", n=4096, num_types=6, radius=0.1, steps=100, seed=0x5EED0001)
README_SCALE = Workload("plain_n100k_t8", n=100_000, num_types=8, radius=0.0920, steps=1000, seed=0x5EED0002,
                        prox_distance=0.05, prox_max_conn=5)
BLOBS_1M = Workload("blobs_n1m_t12", n=1_000_000, num_types=12, radius=0.02, steps=500, table_mean=0.1,
                    table_sigma=0.6, blobs=64, blob_sigma=0.02, seed=0x5EED0003)
WORKLOADS = {w.name: w for w in (PLAIN_SMALL, README_SCALE, BLOBS_1M)}
BATCHED_256 = BatchedWorkload("batched_256w", worlds=256, n_min=2048, n_max=65536, num_types=6, radius=0.1,
                              graph_steps=100, seed=0x5EED0004)
BATCHED = {BATCHED_256.name: BATCHED_256}
