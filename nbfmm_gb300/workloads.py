"""Seeded synthetic particle systems for the engine's benchmarks and tests.

These stand in for the workloads the engine is measured on; no dataset is involved. Velocities enter the
Stormer-Verlet state as x_prev = x0 - v0 * tick (tick = dt * sqrt(G)), the convention of the reference's
model generators (e.g. source/nbfmm/model/disk.cu:49-55 rotates the previous position back by one tick).

  plain       N uniform in [-1, 1)^2, masses U[0.5, 1.5], zero velocity, limits [-1, 1]^2
  disk        one disk: N-1 particles uniform in area on r in (0.1 R, R), equal masses summing to 1, a central
              point mass of 10; circular velocity sqrt(G M(<r) / r) around the centre
  two_disks   two such disks of radius 0.5 centred at (-0.6, 0) and (0.6, 0) with bulk velocities
              (+0.3, +0.05) and (-0.3, -0.05), N/2 particles each
"""
import dataclasses

import numpy as np

DOMAIN = (-1.25, -1.25, 1.25, 1.25)


@dataclasses.dataclass
class System:
    name: str
    position: np.ndarray  # (n, 2) float32
    weight: np.ndarray    # (n,) float32
    velocity: np.ndarray  # (n, 2) float32
    limits: tuple
    num_level: int
    epsilon: float
    dt: float
    steps: int
    grav_const: float = 1.0
    seed: int = 0

    @property
    def n(self) -> int:
        return int(self.weight.shape[0])

    def tick(self) -> float:
        return float(np.float32(self.dt) * np.sqrt(np.float32(self.grav_const)))

    def previous(self) -> np.ndarray:
        """x_prev = x0 - v0 * tick in FP32."""
        t = np.float32(self.tick())
        return (self.position - self.velocity * t).astype(np.float32)


def plain(n: int = 16384, seed: int = 1, num_level: int = 3) -> System:
    rng = np.random.default_rng(seed)
    pos = rng.uniform(-1.0, 1.0, size=(n, 2)).astype(np.float32)
    w = rng.uniform(0.5, 1.5, size=n).astype(np.float32)
    return System("plain", pos, w, np.zeros_like(pos), (-1.0, -1.0, 1.0, 1.0), num_level, 1e-3, 1e-4, 100, seed=seed)


def _disk(rng, n, radius, centre, bulk, grav_const=1.0, central_mass=10.0, disk_mass=1.0):
    nd = n - 1
    r_in = 0.1 * radius
    u = rng.uniform(0.0, 1.0, size=nd)
    r = np.sqrt(r_in * r_in + u * (radius * radius - r_in * r_in))
    theta = rng.uniform(0.0, 2.0 * np.pi, size=nd)
    m = disk_mass / nd
    enclosed = central_mass + disk_mass * (r * r - r_in * r_in) / (radius * radius - r_in * r_in)
    speed = np.sqrt(grav_const * enclosed / r)
    pos = np.empty((n, 2), np.float64)
    vel = np.empty((n, 2), np.float64)
    pos[0] = centre
    vel[0] = bulk
    pos[1:, 0] = centre[0] + r * np.cos(theta)
    pos[1:, 1] = centre[1] + r * np.sin(theta)
    vel[1:, 0] = bulk[0] - speed * np.sin(theta)
    vel[1:, 1] = bulk[1] + speed * np.cos(theta)
    w = np.full(n, m, np.float64)
    w[0] = central_mass
    return pos, w, vel


def disk(n: int = 1 << 20, seed: int = 2, num_level: int = 6) -> System:
    rng = np.random.default_rng(seed)
    pos, w, vel = _disk(rng, n, 1.0, (0.0, 0.0), (0.0, 0.0))
    return System("disk", pos.astype(np.float32), w.astype(np.float32), vel.astype(np.float32), DOMAIN, num_level,
                  1e-3, 1e-4, 1000, seed=seed)


def two_disks(n: int = 1 << 24, seed: int = 3, num_level: int = 8) -> System:
    rng = np.random.default_rng(seed)
    half = n // 2
    p1, w1, v1 = _disk(rng, half, 0.5, (-0.6, 0.0), (0.3, 0.05))
    p2, w2, v2 = _disk(rng, n - half, 0.5, (0.6, 0.0), (-0.3, -0.05))
    pos = np.concatenate([p1, p2]).astype(np.float32)
    w = np.concatenate([w1, w2]).astype(np.float32)
    vel = np.concatenate([v1, v2]).astype(np.float32)
    return System("two_disks", pos, w, vel, DOMAIN, num_level, 5e-4, 5e-5, 200, seed=seed)


# The measured configurations; depth d = log2(leaf cells per side) = num_level + 1.
CONFIGS = {
    "plain_16k": lambda: plain(16384, 1, 3),
    "disk_1m": lambda: disk(1 << 20, 2, 6),
    "two_disks_16m": lambda: two_disks(1 << 24, 3, 8),
    # a quarter of the particles on a quarter of the leaf cells: the same particles per cell as two_disks_16m
    "two_disks_4m": lambda: two_disks(1 << 22, 3, 7),
    # a quarter of the particles on the same leaf cells: two_disks_16m's cell size (so P2P's reciprocal series
    # applies as it does there), a quarter of its particles per cell
    "two_disks_4m_fine": lambda: two_disks(1 << 22, 3, 8),
}


@dataclasses.dataclass
class BatchSystem:
    """Many independent systems: particles concatenated, per-system ranges, limits and kinds."""
    name: str
    position: np.ndarray   # (n, 2) float32, systems concatenated
    weight: np.ndarray     # (n,)
    velocity: np.ndarray   # (n, 2)
    offsets: np.ndarray    # (S + 1,) int64
    limits: np.ndarray     # (S, 4) float32
    kinds: list            # "square" | "disk" per system
    epsilon: float
    dt: float
    steps: int
    grav_const: float = 1.0
    seed: int = 0

    @property
    def n(self) -> int:
        return int(self.offsets[-1])

    @property
    def num_systems(self) -> int:
        return len(self.kinds)

    def tick(self) -> float:
        return float(np.float32(self.dt) * np.sqrt(np.float32(self.grav_const)))

    def previous(self) -> np.ndarray:
        t = np.float32(self.tick())
        return (self.position - self.velocity * t).astype(np.float32)

    def sizes(self) -> np.ndarray:
        return np.diff(self.offsets)


def batched(num_systems: int = 512, seed: int = 4, median: int = 20000, lo: int = 2000, hi: int = 262144,
            sigma: float = 0.8) -> BatchSystem:
    """Systems with N ~ lognormal(median 20k, log-sd 0.8: about 14M particles for 512 systems), clipped to
    [2k, 262k]; each a uniform square (limits [-1, 1]^2) or a rotating disk (limits [-1.25, 1.25]^2) by a seeded
    coin flip."""
    rng = np.random.default_rng(seed)
    sizes = np.clip(np.round(median * np.exp(rng.normal(0.0, sigma, num_systems))), lo, hi).astype(np.int64)
    kinds = ["square" if c else "disk" for c in rng.integers(0, 2, num_systems)]
    pos, w, vel, lim = [], [], [], []
    for n, kind in zip(sizes, kinds):
        if kind == "square":
            pos.append(rng.uniform(-1.0, 1.0, (n, 2)))
            w.append(rng.uniform(0.5, 1.5, n) / n)
            vel.append(np.zeros((n, 2)))
            lim.append((-1.0, -1.0, 1.0, 1.0))
        else:
            p, m, v = _disk(rng, int(n), 1.0, (0.0, 0.0), (0.0, 0.0))
            pos.append(p)
            w.append(m)
            vel.append(v)
            lim.append(DOMAIN)
    offsets = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    return BatchSystem("batched", np.concatenate(pos).astype(np.float32), np.concatenate(w).astype(np.float32),
                       np.concatenate(vel).astype(np.float32), offsets, np.asarray(lim, np.float32), kinds,
                       1e-3, 1e-4, 100, seed=seed)
