"""Synthetic scenes: the reference's Example01 and the dam-break benchmark
configurations.  Every random number comes from SplitMix64 over a counter, so
the same (seed, particle index) gives the same float32 state everywhere.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import params as P

_GOLD = np.uint64(0x9E3779B97F4A7C15)


def splitmix64(x: np.ndarray) -> np.ndarray:
    """SplitMix64 finaliser (Steele, Lea, Flood 2014) over uint64 counters."""
    with np.errstate(over="ignore"):
        z = (x.astype(np.uint64) + _GOLD).astype(np.uint64)
        z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)).astype(np.uint64)
        z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)).astype(np.uint64)
        return z ^ (z >> np.uint64(31))


def uniform(seed: int, counter: np.ndarray) -> np.ndarray:
    """U[0, 1) with 24-bit resolution from (seed, counter)."""
    key = (np.uint64(seed) << np.uint64(40)) ^ counter.astype(np.uint64)
    return (splitmix64(key) >> np.uint64(40)).astype(np.float64) * (1.0 / (1 << 24))


def lattice_block(nx: int, ny: int, nz: int, corner, spacing: float, seed: int,
                  jitter: float) -> np.ndarray:
    """(nx*ny*nz, 3) float32 lattice, x fastest (as create_particle_box,
    particle_simulation.cu:2900-2912), node (i,j,k) at corner + (i+1/2,j+1/2,k+1/2)*spacing
    plus a uniform jitter in [-jitter, jitter) per component."""
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    base = np.stack([i.ravel(), j.ravel(), k.ravel()], axis=1).astype(np.float64)
    pos = np.asarray(corner, np.float64) + (base + 0.5) * spacing
    n = len(pos)
    ctr = np.arange(3 * n, dtype=np.uint64).reshape(n, 3)
    pos += (2.0 * uniform(seed, ctr) - 1.0) * jitter
    return pos.astype(np.float32)


def create_particle_box(sx, sy, sz, d, num):
    """create_particle_box (particle_simulation.cu:2866-2917): a cube of
    floor(num^(1/3))^3 particles from (sx, sy, sz) with edge d."""
    m = int(math.pow(float(num), 1.0 / 3.0))
    dx = np.float32(d) / np.float32(m - 1)
    k, j, i = np.meshgrid(np.arange(m), np.arange(m), np.arange(m), indexing="ij")
    pos = np.stack([np.float32(sx) + i.ravel().astype(np.float32) * dx,
                    np.float32(sy) + j.ravel().astype(np.float32) * dx,
                    np.float32(sz) + k.ravel().astype(np.float32) * dx], axis=1)
    return pos.astype(np.float32)


@dataclass
class Scene:
    name: str
    params: P.SimulationParameters
    options: P.Options
    positions: np.ndarray
    velocities: np.ndarray
    boundary: P.BoundaryDesc | None = None
    steps: int = 0
    extra: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return len(self.positions)


def example01() -> Scene:
    """The reference's own scene (Example01 + Init, particle_simulation.cu:1745-1817)."""
    pos = create_particle_box(-0.65, -0.45, -0.25, 0.5, 40000)
    p = P.example01_params(len(pos))
    o = P.default_options(gravity_axis=1, box_collision=False)
    return Scene("example01", p, o, pos, np.zeros_like(pos), P.example01_boundary(p), steps=0)


def dam_break(nx, ny, nz, box_lo, box_hi, seed, name, steps, obstacle=False, dt=1e-4) -> Scene:
    pos = lattice_block(nx, ny, nz, box_lo, P.SPACING, seed, 0.01 * P.H)
    p = P.dam_break_params(box_lo, box_hi, len(pos), dt=dt)
    o = P.default_options(gravity_axis=2, box_collision=True)
    bd = None
    if obstacle:
        cx = 0.5 * (box_lo[0] + box_hi[0])
        cy = 0.5 * (box_lo[1] + box_hi[1])
        cz = 0.5 * (box_lo[2] + box_hi[2])
        pitch = np.float32(P.H) / np.float32(4.0)
        half = float(pitch) * 127 / 2
        start = (cx - half, cy - half, box_lo[2] - 0.05)
        shapes = [(P.SHAPE_SPHERE, (cx, cy, cz, 0.15)),
                  (P.SHAPE_CONE, (cx, cy, box_lo[2], 0.2, 0.3))]
        bd = P.obstacle_boundary(p, start, 128, shapes)
    return Scene(name, p, o, pos, np.zeros_like(pos), bd, steps)


def config1() -> Scene:
    """Plain dam break: 32x32x16 block in the unit box's corner, 16,384 particles."""
    return dam_break(32, 32, 16, (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), 1, "plain_16k", 1000)


def config2(nx=128, ny=128, nz=64) -> Scene:
    """SDF-obstacle dam break: 128x128x64 block (1,048,576 particles) in a
    [0,4]x[0,4]x[0,1] tank; sphere r=0.15 at the tank centre and a cone of base
    radius 0.2, height 0.3 on the floor below it, on a 128^3 map of pitch h/4."""
    return dam_break(nx, ny, nz, (0.0, 0.0, 0.0), (4.0, 4.0, 1.0), 2, "sdf_obstacle_1m", 500,
                     obstacle=True)


def small_obstacle(nx=24, ny=24, nz=12) -> Scene:
    """A small version of the obstacle scene for parity tests."""
    s = dam_break(nx, ny, nz, (0.0, 0.0, 0.0), (1.0, 1.0, 0.5), 7, "sdf_obstacle_small", 10,
                  obstacle=True)
    return s


def two_scale(nb=64, region=(0.4, 0.6), box=1.0, seed=3, name="two_scale_262k") -> Scene:
    """Two-scale run: an nb^3 block in the corner of a box of side `box`;
    particles inside the axis-aligned region [region[0], region[1]]^3 split
    into 8 children of half the smoothing length.  nb = 64 is the
    262,144-particle configuration."""
    pos = lattice_block(nb, nb, nb, (0.0, 0.0, 0.0), P.SPACING, seed, 0.01 * P.H)
    p = P.dam_break_params((0, 0, 0), (box, box, box), len(pos))
    o = P.default_options(gravity_axis=2, box_collision=True)
    for a in range(3):
        o.splitMin[a] = region[0]
        o.splitMax[a] = region[1]
    return Scene(name, p, o, pos, np.zeros_like(pos), None, 500)


def config3() -> Scene:
    """The 262,144-particle two-scale run: split region [0.4, 0.6]^3, children
    kept while their parent stays split and merged back on exit (childMode 1)."""
    sc = two_scale()
    sc.options.childMode = 1
    return sc


def batched_scene(n: int, frac: float, seed: int, name: str) -> Scene:
    """One scene of the batched workload: a cube lattice block of n particles
    (pitch h/2, x fastest, jittered like the other scenes) in the corner of a
    box of side 2.5x the block side, and a solid sphere of radius frac x box
    side at the box centre on a 64^3 boundary map.  Lattice nodes inside the
    sphere (+ h/2) are dropped and the lattice grows until it holds n."""
    m = int(math.ceil(n ** (1.0 / 3.0) - 1e-9))
    while True:
        side = 2.5 * m * P.SPACING
        r = frac * side
        c = (0.5 * side, 0.5 * side, 0.5 * side)
        pos = lattice_block(m, m, m, (0.0, 0.0, 0.0), P.SPACING, seed, 0.01 * P.H)
        keep = np.linalg.norm(pos.astype(np.float64) - np.asarray(c), axis=1) > r + 0.5 * P.H
        if keep.sum() >= n:
            pos = pos[keep][:n]
            break
        m += 1
    p = P.dam_break_params((0.0, 0.0, 0.0), (side, side, side), n)
    o = P.default_options(gravity_axis=2, box_collision=True)
    return Scene(name, p, o, pos, np.zeros_like(pos), P.sphere_boundary(p, c, r), 200)


def batch_sizes(count: int = 64, seed: int = 4, lo: int = 4096, hi: int = 262144):
    """Particle counts log-uniform in [lo, hi] and sphere radii (as fractions
    of the box side) uniform in [0.05, 0.2], from SplitMix64."""
    u = uniform(seed, np.arange(2 * count, dtype=np.uint64)).reshape(count, 2)
    ns = np.rint(np.exp(np.log(lo) + u[:, 0] * (np.log(hi) - np.log(lo)))).astype(np.int64)
    return [int(v) for v in ns], [float(0.05 + 0.15 * v) for v in u[:, 1]]


def config4(count: int = 64, seed: int = 4):
    """The batched workload: `count` independent dam breaks (about 4M
    particles for 64 scenes), each with its own seeded sphere obstacle."""
    ns, fr = batch_sizes(count, seed)
    return [batched_scene(n, f, seed * 1000 + k, f"batch_{k}") for k, (n, f) in enumerate(zip(ns, fr))]

