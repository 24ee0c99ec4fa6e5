"""Regenerates tests/golden/ref_steps.npz: one plain step of the reference's own
code (its kernels compiled for the host by oracle/build_ref.py; see
oracle/ref_harness.cpp) on four small scenes, inputs and outputs.

Run where the reference checkout is available (oracle/build_ref.py finds it
through $SPH_REFERENCE_DIR):

    python tests/golden/make_ref_steps.py

The reference subtracts gravity from the y component of the acceleration
(particle_simulation.cu:471), so every scene here uses gravityAxis 1.  The
boundary maps are not stored: they are rebuilt from each scene's description
(the oracle's SetBox restatement is pinned to the reference's own map images).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

from cudasphnew_gb300 import params as P  # noqa: E402
from cudasphnew_gb300 import scenes  # noqa: E402

OUT = os.path.join(HERE, "ref_steps.npz")


def ref_scenes():
    """(name, scene, collide) of the fixtures; deterministic."""
    out = []
    tiny = scenes.dam_break(8, 8, 8, (0, 0, 0), (0.5, 0.5, 0.5), 3, "ref_tiny", 1)
    tiny.options.gravityAxis = 1
    out.append(("tiny", tiny, True))
    mov = scenes.dam_break(16, 16, 8, (0.1, 0.1, 0.1), (0.5, 0.5, 0.5), 5, "ref_moving", 1)
    mov.options.gravityAxis = 1
    rng = np.random.default_rng(17)
    mov.velocities[:] = rng.uniform(-1.5, 1.5, mov.velocities.shape).astype(np.float32)
    # the lattice's first x column just outside the container wall, moving out:
    # collision_handling puts them back on the wall
    wall = np.float32(mov.params.boxCen[0] - mov.params.boxDim[0])
    first = mov.positions[:, 0] < wall + np.float32(0.5 * P.SPACING + 0.02 * P.H)
    mov.positions[first, 0] = wall - np.float32(1e-4)
    mov.velocities[first, 0] = -1.0
    out.append(("moving", mov, True))
    # the reference's own scene set-up (Example01 + create_particle_box) with 16^3 particles
    pos = scenes.create_particle_box(-0.65, -0.45, -0.25, 0.5, 4096)
    p = P.example01_params(len(pos))
    o = P.default_options(gravity_axis=1, box_collision=False)
    ex = scenes.Scene("ref_example01_4096", p, o, pos, np.zeros_like(pos), P.example01_boundary(p))
    out.append(("example01", ex, False))
    # a block over the top of the sphere + cone obstacle, the lattice nodes
    # within 0.3 h of the solid (or inside it) left out: many particles feel the
    # wall terms of the obstacle's maps
    import oracle
    obs = scenes.small_obstacle()
    d = obs.boundary
    pos = scenes.lattice_block(20, 20, 16, (0.375, 0.375, 0.3), P.SPACING, 13, 0.01 * P.H)
    dist = -oracle.tex3d(oracle.boundary_maps(d), 0, pos.astype(np.float64))
    pos = pos[dist > 0.3 * P.H]
    p = P.dam_break_params((0, 0, 0), (1, 1, 0.5), len(pos))
    o = P.default_options(gravity_axis=1, box_collision=True)
    out.append(("obstacle", scenes.Scene("ref_obstacle", p, o, pos, np.zeros_like(pos), d), True))
    return out


def main():
    import oracle
    if oracle.ref_build() is None:
        sys.exit("the reference checkout is absent: set SPH_REFERENCE_DIR")
    arrays = {}
    for name, sc, collide in ref_scenes():
        bm = oracle.boundary_maps(sc.boundary) if sc.boundary is not None else None
        r = oracle.ref_step_plain(sc.params, bm, sc.positions, sc.velocities, collide)
        arrays[f"{name}/params"] = np.frombuffer(bytes(sc.params), np.uint8)
        arrays[f"{name}/in_pos"] = sc.positions
        arrays[f"{name}/in_vel"] = sc.velocities
        for k, v in r.items():
            arrays[f"{name}/{k}"] = v
    np.savez_compressed(OUT, **arrays)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
