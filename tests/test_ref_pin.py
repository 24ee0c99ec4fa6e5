"""The oracle pinned to the reference's own code.

tests/golden/ref_steps.npz holds one plain step of the reference's kernels
(compute_particle_hash, compute_particle_density_pressure,
compute_particle_acceleration_ifsurf, integrate_euler, collision_handling and
the device functions they call, particle_simulation.cu:89-474, 632-834,
1238-1556), compiled for the host without fused multiply-adds (oracle/_ref,
made by oracle/build_ref.py from the reference checkout; fixtures made by
tests/golden/make_ref_steps.py) on four scenes, one with the reference's own
Example01 box maps and one with a sphere and cone obstacle.  The oracle's
FP32 restatement must reproduce every output bit for bit; where the checkout
is present the harness is rebuilt and must reproduce the fixtures.
"""
import os
import sys

import numpy as np
import pytest

from cudasphnew_gb300 import params as P

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
if GOLDEN not in sys.path:
    sys.path.insert(0, GOLDEN)

import make_ref_steps  # noqa: E402

KEYS = ("hash", "ids", "start", "end", "rho", "p", "acc", "pos", "vel")


def fixtures():
    z = np.load(os.path.join(GOLDEN, "ref_steps.npz"))
    out = []
    for name, sc, collide in make_ref_steps.ref_scenes():
        f = {k: z[f"{name}/{k}"] for k in KEYS + ("params", "in_pos", "in_vel")}
        # the scene is rebuilt exactly as the fixture was made
        assert bytes(sc.params) == f["params"].tobytes(), name
        np.testing.assert_array_equal(sc.positions, f["in_pos"])
        np.testing.assert_array_equal(sc.velocities, f["in_vel"])
        out.append((name, sc, collide, f))
    return out


def test_restatement_reproduces_the_reference_code_bit_for_bit(orc):
    for name, sc, collide, f in fixtures():
        sc.options.boxCollision = 1 if collide else 0
        bm = orc.boundary_maps(sc.boundary) if sc.boundary is not None else None
        r32 = orc.step_plain(sc.params, sc.options, bm, sc.positions, sc.velocities)
        for k in KEYS:
            np.testing.assert_array_equal(r32[k], f[k], err_msg=f"{name} {k}")
        # and both are within the FP64 bars of the parity tests
        r64 = orc.step_plain(sc.params, sc.options, bm, sc.positions, sc.velocities, fp64=True)
        assert (np.abs(f["rho"] - r64["rho"]) <= 1e-5 * r64["scale_rho"]).all(), name
        assert (np.abs(f["acc"] - r64["acc"]).max(1) <= 1e-5 * r64["scale_acc"]).all(), name


def test_fixtures_cover_walls_collisions_and_motion(orc):
    fx = {name: (sc, f) for name, sc, collide, f in fixtures()}
    sc, f = fx["obstacle"]
    bm = orc.boundary_maps(sc.boundary)
    dist = -orc.tex3d(bm, 0, sc.positions.astype(np.float64))
    assert (dist < sc.boundary.restDistance).sum() > 50  # wall terms of the obstacle maps
    sc, f = fx["example01"]
    bm = orc.boundary_maps(sc.boundary)
    assert (-orc.tex3d(bm, 0, sc.positions.astype(np.float64)) < sc.boundary.restDistance).sum() > 50
    sc, f = fx["moving"]
    wall = np.float32(sc.params.boxCen[0] - sc.params.boxDim[0])
    outside = sc.positions[:, 0] < wall
    assert outside.sum() == 16 * 8 and np.abs(sc.velocities).max() > 1.0  # the collision path is taken
    assert (f["pos"][outside, 0] >= wall).all() and (f["vel"][outside, 0] > -1.0).all()


def test_reference_harness_reproduces_the_fixtures(orc):
    if not orc.ref_available():
        pytest.skip("the reference checkout is absent (the fixtures stand in for it)")
    for name, sc, collide, f in fixtures():
        bm = orc.boundary_maps(sc.boundary) if sc.boundary is not None else None
        r = orc.ref_step_plain(sc.params, bm, sc.positions, sc.velocities, collide)
        for k in KEYS:
            np.testing.assert_array_equal(r[k], f[k], err_msg=f"{name} {k}")


def test_restatement_equals_reference_on_the_full_example01_scene(orc):
    """The reference's own scene, 39,304 particles, its box maps: identical."""
    if not orc.ref_available():
        pytest.skip("the reference checkout is absent")
    from cudasphnew_gb300 import scenes
    sc = scenes.example01()
    bm = orc.boundary_maps(sc.boundary)
    r = orc.ref_step_plain(sc.params, bm, sc.positions, sc.velocities, False)
    r32 = orc.step_plain(sc.params, sc.options, bm, sc.positions, sc.velocities)
    for k in KEYS:
        np.testing.assert_array_equal(r32[k], r[k], err_msg=k)
