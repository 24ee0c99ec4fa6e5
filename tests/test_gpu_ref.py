"""GPU step against the reference's own code.

tests/golden/ref_steps.npz holds one plain step of the reference's kernels
compiled for the host (see tests/test_ref_pin.py) on four scenes.  The GPU
step from the same state must give the same cell tables bit for bit, and
density, pressure and acceleration within 1e-5 of the FP64 magnitude scale
(the reference sums in its own FP32 order; the GPU adds each stencil row's
sum with compensation), the acceleration also within 1e-5 of the terms' own
magnitude (the wall terms follow the reference's FP32 operation order).
"""
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
if os.path.join(HERE, "golden") not in sys.path:
    sys.path.insert(0, os.path.join(HERE, "golden"))

from test_ref_pin import KEYS, fixtures  # noqa: E402

TOL = 1e-5


@pytest.mark.parametrize("skin", [0.0, 0.1])
def test_gpu_step_matches_the_reference_code(sphlib, orc, skin):
    for name, sc, collide, f in fixtures():
        sc.options.boxCollision = 1 if collide else 0
        sc.options.neighbourSkin = skin
        with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options, sc.boundary) as sim:
            sim.Advance()
            h, ids, start, end = sim.cells()
            g = dict(hash=h, ids=ids, start=start, end=end, rho=sim.read(sphlib.FIELD_DENSITY),
                     p=sim.read(sphlib.FIELD_PRESSURE), acc=sim.read(sphlib.FIELD_ACCELERATION),
                     pos=sim.positions(), vel=sim.velocities())
        for k in ("hash", "ids", "start", "end"):
            np.testing.assert_array_equal(g[k], f[k], err_msg=f"{name} {k}")
        bm = orc.boundary_maps(sc.boundary) if sc.boundary is not None else None
        r64 = orc.step_plain(sc.params, sc.options, bm, sc.positions, sc.velocities, fp64=True)
        assert (np.abs(g["rho"] - f["rho"]) <= TOL * r64["scale_rho"]).all(), name
        kscale = float(sc.params.gasStiffness) * (r64["rho"] + float(sc.params.restDensity))
        assert (np.abs(g["p"] - f["p"]) <= TOL * kscale).all(), name
        err = np.abs(g["acc"] - f["acc"]).max(1)
        assert (err <= TOL * r64["scale_acc"]).all(), name
        assert (err <= TOL * r64["scale_acc_direct"]).all(), name
        dt = float(sc.params.timeStep)
        vtol = dt * TOL * r64["scale_acc"] + 4 * np.spacing(np.abs(f["vel"]).max(1).astype(np.float32))
        # collision_handling (:742-834) removes the velocity along the normal
        # (pos - contact) / depth: a last-place difference in the integrated
        # position (the GPU fuses x + dt v, the host build of the reference
        # does not) turns that normal by ~ulp(x) / depth, and the removed
        # component by |v| ulp(x) / depth, for a particle put back on a wall
        cen = np.asarray(sc.params.boxCen, np.float64)
        dim = np.asarray(sc.params.boxDim, np.float64)
        lo, hi = np.float32(cen - dim), np.float32(cen + dim)
        walled = ((f["pos"] == lo) | (f["pos"] == hi)).any(1)
        x_in, v_in = sc.positions.astype(np.float64), sc.velocities.astype(np.float64)
        depth = np.linalg.norm(np.maximum(np.abs(x_in + dt * v_in - cen) - dim, 0.0), axis=1)
        turn = 8 * np.abs(v_in).max(1) * np.spacing(np.abs(f["pos"]).max(1).astype(np.float32)) \
            / np.maximum(depth, 1e-7)
        vtol = vtol + walled * turn
        assert (np.abs(g["vel"] - f["vel"]).max(1) <= vtol).all(), name
        if name == "moving":
            assert walled.sum() >= 128  # the particles started outside the wall
        xtol = dt * vtol + 4 * np.spacing(np.abs(f["pos"]).max(1).astype(np.float32))
        assert (np.abs(g["pos"] - f["pos"]).max(1) <= xtol).all(), name
