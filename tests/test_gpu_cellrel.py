"""GPU checks of cell-relative positions (sph_options.cellRelative = 1).

Positions are stored as an offset from the low corner of their grid cell plus
the cell's integer coordinates; pair offsets are formed in the particle's own
cell frame and the step is integrated there.  No reference counterpart, so
the oracle is the FP64 restatement of the reference step:

* one step from the same absolute input: hash, permutation and cell tables
  bit-exact (the cells come from the reference's hash of that input), and
  density, pressure, acceleration and the new state within the plain step's
  bars against the FP64 oracle;
* far from the grid origin (a scene moved by 256 in every axis, where an
  absolute FP32 position resolves only 3e-5) the stored state keeps tracking
  the FP64 trajectory to within the final read-back rounding, while the
  absolute store drifts by several units in the last place;
* conversions are exact (to half a unit in the last place of the cell size
  near zero), the launch shapes change no bit, and the other step kinds are
  refused.
"""
import ctypes

import numpy as np
import pytest

from cudasphnew_gb300 import params as P
from cudasphnew_gb300 import scenes

from test_gpu_step import TOL, check_step, maps_for, obstacle_block

pytestmark = pytest.mark.gpu


def rel_options(sc, on=1):
    o = P.Options.from_buffer_copy(bytes(sc.options))
    o.cellRelative = on
    return o


def run(sphlib, sc, opts, steps=1):
    with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, opts, sc.boundary) as sim:
        for _ in range(steps):
            sim.Advance()
        sim.synchronize()
        h, ids, start, end = sim.cells()
        return dict(hash=h, ids=ids, start=start, end=end, rho=sim.read(sphlib.FIELD_DENSITY),
                    p=sim.read(sphlib.FIELD_PRESSURE), acc=sim.read(sphlib.FIELD_ACCELERATION),
                    pos=sim.positions(), vel=sim.velocities())


SCENES = {
    "tiny": lambda: scenes.dam_break(8, 8, 8, (0, 0, 0), (0.5, 0.5, 0.5), 3, "tiny", 1),
    "config1": scenes.config1,
    "obstacle_block": obstacle_block,
}


@pytest.mark.parametrize("name", sorted(SCENES))
def test_one_step_parity(sphlib, orc, name):
    sc = SCENES[name]()
    g = run(sphlib, sc, rel_options(sc))
    check_step(orc, sc, g, maps_for(orc, sc))


def test_conversion_round_trip(sphlib):
    """Absolute -> cell-relative -> absolute.  The offset is an FP32 number
    below one cell, so it resolves half a unit in the last place of the cell
    size: a coordinate at least two cells from zero comes back bit for bit,
    one nearer zero (where FP32 itself is finer) to within that resolution."""
    sc = scenes.config1()
    rng = np.random.default_rng(3)
    lo = np.asarray(sc.params.gridOrigin, np.float64)
    hi = lo + np.asarray(sc.params.gridDim, np.float64) * float(sc.params.gridSpacing)
    x = rng.uniform(lo, hi, (sc.n, 3)).astype(np.float32)
    dx = float(sc.params.gridSpacing)
    res = float(np.spacing(np.float32(dx))) / 2
    far = np.abs(x) >= 2 * dx
    assert far.mean() > 0.8
    with sphlib.ParticleSimulation(sc.params, x, sc.velocities, rel_options(sc)) as sim:
        got = sim.positions()
        np.testing.assert_array_equal(got[far], x[far])
        assert np.abs(got[~far].astype(np.float64) - x[~far]).max() <= res
        sim.write_state(sc.positions, sc.velocities)
        got = sim.positions()
    far = np.abs(sc.positions) >= 2 * dx
    np.testing.assert_array_equal(got[far], sc.positions[far])
    assert np.abs(got[~far].astype(np.float64) - sc.positions[~far]).max() <= res


def shifted(sc, shift):
    """The same scene moved by `shift` in every axis, grid and walls included."""
    p = P.SimulationParameters.from_buffer_copy(bytes(sc.params))
    for a in range(3):
        p.gridOrigin[a] = float(np.float32(p.gridOrigin[a] + shift))
        p.boxCen[a] = float(np.float32(p.boxCen[a] + shift))
    pos = (sc.positions.astype(np.float64) + shift).astype(np.float32)
    return scenes.Scene(sc.name + "_far", p, sc.options, pos, sc.velocities.copy())


def test_far_from_the_origin_keeps_fp32_resolution(sphlib, orc):
    sc = shifted(SCENES["tiny"](), 256.0)
    steps = 200
    x, v = sc.positions.astype(np.float64), sc.velocities.astype(np.float64)
    for _ in range(steps):
        r = orc.step_plain(sc.params, sc.options, None, x, v, fp64=True)
        x, v = r["pos"], r["vel"]
    ulp = np.spacing(np.abs(x).astype(np.float32)).astype(np.float64)
    err = {}
    for mode in (0, 1):
        with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, rel_options(sc, mode)) as sim:
            sim.step(count=steps)
            err[mode] = np.abs(sim.positions().astype(np.float64) - x) / ulp
    # cell-relative: the FP64 trajectory up to the read-back's own rounding
    assert err[1].max() <= 1.0, err[1].max()
    # absolute: each step's x + dt v (a few 1e-6 .. 1e-5) is rounded to 3e-5
    assert err[0].max() > 2.0, err[0].max()


def test_launch_shapes_change_no_bit(sphlib):
    sc = obstacle_block()
    configs = [dict(forceVariant=0, prune=0, forceBlock=128, densityBlock=128),
               dict(forceVariant=1, prune=1, forceBlock=64, densityBlock=256),
               dict(forceVariant=2, prune=1, forceBlock=128, densityBlock=128),
               dict(forceVariant=2, prune=0, forceBlock=256, densityBlock=64)]
    outs = []
    for cfg in configs:
        with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, rel_options(sc),
                                       sc.boundary) as sim:
            sim.set_tuning(kahan=1, **cfg)
            for _ in range(3):
                sim.Advance()
            outs.append([sim.read(sphlib.FIELD_DENSITY), sim.read(sphlib.FIELD_ACCELERATION),
                         sim.positions(), sim.velocities()])
    for o in outs[1:]:
        for a, b in zip(outs[0], o):
            np.testing.assert_array_equal(a, b)


def test_trajectory_close_to_the_absolute_store(sphlib):
    """Near the origin both stores follow the same physics: after 50 steps of
    the 16,384-particle dam break their mean densities agree to 1e-4."""
    sc = scenes.config1()
    out = []
    for mode in (0, 1):
        with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, rel_options(sc, mode)) as sim:
            sim.step(count=50)
            sim.Advance()
            out.append(sim.read(sphlib.FIELD_DENSITY).astype(np.float64))
    assert abs(out[0].mean() - out[1].mean()) <= 1e-4 * out[0].mean()


def test_diagnostics_and_surface_use_absolute_positions(sphlib):
    sc = scenes.config1()
    res = []
    for mode in (0, 1):
        with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, rel_options(sc, mode)) as sim:
            sim.Advance()
            d = sim.diagnostics()
            res.append((d.potentialEnergy, d.mass, sim.surface_particles()))
    assert abs(res[0][0] - res[1][0]) <= 1e-6 * abs(res[0][0])
    assert res[0][1] == res[1][1]
    # the flags of a state that came through both stores alike
    assert (res[0][2] != res[1][2]).mean() < 0.01


def test_other_step_kinds_are_refused(sphlib):
    sc = SCENES["tiny"]()
    with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, rel_options(sc)) as sim:
        for mode in (sphlib.SPH_STEP_TWO_SCALE, sphlib.SPH_STEP_SUB_ONLY, sphlib.SPH_STEP_LEARNED):
            with pytest.raises(sphlib.SphError):
                sim.step(mode=mode)
        L = sphlib.load()
        ptr = ctypes.c_void_p()
        assert L.sph_device_pointer(sim._h, 0, ctypes.byref(ptr)) == 6  # SPH_ERR_NOT_SUPPORTED
        assert L.sph_device_pointer(sim._h, 1, ctypes.byref(ptr)) == 0


def test_grid_limit(sphlib):
    sc = SCENES["tiny"]()
    p = P.SimulationParameters.from_buffer_copy(bytes(sc.params))
    p.gridDim[2] = 1025
    with pytest.raises(sphlib.SphError):
        sphlib.ParticleSimulation(p, sc.positions, sc.velocities, rel_options(sc))
