"""GPU checks of the reused neighbour lists (sph_options.neighbourSkin > 0).

A plain step either builds the lists (the reference's stencil rows first, in
its order, plus the rows within the skin radius) or reuses them (the state is
gathered into the working order of the build and only the recorded
candidates are visited).  The bars:
* a building step is bit-identical to the per-step search (skin 0): the
  extra candidates lie beyond h and add exactly nothing;
* every reusing step is checked like any plain step, from the GPU's own state
  before it: cell tables bit-exact against the FP32 restatement, density,
  pressure and acceleration within 1e-5 of the FP64 scale;
* the lists are built again before any pair can come within h unseen: a
  particle thrown at a block gains its neighbours in the step they arrive.
"""
import numpy as np
import pytest

from cudasphnew_gb300 import params as P
from cudasphnew_gb300 import scenes

from test_gpu_step import check_step, obstacle_block

pytestmark = pytest.mark.gpu


def with_skin(sc, skin):
    o = P.Options.from_buffer_copy(bytes(sc.options))
    o.neighbourSkin = skin
    return o


def state(sphlib, sim):
    h, ids, start, end = sim.cells()
    return dict(hash=h, ids=ids, start=start, end=end, rho=sim.read(sphlib.FIELD_DENSITY),
                p=sim.read(sphlib.FIELD_PRESSURE), acc=sim.read(sphlib.FIELD_ACCELERATION),
                pos=sim.positions(), vel=sim.velocities())


SCENES = {
    "tiny": lambda: scenes.dam_break(8, 8, 8, (0, 0, 0), (0.5, 0.5, 0.5), 3, "tiny", 1),
    "config1": scenes.config1,
    "obstacle_block": obstacle_block,
    "small_obstacle": scenes.small_obstacle,
}


@pytest.mark.parametrize("name", list(SCENES))
def test_building_step_equals_the_per_step_search(sphlib, name):
    sc = SCENES[name]()
    outs = []
    for skin in (0.0, 0.1, 0.4):
        with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, with_skin(sc, skin),
                                       sc.boundary) as sim:
            sim.Advance()
            outs.append(state(sphlib, sim))
            assert sim.neighbour_builds() == (1 if skin > 0 else 0)
    for o in outs[1:]:
        for k in outs[0]:
            np.testing.assert_array_equal(o[k], outs[0][k], err_msg=k)


def moving_scene(speed, seed=5):
    sc = scenes.dam_break(16, 16, 8, (0.1, 0.1, 0.1), (0.5, 0.5, 0.5), seed, "moving", 1)
    rng = np.random.default_rng(seed)
    sc.velocities[:] = rng.uniform(-speed, speed, sc.velocities.shape).astype(np.float32)
    return sc


def test_graph_steps_equal_eager_steps(sphlib):
    """Steps replayed from the captured step graph and steps launched one by
    one (no graph) give the same bits, across builds and reuses: the decision
    made on the device alone selects which kernels work in each step."""
    sc = moving_scene(1.0)
    outs = []
    for graph in (True, False):
        with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, with_skin(sc, 0.1),
                                       sc.boundary) as sim:
            if graph:
                sim.step(count=24)
            else:
                for _ in range(24):
                    sim.step()
            outs.append(state(sphlib, sim) | {"builds": sim.neighbour_builds()})
    assert 1 < outs[0]["builds"] < 24
    for k in outs[0]:
        np.testing.assert_array_equal(outs[1][k], outs[0][k], err_msg=k)


def test_reusing_steps_match_the_oracle_across_builds(sphlib, orc):
    """12 steps at up to 2 m/s per axis (up to 3.5e-4 m per step against a
    rebuild distance of 0.45 * 0.1 h = 1.1e-3 m): the lists are built every few
    steps; each step is checked from the state before it."""
    sc = moving_scene(2.0)
    with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options) as sim:
        for k in range(12):
            x0, v0 = sim.positions(), sim.velocities()
            sim.Advance()
            check_step(orc, scenes.Scene("moving", sc.params, sc.options, x0, v0), state(sphlib, sim), None)
        builds = sim.neighbour_builds()
    assert 2 <= builds <= 10, builds


def test_lists_are_rebuilt_before_a_pair_arrives(sphlib, orc):
    """A particle thrown at a resting block from just outside the skin radius,
    moving 0.6 of the rebuild distance per step (so the lists are reused for
    a step, then built again), must see the block's particles from the step
    it reaches them: its density is checked against the oracle at every step."""
    sc = scenes.dam_break(8, 8, 8, (0.1, 0.1, 0.1), (0.5, 0.5, 0.5), 3, "target", 1)
    h = float(sc.params.compactSupport)
    skin = float(sc.options.neighbourSkin)
    face = float(sc.positions[:, 0].max())
    mid = sc.positions[:, 1:].mean(0)
    bullet = np.array([[face + 1.12 * h, mid[0], mid[1]]], np.float32)
    pos = np.concatenate([sc.positions, bullet])
    vel = np.zeros_like(pos)
    dt = float(sc.params.timeStep)
    vel[-1, 0] = -0.6 * 0.45 * skin * h / dt
    p = P.SimulationParameters.from_buffer_copy(bytes(sc.params))
    p.numParticles = len(pos)
    inside = 0
    with sphlib.ParticleSimulation(p, pos, vel, sc.options) as sim:
        for k in range(14):
            x0, v0 = sim.positions(), sim.velocities()
            sim.Advance()
            check_step(orc, scenes.Scene("target", p, sc.options, x0, v0), state(sphlib, sim), None)
            if np.linalg.norm(x0[:-1] - x0[-1], axis=1).min() < 0.95 * h:
                inside += 1
        builds = sim.neighbour_builds()
    assert inside >= 4, inside  # steps in which a missed pair would show in the bullet's density
    assert 5 <= builds <= 9, builds  # every second step: reused once, then built again


def test_writes_and_other_steps_rebuild_the_lists(sphlib):
    """Written positions keep the lists while every particle stays within the
    rebuild distance of the build; other step kinds always rebuild them."""
    sc = moving_scene(0.01)
    limit = 0.45 * float(sc.options.neighbourSkin) * float(sc.params.compactSupport)
    with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options) as sim:
        sim.step(count=3)
        assert sim.neighbour_builds() == 1
        x, v = sim.positions(), sim.velocities()
        sim.write_state(x, v)  # the same state: the lists stay
        sim.step(count=2)
        assert sim.neighbour_builds() == 1
        x = sim.positions()
        x[7, 2] += np.float32(1.5 * limit)  # one particle beyond the rebuild distance
        sim.write_state(x, sim.velocities())
        sim.step(count=2)
        assert sim.neighbour_builds() == 2
        sim.step(mode=sphlib.SPH_STEP_TWO_SCALE)
        sim.step(count=2)
        assert sim.neighbour_builds() == 3


def test_mixed_steps_follow_the_per_step_search(sphlib):
    """Plain steps over the lists between two-scale steps: the same trajectory
    as the per-step search up to the order of the neighbour sums."""
    sc = moving_scene(0.2)
    sc.options.childMode = 1
    for a in range(3):
        sc.options.splitMin[a] = 0.2
        sc.options.splitMax[a] = 0.3
    out = []
    for skin in (0.0, 0.1):
        with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, with_skin(sc, skin)) as sim:
            for mode in (0, 0, 0, 1, 0, 0, 1, 0):
                sim.step(mode=mode)
            out.append((sim.positions(), sim.velocities(), sim.read(sphlib.FIELD_DENSITY)))
    x0, v0, r0 = out[0]
    x1, v1, r1 = out[1]
    assert np.abs(x1 - x0).max() < 1e-6
    assert np.abs(v1 - v0).max() < 1e-4 * max(1.0, np.abs(v0).max())
    assert (np.abs(r1 - r0) <= 1e-5 * r0).all()


def test_full_size_reusing_steps(sphlib, orc):
    """The 1,048,576-particle obstacle scene: the third step (reusing the
    lists) against the oracle from the GPU's state before it."""
    sc = scenes.config2()
    bm = orc.boundary_maps(sc.boundary)
    with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options, sc.boundary) as sim:
        sim.step(count=2)
        x0, v0 = sim.positions(), sim.velocities()
        sim.Advance()
        assert sim.neighbour_builds() == 1
        check_step(orc, scenes.Scene("c2", sc.params, sc.options, x0, v0, sc.boundary), state(sphlib, sim), bm)
