"""GPU parity tests of the plain SPH step, through the C ABI (libsph_gb300.so).

Bars: hash, sort permutation and cell start/end tables bit-exact against the
oracle's FP32 restatement; density, pressure and acceleration within 1e-5 of
the FP64 oracle's per-particle magnitude scale (sum of |terms|, see
oracle/sph_oracle.cpp); boundary maps bit-exact.
"""
import numpy as np
import pytest

from cudasphnew_gb300 import params as P
from cudasphnew_gb300 import scenes

pytestmark = pytest.mark.gpu

TOL = 1e-5  # relative to the FP64 oracle's magnitude scale


def run_gpu(sphlib, sc, steps=1, graph=False):
    with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options, sc.boundary) as sim:
        if graph:
            sim.step(count=steps)
        else:
            for _ in range(steps):
                sim.Advance()
        sim.synchronize()
        h, ids, start, end = sim.cells()
        return dict(hash=h, ids=ids, start=start, end=end, rho=sim.read(sphlib.FIELD_DENSITY),
                    p=sim.read(sphlib.FIELD_PRESSURE), acc=sim.read(sphlib.FIELD_ACCELERATION),
                    pos=sim.positions(), vel=sim.velocities(),
                    sd=sim.read(sphlib.FIELD_SIMULATION_DATA))


def maps_for(orc, sc):
    return orc.boundary_maps(sc.boundary) if sc.boundary is not None else None


def check_step(orc, sc, g, bm):
    r32 = orc.step_plain(sc.params, sc.options, bm, sc.positions, sc.velocities)
    r64 = orc.step_plain(sc.params, sc.options, bm, sc.positions, sc.velocities, fp64=True)
    np.testing.assert_array_equal(g["hash"], r32["hash"])
    np.testing.assert_array_equal(g["ids"], r32["ids"])
    np.testing.assert_array_equal(g["start"], r32["start"])
    np.testing.assert_array_equal(g["end"], r32["end"])
    assert (np.abs(g["rho"] - r64["rho"]) <= TOL * r64["scale_rho"]).all()
    kscale = float(sc.params.gasStiffness) * (r64["rho"] + float(sc.params.restDensity))
    assert (np.abs(g["p"] - r64["p"]) <= TOL * kscale).all()
    assert (np.abs(g["acc"] - r64["acc"]).max(1) <= TOL * r64["scale_acc"]).all()
    # the wall terms follow the reference's FP32 operation order exactly, so
    # against the FP32 restatement they must agree at their own magnitude too
    assert (np.abs(g["acc"] - r32["acc"]).max(1) <= TOL * r64["scale_acc_direct"]).all()
    # new state: v' = v + dt a, x' = x + dt v' (+ collision), errors bounded by dt * acc error
    dt = float(sc.params.timeStep)
    vtol = dt * TOL * r64["scale_acc"] + 4 * np.spacing(np.abs(r64["vel"]).max(1).astype(np.float32))
    assert (np.abs(g["vel"] - r64["vel"]).max(1) <= vtol).all()
    xtol = dt * vtol + 4 * np.spacing(np.abs(r64["pos"]).max(1).astype(np.float32))
    assert (np.abs(g["pos"] - r64["pos"]).max(1) <= xtol).all()
    return r32, r64


def obstacle_block():
    """Particles packed around the sphere + cone obstacle, many within the wall band."""
    sc = scenes.small_obstacle()
    d = sc.boundary
    pos = scenes.lattice_block(40, 40, 40, (0.25, 0.25, 0.0), P.SPACING, 11, 0.01 * P.H)
    import oracle
    bm = oracle.boundary_maps(d)
    dist = -oracle.tex3d(bm, 0, pos.astype(np.float64))  # distWall > 0 in the fluid
    keep = dist > 0.3 * P.H
    pos = pos[keep]
    p = P.dam_break_params((0, 0, 0), (1, 1, 0.5), len(pos))
    return scenes.Scene("obstacle_block", p, sc.options, pos, np.zeros_like(pos), d)


SCENES = {
    "tiny": lambda: scenes.dam_break(8, 8, 8, (0, 0, 0), (0.5, 0.5, 0.5), 3, "tiny", 1),
    "config1": scenes.config1,
    "example01": scenes.example01,
    "obstacle_block": obstacle_block,
}


@pytest.mark.parametrize("name", list(SCENES))
def test_one_step_parity(sphlib, orc, name):
    sc = SCENES[name]()
    g = run_gpu(sphlib, sc)
    check_step(orc, sc, g, maps_for(orc, sc))


def test_wall_terms_are_exercised(orc):
    sc = obstacle_block()
    bm = orc.boundary_maps(sc.boundary)
    dist = -orc.tex3d(bm, 0, sc.positions.astype(np.float64))
    assert (dist < sc.boundary.restDistance).sum() > 500


def test_single_particle(sphlib, orc):
    sc = scenes.dam_break(1, 1, 1, (0.4, 0.4, 0.4), (1, 1, 1), 1, "one", 1)
    g = run_gpu(sphlib, sc, steps=1)
    check_step(orc, sc, g, None)


def test_simulation_data_layout(sphlib, orc):
    sc = SCENES["tiny"]()
    n = sc.n
    sd_in = np.zeros((n, 10), np.float32)
    sd_in[:, 0] = 0.5  # SD_MASS is carried, never read by the step
    sd_in[:, 6:9] = 0.01
    sd_in[:, 9] = 7.0  # SD_ENERGY likewise
    with sphlib.ParticleSimulation(sc.params, sc.positions, options=sc.options,
                                   simulation_data=sd_in) as sim:
        sim.Advance()
        sd = sim.read(sphlib.FIELD_SIMULATION_DATA)
        rho = sim.read(sphlib.FIELD_DENSITY)
        acc = sim.read(sphlib.FIELD_ACCELERATION)
        vel = sim.velocities()
    np.testing.assert_array_equal(sd[:, 0], 0.5)
    np.testing.assert_array_equal(sd[:, 1], rho)
    np.testing.assert_array_equal(sd[:, 3:6], acc)
    np.testing.assert_array_equal(sd[:, 6:9], vel)
    np.testing.assert_array_equal(sd[:, 9], 7.0)


def test_per_step_parity_over_a_trajectory(sphlib, orc):
    """Each of 20 steps is checked from the GPU's own state of the step before."""
    sc = scenes.config1()
    with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options) as sim:
        for k in range(20):
            x0, v0 = sim.positions(), sim.velocities()
            sim.Advance()
            h, ids, start, end = sim.cells()
            g = dict(hash=h, ids=ids, start=start, end=end, rho=sim.read(sphlib.FIELD_DENSITY),
                     p=sim.read(sphlib.FIELD_PRESSURE), acc=sim.read(sphlib.FIELD_ACCELERATION),
                     pos=sim.positions(), vel=sim.velocities())
            step = scenes.Scene("c1", sc.params, sc.options, x0, v0)
            check_step(orc, step, g, None)


def test_graph_replay_matches_eager(sphlib):
    sc = scenes.example01()
    a = run_gpu(sphlib, sc, steps=7, graph=False)
    b = run_gpu(sphlib, sc, steps=7, graph=True)
    for k in ("ids", "rho", "acc", "pos", "vel"):
        np.testing.assert_array_equal(a[k], b[k])


def test_deterministic(sphlib):
    sc = scenes.small_obstacle()
    a = run_gpu(sphlib, sc, steps=5)
    b = run_gpu(sphlib, sc, steps=5)
    for k in ("ids", "rho", "acc", "pos", "vel"):
        np.testing.assert_array_equal(a[k], b[k])


def test_trajectory_density_error_vs_fp64(sphlib, orc):
    """50 steps of config 1's scene: mean and max density error of the GPU
    trajectory against an FP64 replay from the same initial state."""
    sc = scenes.config1()
    g = run_gpu(sphlib, sc, steps=50, graph=True)
    x = sc.positions.astype(np.float64)
    v = sc.velocities.astype(np.float64)
    for _ in range(50):
        r = orc.step_plain(sc.params, sc.options, None, x, v, fp64=True)
        x, v = r["pos"], r["vel"]
    rel = np.abs(g["rho"] - r["rho"]) / r["rho"]
    assert rel.mean() < 1e-5 and rel.max() < 1e-3


@pytest.mark.parametrize("name", ["example01", "obstacle"])
def test_boundary_maps_match_oracle(sphlib, orc, name):
    if name == "example01":
        p = P.example01_params()
        d = P.example01_boundary(p)
    else:
        d = scenes.small_obstacle().boundary
    dist, dens, visc = sphlib.boundary_maps(d)
    bm = orc.boundary_maps(d)
    np.testing.assert_array_equal(dist, bm.dist)
    np.testing.assert_allclose(dens, bm.dens, rtol=1e-6, atol=1e-6 * float(bm.dens.max()))
    np.testing.assert_allclose(visc, bm.visc, rtol=1e-6, atol=1e-6 * float(bm.visc.max()))


def test_far_particle_wraps_like_the_reference(sphlib, orc):
    """compute_particle_hash wraps coordinates beyond the grid with `% dim`
    (particle_simulation.cu:108-112): no error, same cell as the reference."""
    sc = SCENES["tiny"]()
    pos = sc.positions.copy()
    pos[3] = (5.0, 5.0, 5.0)
    with sphlib.ParticleSimulation(sc.params, pos, options=sc.options) as sim:
        sim.Advance()
        sim.synchronize()
        h, ids, start, end = sim.cells()
    r = orc.hash_sort_cells(sc.params, pos)
    np.testing.assert_array_equal(h, r[0])
    np.testing.assert_array_equal(ids, r[1])


def test_out_of_domain_is_reported(sphlib):
    """Far below the origin the truncated coordinate is negative and so is the
    hash: the reference would write outside its cell table; here the step
    clamps the write and reports SPH_ERR_OUT_OF_DOMAIN."""
    sc = SCENES["tiny"]()
    pos = sc.positions.copy()
    pos[3] = (-5.0, -5.0, -5.0)
    with sphlib.ParticleSimulation(sc.params, pos, options=sc.options) as sim:
        sim.Advance()
        with pytest.raises(sphlib.SphError) as e:
            sim.synchronize()
        assert e.value.status == 4


def test_non_finite_is_reported(sphlib):
    sc = SCENES["tiny"]()
    pos = sc.positions.copy()
    pos[0, 1] = np.nan
    with sphlib.ParticleSimulation(sc.params, pos, options=sc.options) as sim:
        sim.Advance()
        with pytest.raises(sphlib.SphError) as e:
            sim.synchronize()
        assert e.value.status == 7


def test_bind_changes_parameters(sphlib, orc):
    sc = SCENES["tiny"]()
    p2 = P.dam_break_params((0, 0, 0), (0.5, 0.5, 0.5), sc.n)
    p2.gravity = 0.0
    with sphlib.ParticleSimulation(sc.params, sc.positions, options=sc.options) as sim:
        sim.Bind(p2)
        sim.Advance()
        acc = sim.read(sphlib.FIELD_ACCELERATION)
    r64 = orc.step_plain(p2, sc.options, None, sc.positions, sc.velocities, fp64=True)
    assert (np.abs(acc - r64["acc"]).max(1) <= TOL * r64["scale_acc"]).all()


def test_counts_and_stage_timing(sphlib):
    sc = SCENES["tiny"]()
    with sphlib.ParticleSimulation(sc.params, sc.positions, options=sc.options) as sim:
        sim.set_stage_timing(4)
        for _ in range(3):
            sim.Advance()
        t = sim.stage_times()
        plain = ("hash_count", "cell_scan", "scatter", "rank_gather", "density", "force_integrate")
        assert all(t[k][1] == 3 and t[k][0] > 0 for k in plain)
        # the two-scale stages are not counted in plain steps
        assert all(c == 0 and ms == 0 for k, (ms, c) in t.items() if k not in plain)
        assert sim.GetNumTimesSteps() == 3 and sim.GetNumParticles() == sc.n
        assert sim.device_pointer(0) != 0


def test_full_size_one_step(sphlib, orc):
    """The 1,048,576-particle obstacle scene: one step against the oracle."""
    sc = scenes.config2()
    g = run_gpu(sphlib, sc)
    r32, r64 = check_step(orc, sc, g, maps_for(orc, sc))
    # size-independent properties
    assert np.array_equal(np.sort(g["ids"]), np.arange(sc.n))
    assert (np.diff(g["hash"]) >= 0).all()


@pytest.mark.parametrize("kahan", [0, 1])
def test_tunings_are_bit_identical(sphlib, kahan):
    """Block sizes, the force form and stencil pruning change no result bit."""
    sc = obstacle_block()
    configs = [dict(forceVariant=0, prune=0, forceBlock=128, densityBlock=128),
               dict(forceVariant=1, prune=1, forceBlock=64, densityBlock=256),
               dict(forceVariant=1, prune=0, forceBlock=256, densityBlock=64),
               dict(forceVariant=0, prune=1, forceBlock=256, densityBlock=128),
               dict(forceVariant=2, prune=1, forceBlock=128, densityBlock=128),
               dict(forceVariant=2, prune=0, forceBlock=64, densityBlock=64),
               dict(forceVariant=3, prune=1, forceBlock=128, densityBlock=128),
               dict(forceVariant=3, prune=0, forceBlock=256, densityBlock=256)]
    outs = []
    for cfg in configs:
        with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options,
                                       sc.boundary) as sim:
            sim.set_tuning(kahan=kahan, **cfg)
            for _ in range(3):
                sim.Advance()
            outs.append([sim.read(sphlib.FIELD_DENSITY), sim.read(sphlib.FIELD_ACCELERATION),
                         sim.positions(), sim.velocities()])
    for o in outs[1:]:
        for a, b in zip(outs[0], o):
            np.testing.assert_array_equal(a, b)


def test_autotune_leaves_state_untouched(sphlib):
    sc = scenes.config1()
    with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options) as sim, \
            sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options) as ref:
        for _ in range(3):
            sim.Advance()
            ref.Advance()
        before = [sim.read(f) for f in (sphlib.FIELD_DENSITY, sphlib.FIELD_ACCELERATION,
                                        sphlib.FIELD_VERTEX_DATA, sphlib.FIELD_VELOCITY)]
        cells_before = sim.cells()
        t = sim.autotune(reps=2)
        assert t.densityBlock in (64, 128, 256) and t.forceVariant in (0, 1, 2, 3)
        after = [sim.read(f) for f in (sphlib.FIELD_DENSITY, sphlib.FIELD_ACCELERATION,
                                       sphlib.FIELD_VERTEX_DATA, sphlib.FIELD_VELOCITY)]
        for a, b in zip(before, after):
            np.testing.assert_array_equal(a, b)
        for a, b in zip(cells_before, sim.cells()):
            np.testing.assert_array_equal(a, b)
        sim.Advance()
        ref.Advance()
        np.testing.assert_array_equal(sim.positions(), ref.positions())


def test_fp64_diagnostics(sphlib):
    """sph_get_diagnostics against an FP64 numpy sum of the same state."""
    sc = scenes.config1()
    with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options, sc.boundary) as sim:
        d0 = sim.diagnostics()
        assert d0.densityMean == 0.0 and d0.densityMaxRelError == 0.0
        sim.step(count=20)
        d = sim.diagnostics()
        d2 = sim.diagnostics()
        x = sim.positions().astype(np.float64)
        v = sim.velocities().astype(np.float64)
        rho = sim.read(sphlib.FIELD_DENSITY).astype(np.float64)
    assert bytes(d) == bytes(d2)  # fixed reduction order
    m = float(np.float32(sc.params.particleMass))
    g = float(np.float32(sc.params.gravity))
    rest = float(np.float32(sc.params.restDensity))
    n = len(x)
    rel = 1e-12
    assert abs(d.mass - n * m) <= rel * n * m
    mom = m * v.sum(0)
    scale = m * np.abs(v).sum(0)
    for a in range(3):
        assert abs(d.momentum[a] - mom[a]) <= rel * scale[a] + 1e-300
    ke = 0.5 * m * (v * v).sum()
    assert abs(d.kineticEnergy - ke) <= rel * ke
    ax = sc.options.gravityAxis
    pe = m * g * x[:, ax].sum()
    assert abs(d.potentialEnergy - pe) <= rel * m * g * np.abs(x[:, ax]).sum()
    # the density terms are of the last density pass, which saw the state
    # before the last integration; FIELD_DENSITY reads that same pass
    assert abs(d.densityMean - rho.mean()) <= rel * rho.mean()
    assert d.densityMaxRelError == np.abs(rho - rest).max() / rest or \
        abs(d.densityMaxRelError - np.abs(rho - rest).max() / rest) <= 1e-15
    # the dam break falls: the potential energy drops and kinetic energy appears
    assert d.kineticEnergy > 0.0


def test_surface_particles(sphlib):
    """CreateIsParticleSurfaceList: fewer than nPartTresh neighbours within h,
    or a neighbour centre of mass farther than cmDistanceThresh * h, in the
    state that entered the last step (brute force in float64)."""
    sc = scenes.dam_break(12, 12, 8, (0, 0, 0), (0.5, 0.5, 0.5), 3, "surface", 1)
    with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options) as sim:
        sim.step(count=5)
        x = sim.positions().astype(np.float64)
        sim.Advance()
        flags = sim.surface_particles()
    h = float(np.float32(sc.params.compactSupport))
    d = x[:, None, :] - x[None, :, :]
    r2 = (d * d).sum(2)
    nb = (r2 <= h * h) & ~np.eye(len(x), dtype=bool)
    cnt = nb.sum(1)
    cm = (nb[..., None] * x[None]).sum(1) / np.maximum(cnt, 1)[:, None]
    off = np.linalg.norm(cm - x, axis=1)
    ref = (cnt < sc.params.nPartTresh) | ((cnt > 0) & (off > sc.params.cmDistanceThresh * h))
    # the GPU tests r^2 in float: a pair exactly at h may count differently
    assert (flags != ref).sum() <= 2
    assert 0 < flags.sum() < len(flags)


def test_time_kernel_leaves_the_plain_step_state(sphlib):
    """sph_time_kernel repeats the density and force kernels on the last
    step's sorted state: the state after it is the state after the step."""
    sc = scenes.config1()
    with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options) as sim, \
            sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options) as ref:
        for s in (sim, ref):
            s.step(count=4)
        assert sim.time_kernel("density", 5) > 0.0
        assert sim.time_kernel("force", 5) > 0.0
        np.testing.assert_array_equal(sim.positions(), ref.positions())
        np.testing.assert_array_equal(sim.velocities(), ref.velocities())
        np.testing.assert_array_equal(sim.read(sphlib.FIELD_DENSITY), ref.read(sphlib.FIELD_DENSITY))
        sim.step(count=2)
        ref.step(count=2)
        np.testing.assert_array_equal(sim.positions(), ref.positions())


@pytest.mark.parametrize("skin", [0.0, 0.1])
def test_scan_wait_give_up_is_reported_and_recovers(sphlib, orc, skin):
    """The cell scan's look-back waits are bounded; a wait that gives up
    latches SPH_ERR_DEVICE_WAIT.  SPH_SCAN_WAIT_LIMIT=-1 makes every wait give
    up at its first poll (read at each eagerly enqueued step): the step must
    stay inside its buffers, report the condition once, and the next step from
    a written state must be the plain step again."""
    import os
    sc = scenes.config1()
    o = P.Options.from_buffer_copy(bytes(sc.options))
    o.neighbourSkin = skin
    with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, o) as sim:
        os.environ["SPH_SCAN_WAIT_LIMIT"] = "-1"
        try:
            sim.Advance()  # eager: the launch reads the limit
            with pytest.raises(sphlib.SphError) as e:
                sim.synchronize()
            assert e.value.status == 5  # SPH_ERR_DEVICE_WAIT
        finally:
            del os.environ["SPH_SCAN_WAIT_LIMIT"]
        sim.synchronize()  # reported once
        sim.write_state(sc.positions, sc.velocities)
        sim.Advance()
        g = dict(zip(("hash", "ids", "start", "end"), sim.cells()))
        g.update(rho=sim.read(sphlib.FIELD_DENSITY), p=sim.read(sphlib.FIELD_PRESSURE),
                 acc=sim.read(sphlib.FIELD_ACCELERATION), pos=sim.positions(), vel=sim.velocities())
    check_step(orc, sc, g, None)
