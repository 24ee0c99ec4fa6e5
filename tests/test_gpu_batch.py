"""GPU checks of batched scenes (sph_create_batch).

A scene's arithmetic inside a batch is the single-scene arithmetic with its
own grid, constants and maps, so every scene's state, densities,
accelerations, sort permutation and cell tables must be bit-identical to the
same scene run alone (shifted by the scene's particle and cell offsets).
"""
import numpy as np
import pytest

from cudasphnew_gb300 import scenes

pytestmark = pytest.mark.gpu

EMPTY = -1  # 0xFFFFFFFF read as int32


def small_batch():
    return [scenes.batched_scene(n, f, 100 + k, f"b{k}")
            for k, (n, f) in enumerate(zip((1500, 4000, 700, 2500), (0.05, 0.2, 0.12, 0.08)))]


def with_skin(o, skin):
    o = type(o).from_buffer_copy(bytes(o))
    if skin is not None:
        o.neighbourSkin = skin
    return o


def run_alone(sphlib, sc, steps, skin=None):
    with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, with_skin(sc.options, skin),
                                   sc.boundary) as sim:
        sim.step(count=steps)
        h, ids, start, end = sim.cells()
        return dict(pos=sim.positions(), vel=sim.velocities(), rho=sim.read(sphlib.FIELD_DENSITY),
                    acc=sim.read(sphlib.FIELD_ACCELERATION), hash=h, ids=ids, start=start, end=end,
                    builds=sim.neighbour_builds())


def run_batch(sphlib, scs, steps, autotune=False, skin=None):
    with sphlib.ParticleSimulation.batch(scs, with_skin(scs[0].options, skin)) as sim:
        if autotune:
            sim.autotune(reps=2)
        sim.step(count=steps)
        fp, fc = sim.scene_ranges()
        h, ids, start, end = sim.cells()
        return fp, fc, dict(pos=sim.positions(), vel=sim.velocities(), rho=sim.read(sphlib.FIELD_DENSITY),
                            p=sim.read(sphlib.FIELD_PRESSURE), acc=sim.read(sphlib.FIELD_ACCELERATION),
                            hash=h, ids=ids, start=start, end=end, builds=sim.neighbour_builds())


def check_scene(k, fp, fc, b, a):
    p0, p1, c0, c1 = int(fp[k]), int(fp[k + 1]), int(fc[k]), int(fc[k + 1])
    for key in ("pos", "vel", "rho", "acc"):
        np.testing.assert_array_equal(b[key][p0:p1], a[key], err_msg=f"scene {k} {key}")
    # the scene's slice of the sorted arrays: its cells are [c0, c1), its
    # particles [p0, p1), and the sorted order inside is the scene's own
    np.testing.assert_array_equal(b["hash"][p0:p1], a["hash"] + c0)
    np.testing.assert_array_equal(b["ids"][p0:p1], a["ids"] + p0)
    st, en = b["start"][c0:c1], b["end"][c0:c1]
    np.testing.assert_array_equal(st == EMPTY, a["start"] == EMPTY)
    occ = a["start"] != EMPTY
    np.testing.assert_array_equal(st[occ], a["start"][occ] + p0)
    np.testing.assert_array_equal(en[occ], a["end"][occ] + p0)


@pytest.mark.parametrize("skin", [0.0, 0.1])
def test_batch_is_bit_identical_to_scenes_alone(sphlib, skin):
    scs = small_batch()
    steps = 6
    fp, fc, b = run_batch(sphlib, scs, steps, skin=skin)
    assert list(np.diff(fp)) == [sc.n for sc in scs]
    assert list(np.diff(fc)) == [sc.params.num_cells for sc in scs]
    for k, sc in enumerate(scs):
        check_scene(k, fp, fc, b, run_alone(sphlib, sc, steps, skin=skin))


def test_batch_rebuilds_each_scenes_lists_when_that_scene_would_alone(sphlib):
    """Scenes moving at different speeds rebuild their reused neighbour lists
    at different steps; each scene's results stay bit-identical to the scene
    run alone, and the batch's builds are the scenes' builds summed."""
    scs = small_batch()
    for k, sc in enumerate(scs):
        sc.velocities[:, 0] = 0.3 * k  # scene 0 at rest, scene 3 at 0.9 m/s
    steps = 40
    fp, fc, b = run_batch(sphlib, scs, steps)
    alone = [run_alone(sphlib, sc, steps) for sc in scs]
    for k in range(len(scs)):
        check_scene(k, fp, fc, b, alone[k])
    builds = [a["builds"] for a in alone]
    assert builds[0] < builds[-1] and len(set(builds)) > 1
    assert b["builds"] == sum(builds)


def test_batch_graph_steps_equal_eager_steps(sphlib):
    """Steps replayed from the captured step graph and steps launched one by
    one (no graph) give the same bits, with scenes building their lists at
    different steps: the per-scene decisions made on the device alone select
    which kernels work for which scene."""
    scs = small_batch()
    for k, sc in enumerate(scs):
        sc.velocities[:, 0] = 0.3 * k
    outs = []
    for graph in (True, False):
        with sphlib.ParticleSimulation.batch(scs, with_skin(scs[0].options, None)) as sim:
            if graph:
                sim.step(count=40)
            else:
                for _ in range(40):
                    sim.step()
            h, ids, start, end = sim.cells()
            outs.append(dict(pos=sim.positions(), vel=sim.velocities(), rho=sim.read(sphlib.FIELD_DENSITY),
                             acc=sim.read(sphlib.FIELD_ACCELERATION), hash=h, ids=ids, start=start, end=end,
                             builds=sim.neighbour_builds()))
    assert len(scs) < outs[0]["builds"] < 40 * len(scs)
    for key in outs[0]:
        np.testing.assert_array_equal(outs[1][key], outs[0][key], err_msg=key)


def test_batch_autotune_keeps_results(sphlib):
    scs = small_batch()
    _, _, b0 = run_batch(sphlib, scs, 4)
    _, _, b1 = run_batch(sphlib, scs, 4, autotune=True)
    for key in ("pos", "vel", "rho", "acc"):
        np.testing.assert_array_equal(b0[key], b1[key])


def test_batch_write_keeps_scene_lanes(sphlib):
    scs = small_batch()
    with sphlib.ParticleSimulation.batch(scs, scs[0].options) as sim:
        sim.step(count=2)
        pos, vel = sim.positions(), sim.velocities()
        sim.write_state(pos, vel)  # a host round trip must not lose the scene of each particle
        sim.step(count=3)
        got = sim.positions()
    with sphlib.ParticleSimulation.batch(scs, scs[0].options) as ref:
        ref.step(count=5)
        np.testing.assert_array_equal(got, ref.positions())


def test_batch_takes_plain_steps_only(sphlib):
    scs = small_batch()
    with sphlib.ParticleSimulation.batch(scs, scs[0].options) as sim:
        for mode in (sphlib.SPH_STEP_TWO_SCALE, sphlib.SPH_STEP_SUB_ONLY, sphlib.SPH_STEP_LEARNED):
            with pytest.raises(sphlib.SphError):
                sim.step(mode=mode)
        with pytest.raises(sphlib.SphError):
            sim.diagnostics()
        sim.step()
        with pytest.raises(sphlib.SphError):
            sim.surface_particles()  # per scene: not for batched handles


def test_batched_workload_runs(sphlib):
    """The 64-scene workload (about 4.4M particles): a few steps, finite."""
    scs = scenes.config4()
    with sphlib.ParticleSimulation.batch(scs, scs[0].options) as sim:
        sim.step(count=5)
        sim.synchronize()
        fp, fc = sim.scene_ranges()
        pos = sim.positions()
    assert len(fp) == 65 and fp[-1] == sum(sc.n for sc in scs)
    assert np.isfinite(pos).all()
    # every particle stays inside its own scene's box
    for k, sc in enumerate(scs):
        p = pos[fp[k]:fp[k + 1]]
        lo = np.asarray(sc.params.boxCen) - np.asarray(sc.params.boxDim)
        hi = np.asarray(sc.params.boxCen) + np.asarray(sc.params.boxDim)
        assert (p >= lo - 1e-6).all() and (p <= hi + 1e-6).all()


def spread(scs, count):
    """Indices of `count` scenes spread over the size range (smallest to largest)."""
    order = np.argsort([sc.n for sc in scs], kind="stable")
    return sorted({int(order[int(round(q))]) for q in np.linspace(0, len(scs) - 1, count)})


def scene_slice(k, fp, fc, b):
    """Scene k's part of a batch result, with the particle and cell offsets removed."""
    p0, p1, c0, c1 = int(fp[k]), int(fp[k + 1]), int(fc[k]), int(fc[k + 1])
    st, en = b["start"][c0:c1].copy(), b["end"][c0:c1].copy()
    occ = st != EMPTY
    st[occ] -= p0
    en[occ] -= p0
    return dict(hash=b["hash"][p0:p1] - c0, ids=b["ids"][p0:p1] - p0, start=st, end=en,
                **{key: b[key][p0:p1] for key in ("rho", "p", "acc", "pos", "vel")})


def test_batched_workload_matches_oracle_and_scenes_alone(sphlib, orc):
    """The full 64-scene workload (about 4.4M particles): after one step a
    mid-size scene matches the oracle (tables bit-exact, rho, p, a within the
    plain step's FP64 bars); after three steps eight scenes spread over the
    size range are bit-identical to the same scenes run alone."""
    from test_gpu_step import check_step, maps_for
    scs = scenes.config4()
    fp, fc, b = run_batch(sphlib, scs, 1)
    k = spread(scs, 3)[1]
    assert 20000 < scs[k].n < 120000
    check_step(orc, scs[k], scene_slice(k, fp, fc, b), maps_for(orc, scs[k]))
    steps = 3
    fp, fc, b = run_batch(sphlib, scs, steps)
    picked = spread(scs, 8)
    assert len(picked) == 8
    for k in picked:
        check_scene(k, fp, fc, b, run_alone(sphlib, scs[k], steps))
