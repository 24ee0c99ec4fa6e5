"""GPU parity of the two-scale pass (AdvanceTwoScale / AdvanceSubParticles).

Particle states, the three-way lists, the child list and the fine level's
hash / permutation / cell tables are bit-exact against the oracle's FP32
restatement fed the GPU's own coarse results; fine-level densities and
accelerations are within 1e-5 of the FP64 restatement's magnitude scale.
"""
import numpy as np
import pytest

from cudasphnew_gb300 import scenes

pytestmark = pytest.mark.gpu

TOL = 1e-5


def small_scene(child_mode=0):
    sc = scenes.two_scale(nb=24, region=(0.1, 0.2), box=0.5, name="two_scale_small")
    sc.options.childMode = child_mode
    return sc


def merge_scene():
    """Persistent children; the block moves down at 1 m/s with the split
    region's lower faces just below a lattice plane, so split parents leave
    the region within a few steps."""
    sc = scenes.two_scale(nb=24, region=(0.106, 0.2), box=0.5, name="two_scale_merge")
    sc.options.childMode = 1
    sc.velocities[:, 2] = -1.0
    return sc


def coarse_inputs(sphlib, sim):
    h, ids, start, end = sim.cells(0)
    return dict(rho=sim.read(sphlib.FIELD_DENSITY), p=sim.read(sphlib.FIELD_PRESSURE), ids=ids, start=start,
                end=end)


def gpu_two_scale(sphlib, sim):
    c = sim.counts()
    sh, sids, sstart, send = sim.cells(1)
    sd = sim.read(sphlib.FIELD_SUB_SIMULATION_DATA)
    return dict(state=sim.read(sphlib.FIELD_STATE), split=sim.read(sphlib.FIELD_SPLIT_IDS),
                boundary=sim.read(sphlib.FIELD_BOUNDARY_IDS), default=sim.read(sphlib.FIELD_DEFAULT_IDS),
                sub_ids=sim.read(sphlib.FIELD_SUB_IDS), sub_hash=sh, sorted_sub_ids=sids, sub_start=sstart,
                sub_end=send, sub_pos=sim.read(sphlib.FIELD_SUB_VERTEX_DATA), sub_rho=sd[:, 1], sub_p=sd[:, 2],
                sub_acc=sd[:, 3:6], sub_vel=sd[:, 6:9], counts=c)


def check_against_oracle(orc, sc, g, o32, o64, x0, v0, coarse):
    for T in (o32, o64):
        T.part(sc.params, sc.options, x0, v0, coarse["rho"], coarse["p"], coarse["ids"], coarse["start"],
               coarse["end"])
    for key in ("state", "split", "boundary", "default", "sub_ids", "sub_hash", "sorted_sub_ids", "sub_start",
                "sub_end"):
        np.testing.assert_array_equal(g[key], o32.get(key), err_msg=key)
    reg = g["sub_ids"][: 8 * len(g["split"])]
    bnd = g["sub_ids"][8 * len(g["split"]):]
    rho64 = o64.get("sub_rho")
    # fine densities of regular children: all-positive sums
    assert (np.abs(g["sub_rho"][reg] - rho64[reg]) <= TOL * rho64[reg]).all()
    # projected (mean) densities of boundary children
    assert (np.abs(g["sub_rho"][bnd] - rho64[bnd]) <= TOL * np.abs(rho64[bnd]) + 1e-3).all()
    acc64 = o64.get("sub_acc")
    scale = o64.get("sub_scale_acc")
    err = np.abs(g["sub_acc"][reg] - acc64[reg]).max(1)
    assert (err <= TOL * scale[reg]).all()
    dt = float(sc.params.timeStepSubParticles)
    pos64 = o64.get("sub_pos")
    ids = g["sub_ids"]
    tol = dt * dt * TOL * np.maximum(scale[ids], 1.0) + 4 * np.spacing(np.abs(pos64[ids]).max(1).astype(np.float32))
    assert (np.abs(g["sub_pos"][ids] - pos64[ids]).max(1) <= tol + 1e-7).all()


def test_two_scale_step_matches_oracle(sphlib, orc):
    sc = small_scene()
    o32 = orc.TwoScale(sc.n)
    o64 = orc.TwoScale(sc.n, fp64=True)
    with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options) as sim:
        for step in range(3):
            x0, v0 = sim.positions(), sim.velocities()
            sim.AdvanceTwoScale()
            g = gpu_two_scale(sphlib, sim)
            assert g["counts"].numParticlesSplit > 0 and g["counts"].numParticlesBoundary > 0
            check_against_oracle(orc, sc, g, o32, o64, x0, v0, coarse_inputs(sphlib, sim))


def test_two_scale_coarse_step_is_the_plain_step_with_walls(sphlib, orc):
    sc = small_scene()
    with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options) as sim:
        sim.AdvanceTwoScale()
        pos, acc = sim.positions(), sim.read(sphlib.FIELD_ACCELERATION)
    r64 = orc.step_plain(sc.params, sc.options, None, sc.positions, sc.velocities, fp64=True)
    assert (np.abs(acc - r64["acc"]).max(1) <= TOL * r64["scale_acc"]).all()
    assert np.abs(pos - r64["pos"]).max() < 1e-6


def test_state_lists_consistent(sphlib):
    """split = particles in the region; boundary = the rest within h of one."""
    sc = small_scene()
    with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options) as sim:
        sim.AdvanceTwoScale()
        state = sim.read(sphlib.FIELD_STATE)
        split = sim.read(sphlib.FIELD_SPLIT_IDS)
        boundary = sim.read(sphlib.FIELD_BOUNDARY_IDS)
        default = sim.read(sphlib.FIELD_DEFAULT_IDS)
        sub = sim.read(sphlib.FIELD_SUB_IDS)
    x = sc.positions
    inside = np.all((x >= 0.1) & (x <= 0.2), axis=1)
    np.testing.assert_array_equal(split, np.nonzero(inside)[0])
    assert len(split) + len(boundary) + len(default) == sc.n
    assert set(boundary).isdisjoint(split)
    np.testing.assert_array_equal(state[split] & 3, 3)
    np.testing.assert_array_equal(state[boundary] & 3, 2)
    np.testing.assert_array_equal(state[default] & 3, 0)
    np.testing.assert_array_equal(sub, np.concatenate([8 * np.repeat(split, 8) + np.tile(np.arange(8), len(split)),
                                                       8 * np.repeat(boundary, 8)
                                                       + np.tile(np.arange(8), len(boundary))]))


def test_sub_only_step(sphlib, orc):
    sc = small_scene()
    o64 = orc.TwoScale(sc.n, fp64=True)
    with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options) as sim:
        x0, v0 = sim.positions(), sim.velocities()
        sim.AdvanceTwoScale()
        co = coarse_inputs(sphlib, sim)
        o64.part(sc.params, sc.options, x0, v0, co["rho"], co["p"], co["ids"], co["start"], co["end"])
        before = sim.read(sphlib.FIELD_SUB_VERTEX_DATA)
        sim.AdvanceSubParticles()
        after = sim.read(sphlib.FIELD_SUB_VERTEX_DATA)
        ids = sim.read(sphlib.FIELD_SUB_IDS)
        xnow = sim.positions()
    assert np.abs(after[ids] - before[ids]).max() > 0
    assert np.isfinite(after[ids]).all()
    # the oracle's sub-only step from the same coarse tables and current coarse positions
    import ctypes
    L = orc.lib()
    fn = L.orc_ts_sub_only_f64
    arrs = [np.ascontiguousarray(a, np.float64) for a in (xnow, co["rho"], co["p"])]
    ints = [np.ascontiguousarray(a, np.int32) for a in (co["ids"], co["start"], co["end"])]
    assert fn(o64._h, ctypes.byref(sc.params), ctypes.byref(sc.options), *[orc._ptr(a) for a in arrs],
              *[orc._ptr(a) for a in ints]) == 0
    pos64 = o64.get("sub_pos")
    assert np.abs(after[ids] - pos64[ids]).max() < 1e-5


def test_persistent_children_and_merge_back(sphlib, orc):
    sc = merge_scene()
    n = sc.n
    o32 = orc.TwoScale(n)
    o64 = orc.TwoScale(n, fp64=True)
    dt = np.float32(sc.params.timeStep)
    merged = kept = 0
    with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options) as sim:
        sp = sv = None
        for step in range(6):
            x0, v0 = sim.positions(), sim.velocities()
            if step > 0:
                sp = sim.read(sphlib.FIELD_SUB_VERTEX_DATA)
                sv = sim.read(sphlib.FIELD_SUB_SIMULATION_DATA)[:, 6:9].copy()
                for T in (o32, o64):
                    T.set_children(sp, sv)
            sim.AdvanceTwoScale()
            g = gpu_two_scale(sphlib, sim)
            check_against_oracle(orc, sc, g, o32, o64, x0, v0, coarse_inputs(sphlib, sim))
            code = g["state"].astype(np.int32) & 15
            if step == 0:
                continue
            # parents split in both steps keep their children: not re-seeded
            stay = np.nonzero(code == 15)[0]
            kept += len(stay)
            # parents leaving the split class: mean of the children, then integrated
            leave = np.nonzero((((code >> 2) & 1) == 1) & ((code & 1) == 0))[0]
            if len(leave) == 0:
                continue
            merged += len(leave)
            cx = sp.reshape(n, 8, 3)[leave]
            cv = sv.reshape(n, 8, 3)[leave]
            mx = np.zeros((len(leave), 3), np.float32)
            mv = np.zeros((len(leave), 3), np.float32)
            for k in range(8):
                mx += cx[:, k]
                mv += cv[:, k]
            mx *= np.float32(0.125)
            mv *= np.float32(0.125)
            acc = sim.read(sphlib.FIELD_ACCELERATION)[leave]
            v = mv + dt * acc
            x = mx + dt * v
            gx, gv = sim.positions()[leave], sim.velocities()[leave]
            np.testing.assert_allclose(gv, v, rtol=0, atol=float(4 * np.spacing(np.abs(v).max())))
            np.testing.assert_allclose(gx, x, rtol=0, atol=float(4 * np.spacing(np.abs(x).max())))
            # the merged position is not where the coarse particle alone would be
            assert np.abs(gx - (x0[leave] + dt * (v0[leave] + dt * acc))).max() > 0
    assert merged > 0 and kept > 0


@pytest.mark.parametrize("child_mode", [0, 1])
def test_two_scale_graph_matches_eager_and_is_deterministic(sphlib, child_mode):
    sc = small_scene(child_mode)
    outs = []
    for graph in (False, True, True):
        with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options) as sim:
            if graph:
                sim.step(mode=sphlib.SPH_STEP_TWO_SCALE, count=4)
            else:
                for _ in range(4):
                    sim.AdvanceTwoScale()
            outs.append([sim.read(sphlib.FIELD_SUB_VERTEX_DATA), sim.read(sphlib.FIELD_STATE),
                         sim.positions(), sim.read(sphlib.FIELD_SUB_IDS)])
    for o in outs[1:]:
        for a, b in zip(outs[0], o):
            np.testing.assert_array_equal(a, b)


def test_two_scale_stage_timing(sphlib):
    """Stage timing of two-scale steps times the fine level too, and changes
    no result (timed steps run eagerly, untimed ones as a graph)."""
    sc = small_scene()
    outs = []
    for timed in (True, False):
        with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options) as sim:
            if timed:
                sim.set_stage_timing(8)
            sim.step(mode=sphlib.SPH_STEP_TWO_SCALE, count=3)
            sim.step(count=2)
            if timed:
                t = sim.stage_times()
                for k in ("hash_count", "cell_scan", "scatter", "rank_gather", "density", "force_integrate"):
                    assert t[k][1] == 5 and t[k][0] > 0, k
                for k in ("ts_children", "sub_sort", "sub_density", "sub_force"):
                    assert t[k][1] == 3 and t[k][0] > 0, k
            outs.append([sim.read(sphlib.FIELD_SUB_VERTEX_DATA), sim.positions(), sim.velocities()])
    for a, b in zip(*outs):
        np.testing.assert_array_equal(a, b)


def test_config3_runs(sphlib):
    """The 262,144-particle two-scale configuration: counts and finiteness."""
    sc = scenes.config3()
    with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options) as sim:
        sim.step(mode=sphlib.SPH_STEP_TWO_SCALE, count=10)
        sim.synchronize()
        c = sim.counts()
        sub = sim.read(sphlib.FIELD_SUB_IDS)
        pos = sim.read(sphlib.FIELD_SUB_VERTEX_DATA)
    assert c.numParticlesSplit > 3000 and c.numSubParticles == 8 * (c.numParticlesSplit + c.numParticlesBoundary)
    assert np.isfinite(pos[sub]).all()


def test_config3_matches_oracle(sphlib, orc):
    """The 262,144-particle two-scale configuration (persistent children,
    merge-back) at full size: coarse tables, states, lists, child list and the
    fine level's tables bit-exact against the FP32 restatement, fine
    densities and accelerations within 1e-5 of the FP64 scale, over two steps
    (the second with the children the first one left)."""
    sc = scenes.config3()
    n = sc.n
    o32 = orc.TwoScale(n)
    o64 = orc.TwoScale(n, fp64=True)
    with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options) as sim:
        for step in range(2):
            x0, v0 = sim.positions(), sim.velocities()
            if step > 0:
                sp = sim.read(sphlib.FIELD_SUB_VERTEX_DATA)
                sv = sim.read(sphlib.FIELD_SUB_SIMULATION_DATA)[:, 6:9].copy()
                for T in (o32, o64):
                    T.set_children(sp, sv)
            sim.AdvanceTwoScale()
            co = coarse_inputs(sphlib, sim)
            r32 = orc.step_plain(sc.params, sc.options, None, x0, v0)
            h, _, _, _ = sim.cells(0)
            for key, got in (("hash", h), ("ids", co["ids"]), ("start", co["start"]), ("end", co["end"])):
                np.testing.assert_array_equal(got, r32[key], err_msg=f"coarse {key}, step {step}")
            g = gpu_two_scale(sphlib, sim)
            c = g["counts"]
            assert c.numParticlesSplit > 3000
            assert c.numSubParticles == 8 * (c.numParticlesSplit + c.numParticlesBoundary)
            check_against_oracle(orc, sc, g, o32, o64, x0, v0, co)
