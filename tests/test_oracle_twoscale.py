"""CPU known-answer checks of the oracle's two-scale restatement (particle
states, the three-way lists, the child list, the child seeding, the
projection and the fine density), against a numpy restatement of
find_split_particles / find_boundary_particles / collect /
initialize_sub_particles / project_quantities /
compute_sub_particle_density_pressure (particle_simulation.cu:259-313,
570-622, 932-1090, 1328-1381, 2509-2567) on a small lattice, and the
merge-back of persistent children."""
import numpy as np

from cudasphnew_gb300 import scenes


def ref_r2(a, b):
    """r^2 as find_boundary_particles forms it: FP32 differences, products and
    a left-to-right sum, each rounded."""
    d = (a.astype(np.float32) - b.astype(np.float32)).astype(np.float32)
    p = (d * d).astype(np.float32)
    return ((p[..., 0] + p[..., 1]).astype(np.float32) + p[..., 2]).astype(np.float32)


SIGNS = np.array([[1 - 2 * ((c >> 2) & 1), 1 - 2 * ((c >> 1) & 1), 1 - 2 * (c & 1)] for c in range(8)], np.float64)


def child_radius(mass, rho):
    """initialize_sub_particles' radius (:1057-1059): 3m in float, the
    quotient in double, the radicand rounded to float, raised to the float
    1/3 in double and rounded to float."""
    three_m = float(np.float32(3.0) * np.float32(mass))
    radicand = (three_m / (4.0 * np.pi * np.asarray(rho, np.float32).astype(np.float64))).astype(np.float32)
    third = float(np.float32(1.0) / np.float32(3.0))
    return (radicand.astype(np.float64) ** third).astype(np.float32)


def seeded_children(sc, x0, rho, parents):
    """The 8 children of each parent in float arithmetic: x + (+-1/sqrt 3) r
    per axis as one fused multiply-add (the product is exact in double)."""
    r = child_radius(sc.params.particleMass, rho[parents]).astype(np.float64)
    step = SIGNS[None] * float(np.float32(0.577350269)) * r[:, None, None]
    return (x0[parents][:, None, :].astype(np.float64) + step).astype(np.float32).reshape(-1, 3)


def run_first_pass(orc):
    sc = scenes.two_scale(nb=12, region=(0.05, 0.1), box=0.5, name="two_scale_kat")
    x0, v0 = sc.positions, sc.velocities
    coarse = orc.step_plain(sc.params, sc.options, None, x0, v0)
    T = orc.TwoScale(sc.n)
    T.part(sc.params, sc.options, x0, v0, coarse["rho"], coarse["p"], coarse["ids"], coarse["start"],
           coarse["end"])
    return sc, x0, v0, coarse, T


def test_states_and_lists(orc):
    sc, x0, _, _, T = run_first_pass(orc)
    lo, hi = np.float32(sc.options.splitMin[0]), np.float32(sc.options.splitMax[0])
    split = np.all((x0 >= lo) & (x0 <= hi), axis=1)
    h2 = np.float32(sc.params.compactSupport) * np.float32(sc.params.compactSupport)
    near = (ref_r2(x0[:, None, :], x0[None, split, :]) <= h2).any(axis=1)
    assert 0 < split.sum() < near.sum() < sc.n
    # first step from the zero history: split particles also mark themselves
    want_state = np.where(split, 3, np.where(near, 2, 0)).astype(np.uint8)
    np.testing.assert_array_equal(T.get("state"), want_state)
    ids = np.arange(sc.n)
    np.testing.assert_array_equal(T.get("split"), ids[split])
    np.testing.assert_array_equal(T.get("boundary"), ids[near & ~split])
    np.testing.assert_array_equal(T.get("default"), ids[~near])
    parents = np.concatenate([ids[split], ids[near & ~split]])
    np.testing.assert_array_equal(T.get("sub_ids"), (8 * parents[:, None] + np.arange(8)).ravel())
    c = T.counts()
    assert (c["split"], c["boundary"], c["sub"]) == (split.sum(), (near & ~split).sum(), 8 * len(parents))


def test_child_seeding_geometry(orc):
    sc, x0, v0, coarse, T = run_first_pass(orc)
    parents = np.concatenate([T.get("split"), T.get("boundary")])
    radius = child_radius(sc.params.particleMass, coarse["rho"][parents])
    assert radius.min() > 0.007 and radius.max() < 0.009
    seeded = seeded_children(sc, x0, coarse["rho"], parents).astype(np.float64).reshape(-1, 8, 3)
    got = T.get("sub_pos").reshape(sc.n, 8, 3)[parents].astype(np.float64)
    # the fine step has already moved the children by dt_sub (v + dt_sub a)
    # from rest: far below a micrometre against a radius of ~8 mm
    assert np.abs(got - seeded).max() < 2e-6
    # every child keeps its parent's start velocity plus one fine-step kick
    vel = T.get("sub_vel").reshape(sc.n, 8, 3)[parents]
    kick = float(sc.params.timeStepSubParticles) * 1e3
    assert np.abs(vel - v0[parents][:, None, :]).max() < kick


def test_projection_means(orc):
    """project_quantities (:570-622, 1328-1381): a boundary child takes the
    unweighted mean coarse density and pressure of the coarse particles within
    compactSupportSub of its seeded position."""
    sc, x0, _, coarse, T = run_first_pass(orc)
    bnd = T.get("boundary")
    kids = seeded_children(sc, x0, coarse["rho"], bnd)
    hs = np.float32(sc.params.compactSupportSub)
    r2 = ref_r2(kids[:, None, :], x0[None, :, :])
    inside = r2 <= hs * hs
    cnt = inside.sum(axis=1)
    assert (cnt > 0).mean() > 0.9
    mean_rho = (inside * coarse["rho"][None, :].astype(np.float64)).sum(1) / np.maximum(cnt, 1)
    mean_p = (inside * coarse["p"][None, :].astype(np.float64)).sum(1) / np.maximum(cnt, 1)
    slots = (8 * bnd[:, None] + np.arange(8)).ravel()
    got_rho, got_p = T.get("sub_rho")[slots], T.get("sub_p")[slots]
    np.testing.assert_allclose(got_rho, np.where(cnt > 0, mean_rho, 0.0), rtol=1e-5)
    np.testing.assert_allclose(got_p, np.where(cnt > 0, mean_p, 0.0), rtol=1e-4, atol=1e-3)


def fp64_pass(orc):
    sc = scenes.two_scale(nb=12, region=(0.05, 0.1), box=0.5, name="two_scale_kat")
    x0, v0 = sc.positions, sc.velocities
    coarse = orc.step_plain(sc.params, sc.options, None, x0, v0, fp64=True)
    T = orc.TwoScale(sc.n, fp64=True)
    T.part(sc.params, sc.options, x0, v0, coarse["rho"], coarse["p"], coarse["ids"], coarse["start"],
           coarse["end"])
    split, bnd = T.get("split"), T.get("boundary")
    parents = np.concatenate([split, bnd])
    kids = seeded_children(sc, x0, coarse["rho"], parents).astype(np.float64)
    return sc, v0, T, split, parents, kids


def test_fine_density_of_regular_children(orc):
    """compute_sub_particle_density_pressure (:259-313): a regular child's
    density is (m/8) poly6_sub sum (h_s^2 - r^2)^3 over every child (regular
    and boundary) within h_s, itself included; checked on the FP64 oracle
    against a brute-force sum over the seeded children."""
    sc, _, T, split, _, kids = fp64_pass(orc)
    hs = float(sc.params.compactSupportSub)
    nreg = 8 * len(split)
    r2 = ((kids[:nreg, None, :] - kids[None, :, :]) ** 2).sum(-1)
    w = np.clip(hs * hs - r2, 0.0, None) ** 3
    want = float(sc.params.subParticleMass) * float(sc.params.poly6Sub) * w.sum(1)
    slots = (8 * split[:, None] + np.arange(8)).ravel()
    np.testing.assert_allclose(T.get("sub_rho")[slots], want, rtol=1e-9)
    assert want.min() > 0.5 * float(sc.params.restDensity)


def test_fine_acceleration_of_regular_children(orc):
    """compute_sub_particle_acceleration (:477-568): pressure (spiky),
    viscosity and colour field at h_s with the sub-particle constants, surface
    tension when the colour gradient exceeds its threshold, gravity; checked
    on the FP64 oracle against a brute-force restatement over the seeded
    children (densities and pressures as the oracle's fine level left them)."""
    sc, v0, T, split, parents, kids = fp64_pass(orc)
    P_ = sc.params
    vel = np.repeat(v0[parents].astype(np.float64), 8, axis=0)
    slots = (8 * parents[:, None] + np.arange(8)).ravel()
    rho = T.get("sub_rho")[slots].astype(np.float64)
    prs = T.get("sub_p")[slots].astype(np.float64)
    nreg = 8 * len(split)
    hs = float(P_.compactSupportSub)
    ms = float(P_.subParticleMass)
    d = kids[:nreg, None, :] - kids[None, :, :]
    r2 = (d ** 2).sum(-1)
    near = (r2 > 0.0) & (r2 <= hs * hs)
    r = np.sqrt(np.where(near, r2, 1.0))
    hr = np.where(near, hs - r, 0.0)
    qi = prs[:nreg] / rho[:nreg] ** 2
    sp = (qi[:, None] + (prs / rho ** 2)[None, :]) * hr * hr / r
    fp = (sp[..., None] * d).sum(1)
    fv = ((hr / rho[None, :])[..., None] * (vel[None, :, :] - vel[:nreg, None, :])).sum(1)
    q = np.where(near, hs * hs - r2, 0.0)
    cg = ((q * q / rho[None, :])[..., None] * d).sum(1)
    cl = (q / rho[None, :] * (3 * hs * hs - 7 * r2)).sum(1)
    force = (float(P_.dynamicViscosity) * ms * float(P_.laplViscSub)) * fv \
        + (-ms * float(P_.gradSpikySub)) * rho[:nreg, None] * fp
    cgv = ms * float(P_.gradPoly6Sub) * cg
    norm = np.linalg.norm(cgv, axis=1)
    on = norm > float(P_.normThresh)
    fc = np.where(on, float(P_.tensionCoefficient) * ms * float(P_.laplPoly6Sub) * cl / np.where(on, norm, 1.0),
                  0.0)
    force -= fc[:, None] * cgv
    acc = force / rho[:nreg, None]
    acc[:, sc.options.gravityAxis] -= float(P_.gravity)
    got = T.get("sub_acc")[slots[:nreg]].astype(np.float64)
    scale = np.abs(acc).max() + float(P_.gravity)
    assert np.abs(got - acc).max() <= 1e-9 * scale
    assert np.abs(acc[:, :2]).max() > 1.0  # the pair terms are there, not just gravity


def test_merge_back_takes_the_childrens_mean(orc):
    """childMode 1 (no reference counterpart): a parent leaving the split
    class takes its eight children's mean position and velocity (slot order,
    times 1/8) and is integrated from there with the acceleration computed at
    its own position (symplectic Euler, away from the walls)."""
    sc = scenes.two_scale(nb=12, region=(0.056, 0.1), box=0.5, name="two_scale_merge_kat")
    sc.options.childMode = 1
    sc.velocities[:, 2] = -1.0
    T = orc.TwoScale(sc.n, fp64=True)
    x, v = sc.positions.astype(np.float64), sc.velocities.astype(np.float64)
    dt = float(sc.params.timeStep)
    merged = 0
    for _ in range(6):
        kids_x = T.get("sub_pos").reshape(sc.n, 8, 3).copy()
        kids_v = T.get("sub_vel").reshape(sc.n, 8, 3).copy()
        r = T.step(sc.params, sc.options, None, x, v)
        code = T.get("state").astype(np.int64) & 15
        was, now = code >> 2, code & 3
        left = ((was & 1) == 1) & ((now & 1) == 0)
        if left.any():
            mx = kids_x[left].sum(1) * 0.125
            mv = kids_v[left].sum(1) * 0.125
            v_new = mv + dt * r["acc"][left]
            x_new = mx + dt * v_new
            np.testing.assert_allclose(r["vel"][left], v_new, rtol=0, atol=1e-12)
            np.testing.assert_allclose(r["pos"][left], x_new, rtol=0, atol=1e-12)
            merged += int(left.sum())
        x, v = r["pos"], r["vel"]
    assert merged > 0
