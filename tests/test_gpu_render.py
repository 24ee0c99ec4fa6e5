"""GPU checks of the headless renderer (sph_render) against the oracle's
float64 restatement of the TwoScaleStateSub shaders with GL's rasterisation
rules (oracle.render_splats).

The kernels work in FP32 and the oracle in float64, so a pixel whose centre
lies on a sphere's rim, or two fragments whose 24-bit depths differ in the
last step, can go either way: the bars are on the fraction of pixels that
agree (winner particle and colour) and on the colour error of the rest."""
import numpy as np
import pytest

from cudasphnew_gb300 import params as P
from cudasphnew_gb300 import scenes

import oracle

pytestmark = pytest.mark.gpu

W, H = 160, 100
UP = (0.0, 1.0, 0.0)
TINY_VIEW = ((0.05, 0.1, 0.18), (0.05, 0.05, 0.05), 0.01, 10.0)   # eye, centre, near, far
PAIR_VIEW = ((0.25, 0.151, 0.13), (0.25, 0.15, 0.0), 0.01, 10.0)
TS_VIEW = ((0.15, 0.3, 0.55), (0.15, 0.12, 0.15), 0.1, 100.0)


def camera(sphlib, view):
    eye, centre, zn, zf = view
    return sphlib.Camera.look(eye, centre, UP, 60.0, W / H, zn, zf)


def reference(view, passes):
    eye, centre, zn, zf = view
    return oracle.render_splats(oracle.look_at(eye, centre, UP), oracle.perspective(60.0, W / H, zn, zf), passes, W, H)


def radius(sc):
    p = sc.params
    return float(np.float32((3.0 * p.fluidVolume / (4.0 * np.pi * p.numParticles)) ** (1.0 / 3.0)))


def compare(img, ref_img, min_equal=0.99):
    cov, rcov = (img[..., :3] != 255).any(-1), (ref_img[..., :3] != 255).any(-1)
    assert rcov.mean() > 0.05  # the scene is in view
    assert (cov != rcov).mean() < 0.01
    same = (img == ref_img).all(-1)
    assert same.mean() >= min_equal, same.mean()


def test_particles_match_oracle(sphlib):
    sc = scenes.dam_break(8, 8, 8, (0, 0, 0), (0.5, 0.5, 0.5), 3, "tiny", 1)
    with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options) as sim:
        sim.step(count=5)
        img, depth = sim.render(camera(sphlib, TINY_VIEW), W, H, sphlib.SPH_RENDER_PARTICLES, depth=True)
        pos = sim.positions()
    ref, win = reference(TINY_VIEW, [(pos, radius(sc), (0.0, 0.0, 0.9))])
    compare(img, ref)
    assert (depth[win < 0] == 1.0).all() and (depth[win >= 0] < 1.0).mean() > 0.99
    # colours are the shader's: blue, shaded 0.9 + 0.1 n.z
    covered = img[..., 2] != 255
    assert (img[covered][:, :2] == 0).all()
    assert img[covered][:, 2].min() >= np.floor(0.9 * 0.9 * 255) - 1


def test_depth_order_and_ties(sphlib):
    """A nearer sphere hides a farther one whatever the draw order; two
    spheres at the same place: the one drawn first stays (GL_LESS)."""
    sc = scenes.dam_break(1, 1, 1, (0.2, 0.2, 0.2), (0.5, 0.5, 0.5), 1, "one", 1)
    p = P.SimulationParameters.from_buffer_copy(bytes(sc.params))
    p.numParticles = 3
    R = radius(scenes.Scene("t", p, sc.options, None, None))
    pos = np.array([[0.25 + 0.8 * R, 0.15, 0.10],   # behind, drawn first
                    [0.25, 0.15, 0.11],             # in front (the eye is at z = 0.13), drawn after
                    [0.25, 0.15, 0.11]],            # the same place as particle 1, drawn last
                   np.float32)
    with sphlib.ParticleSimulation(p, pos, np.zeros_like(pos), sc.options) as sim:
        img = sim.render(camera(sphlib, PAIR_VIEW), W, H, sphlib.SPH_RENDER_PARTICLES)
    ref, win = reference(PAIR_VIEW, [(pos, R, (0.0, 0.0, 0.9))])
    assert (win == 0).sum() > 100 and (win == 1).sum() > 100 and (win == 2).sum() == 0
    compare(img, ref, min_equal=0.995)


def test_two_scale_render_matches_oracle(sphlib):
    sc = scenes.two_scale(nb=24, region=(0.1, 0.2), box=0.5, name="two_scale_small")
    with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options) as sim:
        for _ in range(3):
            sim.step(mode=sphlib.SPH_STEP_TWO_SCALE)
        cam = camera(sphlib, TS_VIEW)
        img = sim.render(cam, W, H, sphlib.SPH_RENDER_TWO_SCALE)
        sub = sim.render(cam, W, H, sphlib.SPH_RENDER_SUB_PARTICLES)
        c = sim.counts()
        pos = sim.positions()
        dflt = sim.read(sphlib.FIELD_DEFAULT_IDS)
        slots = sim.read(sphlib.FIELD_SUB_IDS)
        spos = sim.read(sphlib.FIELD_SUB_VERTEX_DATA)
    reg = 8 * c.numParticlesSplit
    assert reg > 0 and len(slots) > reg
    R = radius(sc)
    passes = [(pos[dflt], R, (0.0, 0.0, 0.9)), (spos[slots[:reg]], R / 2, (0.9, 0.9, 0.0)),
              (spos[slots[reg:]], R / 2, (0.9, 0.0, 0.0))]
    ref, _ = reference(TS_VIEW, passes)
    compare(img, ref)
    ref_sub, _ = reference(TS_VIEW, passes[1:])
    compare(sub, ref_sub)
    # the default particles are blue; without them the boundary children (red)
    # that wrap the split region are in view
    assert ((img[..., 2] > 200) & (img[..., 0] < 30)).any()
    assert ((sub[..., 0] > 200) & (sub[..., 1] < 30)).any()


def test_render_refuses_before_a_two_scale_step(sphlib):
    sc = scenes.dam_break(8, 8, 8, (0, 0, 0), (0.5, 0.5, 0.5), 3, "tiny", 1)
    with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options) as sim:
        with pytest.raises(sphlib.SphError):
            sim.render(camera(sphlib, TINY_VIEW), W, H, sphlib.SPH_RENDER_TWO_SCALE)


def test_cell_relative_renders_the_same_image(sphlib):
    sc = scenes.dam_break(8, 8, 8, (0, 0, 0), (0.5, 0.5, 0.5), 3, "tiny", 1)
    o = P.Options.from_buffer_copy(bytes(sc.options))
    o.cellRelative = 1
    imgs = []
    for opts in (sc.options, o):
        with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, opts) as sim:
            imgs.append(sim.render(camera(sphlib, TINY_VIEW), W, H, sphlib.SPH_RENDER_PARTICLES))
    np.testing.assert_array_equal(imgs[0], imgs[1])
