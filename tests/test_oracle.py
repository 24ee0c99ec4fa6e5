"""CPU tests of the oracle: pinned against the reference's recorded boundary
maps, known-answer kernels, hash/sort/cell semantics and FP32/FP64 agreement."""
import math
import os

import numpy as np
import pytest

from cudasphnew_gb300 import params as P
from cudasphnew_gb300 import scenes

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "example01_map_slices.npz")


# ---------------------------------------------------------------------------
# Pin: Example01's box maps reproduce the reference's distances.ppm and
# viscosities.ppm (SphInComplexShapes.cpp:429-558 via particle_simulation.cu:2613)
# ---------------------------------------------------------------------------
@pytest.fixture(scope="module")
def example01_maps(orc):
    p = P.example01_params()
    return p, orc.boundary_maps(P.example01_boundary(p))


def test_example01_grid_shape(example01_maps):
    p, bm = example01_maps
    assert list(p.gridDim) == [81, 81, 81]
    assert bm.dims == (259, 194, 130)


def test_distance_map_matches_reference_image(orc, example01_maps):
    p, bm = example01_maps
    ref = np.load(GOLDEN)["distances"].astype(np.int64)
    k = bm.dims[2] // 2
    mine = orc.jet_slice(bm.dist[k].T, bm.desc.restDistance)
    diff = np.abs(mine - ref)
    # the reference ran on 32-bit x87 (extended precision): 1 colour level slack
    assert diff.max() <= 1
    assert (diff > 0).mean() < 0.005


def test_viscosity_map_matches_reference_image(orc, example01_maps):
    p, bm = example01_maps
    ref = np.load(GOLDEN)["viscosities"].astype(np.int64)
    k = bm.dims[2] // 2
    mine = orc.jet_slice(bm.visc[k].T, float(bm.visc.max()))
    diff = np.abs(mine - ref)
    assert diff.max() <= 1
    assert (diff > 0).mean() < 0.001


def test_map_defaults_outside_band(example01_maps):
    """Nodes farther than compactSupport from the wall read entry 0 of the node
    lists: distance -restDistance, density 0, viscosity 0 (reset(), :641-652)."""
    p, bm = example01_maps
    far = bm.dist == np.float32(-bm.desc.restDistance)
    assert far.any()
    assert (bm.dens[far] == 0).all() and (bm.visc[far] == 0).all()
    kept = ~far
    assert (np.abs(bm.dist[kept]) < bm.desc.compactSupport).all()


# ---------------------------------------------------------------------------
# Known answers
# ---------------------------------------------------------------------------
def _two_particle_scene(r, v_rel=(0.0, 0.0, 0.0)):
    p = P.dam_break_params((0, 0, 0), (1, 1, 1), 2)
    o = P.default_options(gravity_axis=2, box_collision=False)
    pos = np.array([[0.5, 0.5, 0.5], [0.5 + r, 0.5, 0.5]], np.float32)
    vel = np.array([[0.0, 0.0, 0.0], v_rel], np.float32)
    return p, o, pos, vel


def test_two_particle_density_and_force(orc):
    r = 0.6 * P.H
    p, o, pos, vel = _two_particle_scene(r, (0.1, -0.2, 0.05))
    out = orc.step_plain(p, o, None, pos, vel, fp64=True)
    h, m = float(p.compactSupport), float(p.particleMass)
    rr = float(pos[1, 0]) - float(pos[0, 0])
    poly6 = float(p.poly6)
    rho = m * poly6 * ((h * h) ** 3 + (h * h - rr * rr) ** 3)
    assert out["rho"] == pytest.approx([rho, rho], rel=1e-12)
    prs = float(p.gasStiffness) * (rho - float(p.restDensity))
    assert out["p"] == pytest.approx([prs, prs], rel=1e-12)
    # particle 0: r_vec = x0 - x1 = (-rr, 0, 0)
    grad, lapl, mu = float(p.gradSpiky), float(p.laplVisc), float(p.dynamicViscosity)
    press = rho * (prs / rho ** 2 + prs / rho ** 2) * m
    fpx = -press * grad * (h - rr) ** 2 / rr * (-rr)
    v64 = vel.astype(np.float64)
    fv = np.array([mu * (v64[1, a] - v64[0, a]) * m / rho * lapl * (h - rr) for a in range(3)])
    acc0 = np.array([fpx + fv[0], fv[1], fv[2]]) / rho
    acc0[2] -= float(p.gravity)
    assert out["acc"][0] == pytest.approx(acc0, rel=1e-9, abs=1e-9)


def test_isolated_particle_free_fall(orc):
    """No neighbours, no walls: symplectic Euler under gravity along -z."""
    p = P.dam_break_params((0, 0, 0), (1, 1, 1), 1)
    o = P.default_options(gravity_axis=2, box_collision=False)
    pos = np.array([[0.5, 0.5, 0.9]], np.float64)
    vel = np.zeros((1, 3))
    dt, g = float(p.timeStep), float(p.gravity)
    x, v = pos.copy(), vel.copy()
    for k in range(1, 21):
        out = orc.step_plain(p, o, None, x, v, fp64=True)
        x, v = out["pos"], out["vel"]
        assert v[0, 2] == pytest.approx(-g * dt * k, rel=1e-12)
    # x_k = x_0 - g dt^2 k(k+1)/2
    assert x[0, 2] == pytest.approx(0.9 - g * dt * dt * 20 * 21 / 2, rel=1e-12)


def test_lattice_rest_density(orc):
    """Bulk density of the h/2 lattice: every neighbour shell of a perfect
    lattice, summed analytically, equals the oracle's interior density."""
    sc = scenes.dam_break(12, 12, 12, (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), 1, "lat", 1)
    pos = scenes.lattice_block(12, 12, 12, (0.0, 0.0, 0.0), P.SPACING, 1, 0.0)
    out = orc.step_plain(sc.params, sc.options, None, pos, np.zeros_like(pos), fp64=True)
    h, s, m = float(sc.params.compactSupport), P.SPACING, float(sc.params.particleMass)
    rng = np.arange(-3, 4)
    d = np.stack(np.meshgrid(rng, rng, rng, indexing="ij"), -1).reshape(-1, 3) * s
    r2 = (d ** 2).sum(1)
    w = np.clip(h * h - r2, 0, None)
    expect = m * float(sc.params.poly6) * (w ** 3).sum()
    centre = np.argmin(((pos - pos.mean(0)) ** 2).sum(1))
    assert out["rho"][centre] == pytest.approx(expect, rel=1e-6)


def test_collision_projects_and_removes_normal_velocity(orc):
    p = P.dam_break_params((0, 0, 0), (1, 1, 1), 1)
    o = P.default_options(gravity_axis=2, box_collision=True)
    p.gravity = 0.0
    pos = np.array([[0.5, 0.5, 0.00001]], np.float64)
    vel = np.array([[0.3, 0.0, -2.0]], np.float64)  # leaves the floor in one step
    out = orc.step_plain(p, o, None, pos, vel, fp64=True)
    assert out["pos"][0, 2] == pytest.approx(0.0, abs=1e-12)
    assert out["vel"][0, 2] == pytest.approx(0.0, abs=1e-12)  # restitution 0
    assert out["vel"][0, 0] == pytest.approx(0.3, rel=1e-12)


def test_collision_guard_at_rest_outside(orc):
    """|v| = 0 outside the box: the reference divides by zero (NaN); the
    restatement drops the restitution term."""
    p = P.dam_break_params((0, 0, 0), (1, 1, 1), 1)
    o = P.default_options(gravity_axis=2, box_collision=True)
    p.gravity = 0.0
    p.restitution = 0.5
    pos = np.array([[1.01, 0.5, 0.5]], np.float32)
    out = orc.step_plain(p, o, None, pos, np.zeros((1, 3), np.float32))
    assert np.isfinite(out["pos"]).all() and np.isfinite(out["vel"]).all()
    assert out["pos"][0, 0] == np.float32(1.0)


# ---------------------------------------------------------------------------
# Hash / sort / cell tables against an independent restatement
# ---------------------------------------------------------------------------
def _py_hash(p, pos):
    c = []
    for a in range(3):
        f = (pos[:, a].astype(np.float32) - np.float32(p.gridOrigin[a])) / np.float32(p.gridSpacing)
        ci = np.trunc(f.astype(np.float32)).astype(np.int64)
        ci = np.fmod(ci, p.gridDim[a])  # C remainder
        c.append(ci)
    return (p.gridDim[0] * (p.gridDim[1] * c[2] + c[1]) + c[0]).astype(np.int32)


def _py_tables(p, pos):
    h = _py_hash(p, pos)
    order = sorted(range(len(h)), key=lambda i: (h[i], i))
    hs = h[order]
    C = p.num_cells
    start = np.full(C, -1, np.int32)
    end = np.full(C, -1, np.int32)
    for i, c in enumerate(hs):
        if i == 0 or c != hs[i - 1]:
            start[c] = i
            if i > 0:
                end[hs[i - 1]] = i
        if i == len(hs) - 1:
            end[c] = i + 1
    return hs, np.array(order, np.int32), start, end


@pytest.mark.parametrize("layout", ["faces", "reverse", "edge", "random"])
def test_hash_sort_cells(orc, layout):
    p = P.dam_break_params((0, 0, 0), (1, 1, 1), 1)
    rng = np.random.default_rng(5)
    g = float(p.gridSpacing)
    o = np.array(p.gridOrigin[:], np.float32)
    if layout == "faces":   # exactly on cell faces
        idx = rng.integers(1, 40, size=(300, 3))
        pos = (o + idx.astype(np.float32) * np.float32(g)).astype(np.float32)
    elif layout == "reverse":  # many particles per cell, ids against position order
        pos = np.repeat(rng.uniform(0.2, 0.8, size=(20, 3)), 15, axis=0)[::-1].astype(np.float32)
    elif layout == "edge":  # the last cell layer of the padded grid
        pos = rng.uniform(0.0, 1.0, size=(400, 3)).astype(np.float32)
        pos[:, 0] = np.float32(o[0] + g * (p.gridDim[0] - 0.5))
    else:
        pos = rng.uniform(0.0, 1.0, size=(2000, 3)).astype(np.float32)
    hs, ids, start, end = orc.hash_sort_cells(p, pos)
    ehs, eids, estart, eend = _py_tables(p, pos)
    np.testing.assert_array_equal(hs, ehs)
    np.testing.assert_array_equal(ids, eids)
    np.testing.assert_array_equal(start, estart)
    np.testing.assert_array_equal(end, eend)


def test_neighbour_range_wraps_at_upper_edge(orc):
    """compute_grid_coordinate's `% dim` wraps c1 to 0 when x + h reaches the
    last cell boundary (particle_simulation.cu:1249-1255): the x-loop is then
    empty.  The restatement keeps the quirk; the padded grid keeps dam-break
    particles away from it."""
    p = P.dam_break_params((0, 0, 0), (1, 1, 1), 2)
    o = P.default_options(gravity_axis=2, box_collision=False)
    top = float(p.gridOrigin[0]) + float(p.gridSpacing) * p.gridDim[0]
    x = np.float32(top - 0.5 * float(p.compactSupport))
    pos = np.array([[x, 0.5, 0.5], [x - 0.7 * P.H, 0.5, 0.5]], np.float32)
    out = orc.step_plain(p, o, None, pos, np.zeros_like(pos))
    m_poly = float(p.particleMass) * float(p.poly6) * float(p.compactSupport) ** 6
    assert out["rho"][0] == 0.0  # not even itself: empty x-range
    # the interior particle sees itself and its neighbour at 0.7 h
    assert out["rho"][1] == pytest.approx(m_poly * (1.0 + 0.51 ** 3), rel=1e-4)


# ---------------------------------------------------------------------------
# FP32 reference order vs FP64 on the benchmark scenes (tolerance self-check)
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("name", ["config1", "example01", "small_obstacle"])
def test_fp32_vs_fp64_within_tolerance(orc, name):
    sc = getattr(scenes, name)()
    bm = orc.boundary_maps(sc.boundary) if sc.boundary is not None else None
    r32 = orc.step_plain(sc.params, sc.options, bm, sc.positions, sc.velocities)
    r64 = orc.step_plain(sc.params, sc.options, bm, sc.positions, sc.velocities, fp64=True)
    np.testing.assert_array_equal(r32["ids"], r64["ids"])
    assert (np.abs(r32["rho"] - r64["rho"]) <= 1e-5 * r64["scale_rho"]).all()
    assert (np.abs(r32["acc"] - r64["acc"]).max(1) <= 1e-5 * r64["scale_acc"]).all()


def test_obstacle_maps_band(orc):
    sc = scenes.small_obstacle()
    bm = orc.boundary_maps(sc.boundary)
    assert bm.dims == (128, 128, 128)
    kept = bm.dist != np.float32(-sc.boundary.restDistance)
    assert kept.sum() > 1000
    # wall density is deposited by ghosts only near the surface
    assert bm.dens.max() > 0 and (bm.dens[~kept] == 0).all()
    # sphere centre column: fluid side negative, solid side positive
    d = sc.boundary
    k = int(round((0.25 - d.gridStart[2]) / d.gridSpacing))
    assert bm.dist[k].max() > 0 and bm.dist[k].min() < 0
