"""GPU mesh signed distance grids (sph_sdf_from_mesh) against the oracle, and
mesh solids (SPH_SHAPE_MESH) in the step's boundary maps."""
import ctypes

import numpy as np
import pytest

from cudasphnew_gb300 import meshes
from cudasphnew_gb300 import params as P
from cudasphnew_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind", ["sphere", "box", "coarse_sphere"])
def test_mesh_sdf_matches_oracle(sphlib, orc, kind):
    if kind == "box":
        v, f = meshes.box((0.3, 0.25, 0.2), (0.7, 0.65, 0.5))
    else:
        v, f = meshes.icosphere(0.2, (0.5, 0.5, 0.5), 4 if kind == "sphere" else 1)
    origin, dx, dims, rest, h = (0.2, 0.15, 0.1), 0.0125, (49, 53, 47), 0.025, 0.03
    g = sphlib.SignedDistanceGrid.from_mesh(v, f, rest, h, dx, origin=origin, dims=dims)
    d, n = orc.mesh_sdf(v, f, origin, dx, dims, max(rest, h))
    assert g.dims == dims and g.maxDist == pytest.approx(max(rest, h))
    # magnitudes: the two closest-point constructions agree to rounding
    np.testing.assert_allclose(np.abs(g.distance), np.abs(d), rtol=0, atol=2e-6)
    # signs: the same ray, so the same parity (ties at the surface aside)
    far = np.abs(d) > 1e-5
    np.testing.assert_array_equal(g.distance[far] < 0, d[far] < 0)
    band = (np.abs(d) < 0.9 * max(rest, h)) & far
    # normals agree except at nodes equidistant from two surface points, where
    # the two constructions' roundings pick different (equally close) points
    diff = np.abs(g.normal[band] - n[band]).max(1)
    assert (diff > 1e-4).mean() < 1e-3
    np.testing.assert_allclose(np.linalg.norm(g.normal[band], axis=1), 1.0, atol=1e-5)


def test_mesh_sdf_on_its_bounding_box(sphlib):
    v, f = meshes.box((0.0, 0.0, 0.0), (0.1, 0.2, 0.05))
    g = sphlib.SignedDistanceGrid.from_mesh(v, f, 0.01, 0.02, 0.01)
    # AddCanvas: ceil(extent / dx) + 1 nodes per axis from the box's low corner
    assert g.dims == (11, 21, 6)
    np.testing.assert_array_equal(g.origin, np.zeros(3, np.float32))
    assert g.distance[0, 0, 0] == 0.0  # a corner node lies on the surface


def mesh_obstacle_desc(sc, grid, index_holder):
    """The obstacle scene's boundary with its sphere replaced by a mesh solid."""
    d = P.BoundaryDesc.from_buffer_copy(bytes(sc.boundary))
    arr = (P.SdfGrid * 1)(grid.struct())
    index_holder += [arr, grid]  # the struct views the grid's arrays
    for i in range(d.numShapes):
        if d.shapes[i].kind == P.SHAPE_SPHERE:
            d.shapes[i].kind = P.SHAPE_MESH
            d.shapes[i].p[0] = 0.0
    d.sdfGrids = ctypes.cast(arr, ctypes.c_void_p)
    d.numSdfGrids = 1
    return d


def sphere_grid(sphlib, sc, subdivisions=4):
    s = [sc.boundary.shapes[i] for i in range(sc.boundary.numShapes) if sc.boundary.shapes[i].kind == P.SHAPE_SPHERE][0]
    c, R = tuple(s.p[:3]), s.p[3]
    v, f = meshes.icosphere(R, c, subdivisions)
    h = float(sc.params.compactSupport)
    dx = h / 4
    pad = R + 3 * h
    n = int(np.ceil(2 * pad / dx)) + 1
    return sphlib.SignedDistanceGrid.from_mesh(v, f, h, h, dx, origin=[x - pad for x in c], dims=(n, n, n))


def test_mesh_obstacle_maps_match_the_analytic_sphere(sphlib):
    sc = scenes.small_obstacle()
    keep = []
    d_mesh = mesh_obstacle_desc(sc, sphere_grid(sphlib, sc), keep)
    dims = sc.boundary.dims()
    maps_a = sphlib.boundary_maps(sc.boundary)
    maps_m = sphlib.boundary_maps(d_mesh)
    dist_a, dist_m = maps_a[0], maps_m[0]
    h = float(sc.params.compactSupport)
    # the maps keep distances within h of a wall and the rest value beyond
    # (SetBox's rule), so compare the nodes well inside that band in both
    sel = (np.abs(dist_a) < 0.8 * h) & (np.abs(dist_m) < 0.8 * h)
    assert sel.sum() > 1000
    # the distance maps differ by the mesh's chord error and the grid's interpolation
    assert np.abs(dist_a - dist_m)[sel].max() < 0.05 * h
    # wall density: the same ghost lattice, except points lying within the
    # surfaces' ~1e-4 m difference of the sphere, which switch sides; one
    # ghost is worth up to m*poly6*h^6 (~0.19 of the maximum) at a node
    rho_a, rho_m = maps_a[1], maps_m[1]
    dr = np.abs(rho_a - rho_m)[sel] / rho_a.max()
    assert dr.mean() < 0.01 and np.quantile(dr, 0.99) < 0.1 and dr.max() < 0.25
    assert len(dims) == 3


def test_step_with_a_mesh_obstacle(sphlib):
    sc = scenes.small_obstacle()
    keep = []
    d_mesh = mesh_obstacle_desc(sc, sphere_grid(sphlib, sc), keep)
    with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options, d_mesh) as sim:
        sim.step(count=20)
        pm = sim.positions()
    with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options, sc.boundary) as sim:
        sim.step(count=20)
        pa = sim.positions()
    assert np.isfinite(pm).all()
    # the mesh sphere stands in for the analytic one: the two runs stay close
    assert np.abs(pm - pa).max() < 0.25 * float(sc.params.compactSupport)
