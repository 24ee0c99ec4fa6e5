"""Meshes and signed distance grids on the host: the OBJ reader, the
reference's boundary-map text format (BoundaryMap::Save / Load,
boundary_map.cpp:161-287) and the oracle's mesh distance grid against
analytic solids."""
import os

import numpy as np
import pytest

from cudasphnew_gb300 import meshes


def test_obj_reader_formats(sphlib, tmp_path):
    p = tmp_path / "m.obj"
    p.write_text("# comment\no thing\nv 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nvt 0 0\nvn 0 0 1\n"
                 "f 1 2 3\nf 1/1 3/1 4/1\nf -4//1 -3//1 -2//1 -1//1\nf 2/1/1 3/1/1 4/1/1\n")
    v, f = sphlib.load_obj(str(p))
    np.testing.assert_array_equal(v, np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]], np.float32))
    # the quad (negative indices) becomes the fan (0,1,2), (0,2,3)
    np.testing.assert_array_equal(f, np.array([[0, 1, 2], [0, 2, 3], [0, 1, 2], [0, 2, 3], [1, 2, 3]], np.uint32))


@pytest.mark.parametrize("text", ["v 0 0 0\nf 1 2 3\n", "v 0 0\n", "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2\n", ""])
def test_obj_reader_rejects(sphlib, tmp_path, text):
    p = tmp_path / "bad.obj"
    p.write_text(text)
    with pytest.raises(sphlib.SphError):
        sphlib.load_obj(str(p))


def test_obj_round_trip(sphlib, tmp_path):
    v, f = meshes.icosphere(0.3, (1, 2, 3), 2)
    p = tmp_path / "ico.obj"
    meshes.write_obj(str(p), v, f)
    v2, f2 = sphlib.load_obj(str(p))
    np.testing.assert_array_equal(f2, f)
    np.testing.assert_allclose(v2, v, rtol=0, atol=1e-7)


def reference_format_file(path, dims, band):
    """A boundary-map file laid out as BoundaryMap::Save writes it."""
    lines = ["0.025", "0.03", "0.03", "0.01", "0", "0", "0", str(0.01 * (dims[0] - 1)),
             str(0.01 * (dims[1] - 1)), str(0.01 * (dims[2] - 1)), *map(str, dims),
             str(dims[0] * dims[1] * dims[2]), str(len(band))]
    for (i, j, k), d, n in band:
        lines += [str(i), str(j), str(k), repr(d), *map(repr, n)]
    path.write_text("\n".join(lines) + "\n")


def test_boundary_map_file_load(sphlib, tmp_path):
    p = tmp_path / "map.txt"
    band = [((1, 2, 3), -0.005, (0.0, 1.0, 0.0)), ((0, 0, 0), 0.0125, (0.6, 0.8, 0.0))]
    reference_format_file(p, (4, 5, 6), band)
    g = sphlib.SignedDistanceGrid.load_file(str(p))
    assert g.dims == (4, 5, 6) and g.dx == pytest.approx(0.01) and g.maxDist == pytest.approx(0.03)
    # nodes the file does not list hold the rest distance (boundary_map.cpp:248-252)
    expect = np.full((6, 5, 4), np.float32(0.025))
    expect[3, 2, 1] = -0.005
    expect[0, 0, 0] = 0.0125
    np.testing.assert_array_equal(g.distance, expect)
    np.testing.assert_allclose(g.normal[3, 2, 1], (0, 1, 0))
    assert not g.normal[1, 1, 1].any()


def test_boundary_map_file_round_trip(sphlib, tmp_path):
    p = tmp_path / "map.txt"
    reference_format_file(p, (3, 3, 3), [((2, 1, 0), -0.01, (0.0, 0.0, -1.0))])
    g = sphlib.SignedDistanceGrid.load_file(str(p))
    q = tmp_path / "again.txt"
    g.save(str(q))
    h = sphlib.SignedDistanceGrid.load_file(str(q))
    np.testing.assert_array_equal(h.distance, g.distance)
    np.testing.assert_array_equal(h.normal, g.normal)
    assert h.dims == g.dims and h.dx == g.dx and h.restDistance == g.restDistance


@pytest.mark.parametrize("text", ["1\n2\n", "0.025\n0.03\n0.03\n0.01\n0\n0\n0\n1\n1\n1\n2\n2\n2\n9\n1\n"])
def test_boundary_map_file_rejects(sphlib, tmp_path, text):
    p = tmp_path / "bad.txt"
    p.write_text(text)
    with pytest.raises(sphlib.SphError):
        sphlib.SignedDistanceGrid.load_file(str(p))


def grid_points(origin, dx, dims):
    axes = [np.float32(origin[a]) + np.arange(dims[a], dtype=np.float32) * np.float32(dx) for a in range(3)]
    Z, Y, X = np.meshgrid(axes[2], axes[1], axes[0], indexing="ij")
    return X.astype(np.float64), Y.astype(np.float64), Z.astype(np.float64)


def test_oracle_mesh_sdf_sphere(orc):
    R, c = 0.2, (0.5, 0.5, 0.5)
    v, f = meshes.icosphere(R, c, 4)
    origin, dx, dims, md = (0.2, 0.2, 0.2), 0.02, (31, 31, 31), 0.03
    d, n = orc.mesh_sdf(v, f, origin, dx, dims, md)
    X, Y, Z = grid_points(origin, dx, dims)
    r = np.sqrt((X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2)
    exact = r - R
    band = np.abs(exact) < md - 1e-3
    assert np.abs(d[band] - exact[band]).max() < 3e-4  # the icosphere's chord error
    assert ((d < 0) == (exact < 0))[np.abs(exact) > 1e-3].all()
    assert (np.abs(d[np.abs(exact) > md + 1e-3]) == np.float32(md)).all()
    # normals point away from the surface, radially
    radial = np.stack([X - c[0], Y - c[1], Z - c[2]], -1) / np.maximum(r, 1e-12)[..., None]
    sel = band & (exact > 2e-3)
    assert (np.einsum("...k,...k", n[sel], radial[sel]) > 0.99).all()


def test_oracle_mesh_sdf_box(orc):
    lo, hi = (0.3, 0.25, 0.2), (0.7, 0.65, 0.5)
    v, f = meshes.box(lo, hi)
    origin, dx, dims, md = (0.2, 0.15, 0.1), 0.025, (25, 25, 21), 0.06
    d, _ = orc.mesh_sdf(v, f, origin, dx, dims, md)
    X, Y, Z = grid_points(origin, dx, dims)
    q = [np.maximum(lo[a] - P, P - hi[a]) for a, P in enumerate((X, Y, Z))]
    outside = np.sqrt(sum(np.maximum(t, 0) ** 2 for t in q))
    inside = np.minimum(np.maximum(np.maximum(q[0], q[1]), q[2]), 0)
    exact = outside + inside
    band = np.abs(exact) < md - 1e-4
    assert np.abs(d[band] - exact[band]).max() < 1e-6
    assert ((d < 0) == (exact < 0))[np.abs(exact) > 1e-4].all()
