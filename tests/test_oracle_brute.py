"""CPU pins of the oracle against independent restatements: the plain step
against a brute-force FP64 restatement of the reference formulas on a small
jittered block with random velocities -- poly6 density + EOS
(compute_particle_density_pressure, particle_simulation.cu:196-256) and
spiky pressure + viscosity Laplacian accelerations with gravity
(compute_particle_acceleration_ifsurf, :315-474, no boundary map, surface
tension off) -- and the boundary-map reads against CUDA's documented
normalised, linear, clamped texture fetch."""
import ctypes

import numpy as np

from cudasphnew_gb300 import scenes


def test_plain_step_matches_brute_force(orc):
    sc = scenes.dam_break(8, 8, 8, (0.0, 0.0, 0.0), (0.5, 0.5, 0.5), 5, "brute_512", 1)
    assert float(sc.params.tensionCoefficient) == 0.0
    rng = np.random.default_rng(2)
    vel = rng.normal(0.0, 0.05, sc.positions.shape).astype(np.float32)
    r = orc.step_plain(sc.params, sc.options, None, sc.positions, vel, fp64=True)
    P_ = sc.params
    x = sc.positions.astype(np.float64)
    v = vel.astype(np.float64)
    h = float(P_.compactSupport)
    m = float(P_.particleMass)
    d = x[:, None, :] - x[None, :, :]
    r2 = (d ** 2).sum(-1)
    within = r2 <= h * h
    rho = m * float(P_.poly6) * (np.where(within, h * h - r2, 0.0) ** 3).sum(1)
    prs = float(P_.gasStiffness) * (rho - float(P_.restDensity))
    np.testing.assert_allclose(r["rho"], rho, rtol=1e-12)
    np.testing.assert_allclose(r["p"], prs, rtol=1e-9, atol=1e-9 * float(P_.gasStiffness) * rho.max())
    near = within & (r2 > 0.0)
    rr = np.sqrt(np.where(near, r2, 1.0))
    hr = np.where(near, h - rr, 0.0)
    q = prs / rho ** 2
    sp = (q[:, None] + q[None, :]) * hr * hr / rr
    fp = (sp[..., None] * d).sum(1)
    fv = ((hr / rho[None, :])[..., None] * (v[None, :, :] - v[:, None, :])).sum(1)
    force = (float(P_.dynamicViscosity) * m * float(P_.laplVisc)) * fv + (-m * float(P_.gradSpiky)) * rho[:, None] * fp
    acc = force / rho[:, None]
    acc[:, sc.options.gravityAxis] -= float(P_.gravity)
    scale = np.abs(acc).max()
    assert np.abs(r["acc"] - acc).max() <= 1e-9 * scale
    # both the pressure and the viscosity terms are exercised
    assert np.abs(fp).max() > 0 and np.abs(fv).max() > 0


def test_oracle_trilinear_follows_cuda_normalised_linear_clamp():
    """The SDF reads (:243-248, 408-452): a normalised-coordinate, linear,
    clamped 3-D texture over the map nodes, u = (x - origin) / ((N-1) dx)
    (the reference's grid length), texel coordinate u N - 1/2.  A node is
    returned exactly where its texel centre falls; between nodes the blend
    is trilinear with exact weights; outside, the edge texels are held."""
    import oracle

    rng = np.random.default_rng(4)
    dims = (5, 6, 7)
    grid = rng.random(dims[::-1]).astype(np.float32)  # z, y, x
    m = oracle.Maps()
    origin, dx = (0.1, -0.2, 0.3), 0.05
    for a in range(3):
        m.origin[a] = origin[a]
        m.dims[a] = dims[a]
    m.spacing = dx
    m.restDistance = 0.0
    m.dist = m.dens = m.visc = grid.ctypes.data
    o = np.array([np.float32(v) for v in origin], np.float64)
    length = np.array([np.float32(np.float32(n - 1) * np.float32(dx)) for n in dims], np.float64)
    N = np.array(dims, np.float64)

    def fetch(xyz):
        xyz = np.ascontiguousarray(xyz, np.float64)
        out = np.zeros(len(xyz))
        oracle.lib().orc_tex3d(ctypes.byref(m), 0, oracle._ptr(xyz), len(xyz), oracle._ptr(out))
        return out

    def restated(xyz):
        t = (xyz - o) / length * N - 0.5
        f = np.floor(t)
        a = t - f
        i0 = np.clip(f.astype(np.int64), 0, N.astype(np.int64) - 1)
        i1 = np.clip(f.astype(np.int64) + 1, 0, N.astype(np.int64) - 1)
        g = grid.astype(np.float64)

        def at(ix, iy, iz):
            return g[iz, iy, ix]
        lerp = lambda v0, v1, s: v0 + s * (v1 - v0)
        c00 = lerp(at(i0[:, 0], i0[:, 1], i0[:, 2]), at(i1[:, 0], i0[:, 1], i0[:, 2]), a[:, 0])
        c10 = lerp(at(i0[:, 0], i1[:, 1], i0[:, 2]), at(i1[:, 0], i1[:, 1], i0[:, 2]), a[:, 0])
        c01 = lerp(at(i0[:, 0], i0[:, 1], i1[:, 2]), at(i1[:, 0], i0[:, 1], i1[:, 2]), a[:, 0])
        c11 = lerp(at(i0[:, 0], i1[:, 1], i1[:, 2]), at(i1[:, 0], i1[:, 1], i1[:, 2]), a[:, 0])
        return lerp(lerp(c00, c10, a[:, 1]), lerp(c01, c11, a[:, 1]), a[:, 2])

    # texel centres return the node values
    idx = np.stack(np.meshgrid(*[np.arange(n) for n in dims], indexing="ij"), -1).reshape(-1, 3)
    centres = o + (idx + 0.5) * length / N
    np.testing.assert_allclose(fetch(centres), grid[idx[:, 2], idx[:, 1], idx[:, 0]], rtol=0, atol=1e-12)
    # inside: trilinear with exact weights; outside: the edge texels held
    pts = o + rng.uniform(-0.3, 1.3, (4000, 3)) * length
    np.testing.assert_allclose(fetch(pts), restated(pts), rtol=0, atol=1e-12)
    far = o + np.array([[-5.0, -5.0, -5.0], [10.0, 10.0, 10.0]]) * length
    np.testing.assert_allclose(fetch(far), [grid[0, 0, 0], grid[-1, -1, -1]], rtol=0, atol=1e-12)
