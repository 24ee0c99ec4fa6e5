"""CPU pin of the oracle's plain step against a brute-force FP64 restatement
of the reference formulas on a small jittered block with random velocities:
poly6 density + EOS (compute_particle_density_pressure,
particle_simulation.cu:196-256) and spiky pressure + viscosity Laplacian
accelerations with gravity (compute_particle_acceleration_ifsurf, :315-474,
no boundary map, surface tension off)."""
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
