"""GPU checks of the learned step corrector (SPH_STEP_LEARNED).

* The tensor-core MLP (predict and loss gradient) against a numpy
  restatement that rounds the same operands to BF16; the remaining differences
  come from FP32 accumulation order and the hardware tanh the SiLU is
  evaluated with (relative error about 2^-11, which now and then moves an
  activation across a BF16 rounding boundary), so the bars are relative
  (4e-3 of the output scale, 2e-2 of each gradient block's norm).
* The neighbour features (recorded by the learned step's force stage)
  against a brute-force float64 restatement; the fused force + MLP kernel
  against a plain long step plus the separate MLP kernel's prediction.
* Training lowers the loss; the learned step beats the uncorrected plain step
  of the same size against the plain trajectory.
* The audit: with tolerance 0 every audited step is rolled back to exactly the
  plain solver's result, with an infinite tolerance it keeps exactly the
  learned result; CUDA-graph replay equals eager launches.
"""
import numpy as np
import pytest

from cudasphnew_gb300 import params as P
from cudasphnew_gb300 import scenes

pytestmark = pytest.mark.gpu

IN, OUT, HID = 24, 6, 64
NPARAM = 7312


def bf16(x):
    """Round float32 to bfloat16 (nearest even), returned as float32."""
    x = np.ascontiguousarray(x, np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32)


def unpack(blob):
    w = blob[:NPARAM]
    W1 = w[0:2048].reshape(64, 32)
    W2 = w[2048:6144].reshape(64, 64)
    W3 = w[6144:7168].reshape(16, 64)
    b1, b2, b3 = w[7168:7232], w[7232:7296], w[7296:7312]
    s = blob[NPARAM:]
    return W1, W2, W3, b1, b2, b3, s[:24], s[24:48], s[48:54], s[54:60]


def target_scales(blob):
    return blob[NPARAM + 60:NPARAM + 66].astype(np.float64)


def decode(blob, y):
    """Correction from the network's standardised output (targetScale aware)."""
    mut, st, sc = blob[NPARAM + 48:NPARAM + 54], blob[NPARAM + 54:NPARAM + 60], target_scales(blob)
    a = mut + st * y
    return np.where(sc > 0, sc * np.sinh(np.clip(a, -np.arcsinh(1000), np.arcsinh(1000))), a)


def encode(blob, t):
    sc = target_scales(blob)
    return np.where(sc > 0, np.arcsinh(t / np.where(sc > 0, sc, 1)), t)


def random_blob(seed):
    rng = np.random.default_rng(seed)
    W1 = np.zeros((64, 32))
    W1[:, :24] = rng.uniform(-1, 1, (64, 24)) / np.sqrt(24)
    W2 = rng.uniform(-1, 1, (64, 64)) / 8
    W3 = np.zeros((16, 64))
    W3[:6] = rng.uniform(-1, 1, (6, 64)) / 8
    b1, b2 = rng.normal(0, 0.1, 64), rng.normal(0, 0.1, 64)
    b3 = np.zeros(16)
    b3[:6] = rng.normal(0, 0.1, 6)
    blob = np.zeros(7378, np.float32)  # target scales 0: corrections used as the network gives them
    blob[:NPARAM] = np.concatenate([W1.ravel(), W2.ravel(), W3.ravel(), b1, b2, b3])
    blob[NPARAM:NPARAM + 24] = rng.normal(0, 1, 24)
    blob[NPARAM + 24:NPARAM + 48] = rng.uniform(0.5, 2.0, 24)
    blob[NPARAM + 48:NPARAM + 54] = rng.normal(0, 1e-4, 6)
    blob[NPARAM + 54:NPARAM + 60] = rng.uniform(1e-5, 1e-4, 6)
    return blob


def forward(blob, feats):
    W1, W2, W3, b1, b2, b3, mux, sx, mut, st = unpack(blob)
    isx = np.where(sx > 1e-8, np.float32(1) / sx, 0).astype(np.float32)
    xn = bf16((feats.astype(np.float32) - mux) * isx)
    z1 = xn.astype(np.float64) @ bf16(W1[:, :24]).astype(np.float64).T
    a = z1 + b1
    a1 = bf16(a / (1 + np.exp(-a)))
    z2 = a1.astype(np.float64) @ bf16(W2).astype(np.float64).T
    a = z2 + b2
    a2 = bf16(a / (1 + np.exp(-a)))
    y = a2.astype(np.float64) @ bf16(W3[:6]).astype(np.float64).T + b3[:6]
    return dict(xn=xn, z1=z1, a1=a1, z2=z2, a2=a2, y=y, corr=mut + st * y)


def gradient(blob, feats, targets):
    W1, W2, W3, b1, b2, b3, mux, sx, mut, st = unpack(blob)
    f = forward(blob, feats)
    n = len(feats)
    tn = (encode(blob, targets.astype(np.float32).astype(np.float64)) - mut) / st
    e = f["y"] - tn
    loss = (e * e).sum()
    dy = 2 * e / (6 * n)
    dyb = bf16(dy).astype(np.float64)
    dW3 = np.zeros((16, 64))
    dW3[:6] = dyb.T @ f["a2"]
    db3 = np.zeros(16)
    db3[:6] = dy.sum(0)

    def dsilu(a):
        s = 1 / (1 + np.exp(-a))
        return s * (1 + a * (1 - s))

    dz2 = (dyb @ bf16(W3[:6]).astype(np.float64)) * dsilu(f["z2"] + b2)
    dW2 = bf16(dz2).astype(np.float64).T @ f["a1"]
    dz1 = (bf16(dz2).astype(np.float64) @ bf16(W2).astype(np.float64)) * dsilu(f["z1"] + b1)
    dW1 = np.zeros((64, 32))
    dW1[:, :24] = bf16(dz1).astype(np.float64).T @ f["xn"]
    blocks = dict(W1=dW1.ravel(), W2=dW2.ravel(), W3=dW3.ravel(), b1=dz1.sum(0), b2=dz2.sum(0), b3=db3)
    return blocks, loss


SLICES = dict(W1=slice(0, 2048), W2=slice(2048, 6144), W3=slice(6144, 7168), b1=slice(7168, 7232),
              b2=slice(7232, 7296), b3=slice(7296, 7312))


def tiny():
    return scenes.dam_break(8, 8, 8, (0, 0, 0), (0.5, 0.5, 0.5), 3, "tiny", 1)


def small():
    return scenes.dam_break(16, 16, 8, (0, 0, 0), (0.5, 0.5, 0.5), 5, "small", 1)


def make(sphlib, sc, pos=None, vel=None, dt_scale=1, skin=None):
    """A handle of `sc` (optionally from another state, with a longer step, or
    with another neighbourSkin: 0 runs the neighbour search in every step)."""
    p = P.SimulationParameters.from_buffer_copy(bytes(sc.params))
    p.timeStep = float(np.float32(p.timeStep * dt_scale))
    p.timeStepSubParticles = p.timeStep
    o = P.Options.from_buffer_copy(bytes(sc.options))
    if skin is not None:
        o.neighbourSkin = skin
    return sphlib.ParticleSimulation(p, sc.positions if pos is None else pos,
                                     sc.velocities if vel is None else vel, o, sc.boundary)


def density_at(sphlib, sc, pos, vel):
    with make(sphlib, sc, pos, vel) as sim:
        sim.Advance()
        return sim.read(sphlib.FIELD_DENSITY)


def scaled_blob(seed):
    """A blob whose targets were compressed: corrections s*sinh(mean + dev*y)."""
    blob = random_blob(seed)
    blob[NPARAM + 48:NPARAM + 54] = np.random.default_rng(seed).normal(0, 0.3, 6)
    blob[NPARAM + 54:NPARAM + 60] = 1.5
    blob[NPARAM + 60:NPARAM + 66] = np.linspace(1e-6, 6e-6, 6)
    return blob


@pytest.mark.parametrize("count", [1, 127, 128, 300, 4099])
@pytest.mark.parametrize("scaled", [False, True])
def test_mlp_predict_matches_numpy(sphlib, count, scaled):
    blob = scaled_blob(1) if scaled else random_blob(1)
    rng = np.random.default_rng(count)
    feats = rng.normal(0, 1.5, (count, IN)).astype(np.float32)
    with make(sphlib, tiny()) as sim:
        sim.load_corrector(blob)
        got = sim.corrector_predict(feats)
    ref = forward(blob, feats)["y"]
    mut, st = blob[NPARAM + 48:NPARAM + 54], blob[NPARAM + 54:NPARAM + 60]
    y = (encode(blob, got.astype(np.float64)) - mut) / st  # back to the network's output space
    assert np.isfinite(got).all()
    assert np.abs(y - ref).max() <= 4e-3 * max(1.0, np.abs(ref).max())
    if scaled:  # and through the decoding itself
        np.testing.assert_allclose(got, decode(blob, ref), rtol=2e-2, atol=1e-9)


@pytest.mark.parametrize("count", [128, 1000])
@pytest.mark.parametrize("scaled", [False, True])
def test_mlp_gradient_matches_numpy(sphlib, count, scaled):
    blob = scaled_blob(2) if scaled else random_blob(2)
    rng = np.random.default_rng(7 + count)
    feats = rng.normal(0, 1.5, (count, IN)).astype(np.float32)
    tgt = decode(blob, rng.normal(0, 1, (count, OUT))).astype(np.float32)
    with make(sphlib, tiny()) as sim:
        sim.load_corrector(blob)
        g, loss = sim.corrector_gradient(feats, tgt)
    ref, rloss = gradient(blob, feats, tgt)
    assert abs(loss - rloss) <= 2e-3 * rloss
    for k, sl in SLICES.items():
        r = ref[k]
        err = np.linalg.norm(g[sl] - r) / max(np.linalg.norm(r), 1e-30)
        assert err < 2e-2, (k, err)
    # padding stays untouched: input columns 24..31, output rows 6..15
    assert not g[SLICES["W1"]].reshape(64, 32)[:, 24:].any()
    assert not g[SLICES["W3"]].reshape(16, 64)[6:].any()
    assert not g[SLICES["b3"]][6:].any()


def features_ref(sc, pos, vel, rho, acc, stride):
    p = sc.params
    f32 = np.float32
    h = float(f32(p.compactSupport))
    h2 = h * h
    m = float(f32(p.particleMass))
    dtL = float(f32(stride) * f32(p.timeStep))
    x = pos.astype(np.float64)
    v = vel.astype(np.float64)
    d = x[:, None, :] - x[None, :, :]
    r2 = (d * d).sum(2)
    mask = (r2 <= h2) & (r2 > 0)
    inv = 1.0 / rho.astype(np.float64)[None, :]
    W = np.where(mask, float(f32(p.poly6) * f32(m)) * (h2 - r2) ** 3 * inv, 0.0)
    r = np.sqrt(np.where(mask, r2, 1.0))
    G = np.where(mask, float(f32(m) * f32(p.gradSpiky)) * (h - r) ** 2 / r * inv, 0.0)
    gv = G[..., None] * d
    u = v[None, :, :] - v[:, None, :]
    out = np.zeros((len(x), IN))
    out[:, 0] = rho / float(f32(p.restDensity)) - 1
    out[:, 1] = W.sum(1)
    out[:, 2:5] = v
    out[:, 5:8] = acc / float(f32(p.gravity))
    out[:, 8:11] = (W[..., None] * u).sum(1)
    out[:, 11] = dtL * (u * gv).sum(2).sum(1)
    out[:, 12:15] = dtL * np.cross(u, gv).sum(1)
    out[:, 15:18] = h * gv.sum(1)
    out[:, 18] = mask.sum(1) / 32
    c = x - np.array(p.boxCen, np.float64)
    da = np.array(p.boxDim, np.float64) - np.abs(c)
    k = da.argmin(1)
    dmin = da[np.arange(len(x)), k]
    near = dmin < 4 * h
    out[:, 19] = np.clip(np.where(near, dmin, 4 * h), 0, 4 * h) / h
    sgn = np.where(c[np.arange(len(x)), k] > 0, -1.0, 1.0)
    for a in range(3):
        out[:, 20 + a] = np.where(near & (k == a), sgn, 0.0)
    out[:, 23] = np.sqrt((v * v).sum(1)) * dtL / h
    return out


def test_features_match_numpy(sphlib):
    """The features the learned step's force stage records, against a
    brute-force restatement from the state the step started from."""
    sc = tiny()
    with make(sphlib, sc) as sim:
        sim.step(count=30)
        x0, v0 = sim.positions(), sim.velocities()
        sim.load_corrector(random_blob(4), stride=4, auditInterval=0)
        with pytest.raises(sphlib.SphError):
            sim.features()  # nothing recorded yet
        sim.record_features()
        sim.step(mode=sphlib.SPH_STEP_LEARNED)
        rho, acc = sim.read(sphlib.FIELD_DENSITY), sim.read(sphlib.FIELD_ACCELERATION)
        got = sim.features()
    ref = features_ref(sc, x0, v0, rho, acc, 4)
    scale = np.abs(ref).max(0) + 1e-6
    err = np.abs(got - ref) / scale
    assert err.max() < 1e-4, (err.max(0))
    assert np.abs(ref[:, 11:18]).max() > 0 and ref[:, 20:23].any()


@pytest.mark.parametrize("skin", [0.0, 0.1])
@pytest.mark.parametrize("scaled", [False, True])
def test_learned_step_is_the_long_step_plus_the_prediction(sphlib, scaled, skin):
    """The fused force + MLP kernel against its definition: a plain step of
    stride*dt from the same state, plus the corrector's prediction from the
    recorded features (evaluated by the separate MLP kernel).  Particles the
    correction pushes through a wall are collided a second time and left out.
    With neighbourSkin 0.1 the learned step builds the lists (a new handle's
    first step) and walks them."""
    sc = tiny()
    stride = 4
    blob = scaled_blob(8) if scaled else random_blob(8)
    with make(sphlib, sc) as sim:
        sim.step(count=20)
        x0, v0 = sim.positions(), sim.velocities()
    with make(sphlib, sc, x0, v0, skin=skin) as sim:
        sim.load_corrector(blob, stride=stride, auditInterval=0)
        sim.record_features()
        sim.step(mode=sphlib.SPH_STEP_LEARNED)
        xl, vl = sim.positions(), sim.velocities()
        c = sim.corrector_predict(sim.features())
    with make(sphlib, sc, x0, v0, dt_scale=stride) as plain:
        plain.step()
        xp, vp = plain.positions(), plain.velocities()
    ex, ev = xp + c[:, :3], vp + c[:, 3:]
    p = sc.params
    inside = (np.abs(ex - np.asarray(p.boxCen, np.float32)) < np.asarray(p.boxDim, np.float32)).all(1)
    assert inside.mean() > 0.5 and np.abs(c).max() > 0
    tol_x = 4 * np.spacing(np.abs(ex[inside]))
    tol_v = 4 * np.spacing(np.abs(ev[inside]))
    assert (np.abs(xl[inside] - ex[inside]) <= tol_x).all()
    assert (np.abs(vl[inside] - ev[inside]) <= tol_v).all()


def test_training_lowers_loss_and_corrects_the_long_step(sphlib):
    sc = small()
    stride, steps = 4, 200
    with make(sphlib, sc) as sim:
        rep = sim.train_corrector(trainSteps=steps, stride=stride, epochs=4, batchTiles=16, auditInterval=0,
                                  seed=3)
        ref_pos, ref_vel = sim.positions(), sim.velocities()  # plain trajectory at t = steps*dt
        assert rep.samples == (steps - stride + 1) * sc.n
        assert rep.optimizerSteps > 0 and rep.lastEpochLoss < rep.firstEpochLoss
        model = sim.save_corrector()
        # learned steps from the same start cover the same time
        sim.write_state(sc.positions, sc.velocities)
        sim.step(mode=sphlib.SPH_STEP_LEARNED, count=steps // stride)
        lpos, lvel = sim.positions(), sim.velocities()
        r = sim.corrector_report()
        assert r.learnedSteps == steps // stride and r.audits == 0
    with make(sphlib, sc, dt_scale=stride) as coarse:  # the uncorrected long step
        coarse.step(count=steps // stride)
        cpos, cvel = coarse.positions(), coarse.velocities()
    rho_ref = density_at(sphlib, sc, ref_pos, ref_vel)
    err_l = np.abs(density_at(sphlib, sc, lpos, lvel) - rho_ref) / rho_ref
    err_c = np.abs(density_at(sphlib, sc, cpos, cvel) - rho_ref) / rho_ref
    print("mean density error: learned %.3e, uncorrected %.3e; loss %.3f -> %.3f"
          % (err_l.mean(), err_c.mean(), rep.firstEpochLoss, rep.lastEpochLoss))
    assert np.isfinite(lpos).all()
    assert err_l.mean() < err_c.mean()
    assert err_l.mean() < 0.01
    # a saved model loads back to the same predictions
    with make(sphlib, sc) as again:
        again.load_corrector(model)
        f = np.random.default_rng(0).normal(0, 1, (256, IN)).astype(np.float32)
        with make(sphlib, sc) as other:
            other.load_corrector(model)
            np.testing.assert_array_equal(again.corrector_predict(f), other.corrector_predict(f))


def test_audit_rolls_back_to_the_plain_solver(sphlib):
    # the per-step search (the lists' form: the next test)
    sc = tiny()
    blob = random_blob(5)
    k, stride = 3, 4
    with make(sphlib, sc, skin=0.0) as sim:
        sim.load_corrector(blob, stride=stride, auditInterval=1, densityTolerance=0.0)
        sim.step(mode=sphlib.SPH_STEP_LEARNED, count=k)
        pos, vel = sim.positions(), sim.velocities()
        rep = sim.corrector_report()
    assert rep.audits == k and rep.rollbacks == k and rep.maxAuditError > 0
    with make(sphlib, sc, skin=0.0) as plain:
        plain.step(count=k * stride)
        np.testing.assert_array_equal(pos, plain.positions())
        np.testing.assert_array_equal(vel, plain.velocities())


def test_audit_over_the_lists_rolls_back_to_the_plain_solver(sphlib):
    """With reused neighbour lists the audit's plain solver is the plain
    solver over the lists: one audited step with tolerance 0 gives the bits
    of four plain steps of a new handle (the first builds the lists, the
    others reuse them)."""
    sc = tiny()
    stride = 4
    with make(sphlib, sc) as sim:
        sim.load_corrector(random_blob(5), stride=stride, auditInterval=1, densityTolerance=0.0)
        sim.step(mode=sphlib.SPH_STEP_LEARNED)
        pos, vel = sim.positions(), sim.velocities()
        rep = sim.corrector_report()
    assert rep.audits == 1 and rep.rollbacks == 1
    with make(sphlib, sc) as plain:
        plain.step(count=stride)
        assert plain.neighbour_builds() == 1
        np.testing.assert_array_equal(pos, plain.positions())
        np.testing.assert_array_equal(vel, plain.velocities())


def test_audit_at_the_default_tolerance_rolls_back_a_drifting_corrector(sphlib):
    """At the default 1 % density tolerance the audit keeps a corrector that
    adds nothing (the uncorrected long step's densities differ from four
    short steps' by far less) and rolls back one whose corrections move
    particles by up to a few tenths of their spacing: every audited step
    then ends in the plain solver's state, bit for bit."""
    sc = tiny()
    k, stride = 3, 4
    zero = random_blob(7)
    zero[:NPARAM] = 0.0                      # the network gives 0 ...
    zero[NPARAM + 48:NPARAM + 54] = 0.0      # ... and the target means are 0: no correction
    drift = random_blob(7)
    drift[NPARAM + 54:NPARAM + 60] *= 30.0   # target deviations 0.3-3 mm (spacing 12.5 mm)
    assert abs(sphlib.CorrectorConfig.default().densityTolerance - 0.01) < 1e-9
    reports, states = [], []
    for blob in (zero, drift):
        with make(sphlib, sc, skin=0.0) as sim:
            sim.load_corrector(blob, stride=stride, auditInterval=1)
            sim.step(mode=sphlib.SPH_STEP_LEARNED, count=k)
            reports.append(sim.corrector_report())
            states.append((sim.positions(), sim.velocities()))
    kept, rolled = reports
    assert kept.audits == k and kept.rollbacks == 0 and kept.maxAuditError < 0.01
    assert rolled.audits == k and rolled.rollbacks == k and rolled.maxAuditError > 0.01
    with make(sphlib, sc, skin=0.0) as plain:
        plain.step(count=k * stride)
        np.testing.assert_array_equal(states[1][0], plain.positions())
        np.testing.assert_array_equal(states[1][1], plain.velocities())


def test_audit_keeps_the_learned_result_within_tolerance(sphlib):
    # the per-step search (with reused lists the run with audits, which
    # rebuild the lists after each, would differ from the one without by the
    # rounding of the reused rows)
    sc = tiny()
    blob = random_blob(6)
    outs = []
    for interval, tol in ((1, 1e9), (0, 0.01)):
        with make(sphlib, sc, skin=0.0) as sim:
            sim.load_corrector(blob, stride=4, auditInterval=interval, densityTolerance=tol)
            sim.step(mode=sphlib.SPH_STEP_LEARNED, count=3)
            outs.append((sim.positions(), sim.velocities(), sim.corrector_report()))
    np.testing.assert_array_equal(outs[0][0], outs[1][0])
    np.testing.assert_array_equal(outs[0][1], outs[1][1])
    assert outs[0][2].audits == 3 and outs[0][2].rollbacks == 0 and outs[1][2].audits == 0


def test_learned_steps_over_reused_lists(sphlib):
    """Learned steps over the reused neighbour lists against the per-step
    search: the first (a building step) bit for bit, the later ones over the
    lists built then within rounding of the search; the lists are reused."""
    sc = small()
    blob = random_blob(9)
    with make(sphlib, sc) as sim:
        sim.step(count=40)
        x0, v0 = sim.positions(), sim.velocities()
    outs, builds = [], []
    for skin in (0.1, 0.0):
        with make(sphlib, sc, x0, v0, skin=skin) as sim:
            sim.load_corrector(blob, stride=4, auditInterval=0)
            sim.step(mode=sphlib.SPH_STEP_LEARNED)
            first = (sim.positions(), sim.velocities())
            sim.step(mode=sphlib.SPH_STEP_LEARNED, count=7)
            outs.append((first, (sim.positions(), sim.velocities())))
            builds.append(sim.neighbour_builds())
    (fa, la), (fb, lb) = outs
    np.testing.assert_array_equal(fa[0], fb[0])
    np.testing.assert_array_equal(fa[1], fb[1])
    assert 1 <= builds[0] < 8 and builds[1] == 0
    # eight long steps: the reused rows sum the same pairs in another grouping
    assert np.abs(la[0] - lb[0]).max() <= 1e-6
    assert np.abs(la[1] - lb[1]).max() <= 1e-4 * max(1.0, np.abs(lb[1]).max())


def test_learned_steps_after_an_audit_over_the_lists(sphlib):
    """An audit over the reused lists takes both densities over them and
    leaves lists that hold for the state it keeps: the learned steps after
    an accepting audit match, within rounding, those of a new handle started
    from the kept state (which builds its lists there)."""
    sc = small()
    blob = random_blob(9)
    with make(sphlib, sc) as sim:
        sim.step(count=40)
        x0, v0 = sim.positions(), sim.velocities()
    with make(sphlib, sc, x0, v0) as sim:
        sim.load_corrector(blob, stride=4, auditInterval=2, densityTolerance=1e9)
        sim.step(mode=sphlib.SPH_STEP_LEARNED, count=2)  # a learned step, then an audited one
        rep = sim.corrector_report()
        assert rep.audits == 1 and rep.rollbacks == 0 and rep.maxAuditError > 0
        x1, v1 = sim.positions(), sim.velocities()
        sim.step(mode=sphlib.SPH_STEP_LEARNED)           # over the lists the audit left
        a = (sim.positions(), sim.velocities())
    with make(sphlib, sc, x1, v1) as sim:
        sim.load_corrector(blob, stride=4, auditInterval=0)
        sim.step(mode=sphlib.SPH_STEP_LEARNED)
        b = (sim.positions(), sim.velocities())
    assert np.abs(a[0] - b[0]).max() <= 1e-6
    assert np.abs(a[1] - b[1]).max() <= 1e-4 * max(1.0, np.abs(b[1]).max())


def test_learned_graph_matches_eager(sphlib):
    sc = tiny()
    blob = random_blob(7)
    outs = []
    for graph in (False, True, True):
        with make(sphlib, sc) as sim:
            sim.load_corrector(blob, stride=4, auditInterval=2, densityTolerance=0.5)
            if graph:
                sim.step(mode=sphlib.SPH_STEP_LEARNED, count=5)
            else:
                for _ in range(5):
                    sim.step(mode=sphlib.SPH_STEP_LEARNED)
            outs.append((sim.positions(), sim.velocities()))
    for o in outs[1:]:
        np.testing.assert_array_equal(o[0], outs[0][0])
        np.testing.assert_array_equal(o[1], outs[0][1])


def test_learned_step_needs_a_corrector(sphlib):
    with make(sphlib, tiny()) as sim:
        with pytest.raises(sphlib.SphError):
            sim.step(mode=sphlib.SPH_STEP_LEARNED)
