"""CPU checks of the renderer's host parts: the camera matrices against the
oracle's float64 restatement of cgtkGLLookAt / cgtkGLPerspective, the
PortablePixmap P3 layout of sph_image_save_ppm, and the oracle's splat
restatement itself (coverage, shading, occlusion, depth ties)."""
import numpy as np

from cudasphnew_gb300 import lib

import oracle


def test_camera_matrices():
    cam = lib.Camera.look((0.0, 0.2, 1.3), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 60.0, 1280.0 / 800.0, 0.1, 100.0)
    np.testing.assert_allclose(np.array(cam.view), oracle.look_at((0, 0.2, 1.3), (0, 0, 0), (0, 1, 0)),
                               rtol=0, atol=1e-6)
    np.testing.assert_allclose(np.array(cam.proj), oracle.perspective(60.0, 1.6, 0.1, 100.0), rtol=1e-6, atol=1e-6)


def test_ppm_layout(tmp_path):
    rgba = np.zeros((2, 3, 4), np.uint8)
    rgba[..., 0] = np.arange(6).reshape(2, 3)
    rgba[..., 1] = 100
    rgba[..., 2] = 255
    rgba[..., 3] = 7  # alpha is not written
    path = str(tmp_path / "img.ppm")
    lib.save_ppm(path, rgba)
    lines = open(path).read().split("\n")
    assert lines[:3] == ["P3", "3 2", "255"]
    vals = [int(v) for v in lines[3:] if v]
    assert vals == [c for px in rgba.reshape(-1, 4) for c in px[:3]]


def test_oracle_splat_coverage_occlusion_and_ties():
    """The renderer's float64 restatement: a sphere impostor covers the pixels
    whose centres fall inside its projected disc, shaded 0.9 + 0.1 n_z (full
    colour at the centre, 90 % at the rim), a nearer particle hides a farther
    one whatever the draw order, an exact depth tie keeps the first drawn,
    and uncovered pixels stay white."""
    W = H = 64
    view = oracle.look_at((0.0, 0.0, 5.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0))
    proj = oracle.perspective(30.0, 1.0, 0.1, 100.0)
    R = 0.2
    rgba, win = oracle.render_splats(view, proj, [([[0.0, 0.0, 0.0]], R, (1.0, 0.0, 0.0))], W, H)
    # coverage: pixel centres within the disc of radius P00 R / w (NDC) at the centre
    Pm = np.asarray(proj).reshape(4, 4).T
    r_ndc = Pm[0, 0] * R / 5.0
    ii, jj = np.meshgrid(np.arange(W), np.arange(H))
    u = ((ii + 0.5) * 2 / W - 1) / r_ndc
    v = ((jj + 0.5) * 2 / H - 1) / r_ndc
    want = (u * u + v * v) <= 1
    np.testing.assert_array_equal(win[::-1] >= 0, want)  # rows top to bottom
    assert (rgba[win < 0] == 255).all()
    c = rgba[H // 2, W // 2]
    assert c[0] >= 250 and c[1] == 0 and c[2] == 0
    # shading 0.9 + 0.1 n_z of the impostor's normal: 255 at the centre, 230 at the rim
    nz = np.sqrt(np.clip(1 - (u * u + v * v), 0, 1))
    red = np.rint(255 * (0.9 + 0.1 * nz))
    assert (np.abs(rgba[::-1][want][:, 0].astype(int) - red[want]) <= 1).all()
    # occlusion: the nearer particle wins in either draw order
    near, far = ([[0.0, 0.0, 1.0]], R, (0.0, 1.0, 0.0)), ([[0.0, 0.0, 0.0]], R, (0.0, 0.0, 1.0))
    for passes, nearest in (([near, far], 0), ([far, near], 1)):
        _, w2 = oracle.render_splats(view, proj, passes, W, H)
        assert w2[H // 2, W // 2] == nearest
    # tie: two particles at the same place, the first drawn keeps the pixel
    _, w3 = oracle.render_splats(view, proj, [([[0.0, 0.0, 0.0], [0.0, 0.0, 0.0]], R, (1.0, 1.0, 1.0))], W, H)
    assert set(np.unique(w3)) <= {-1, 0}
