"""CPU checks of the renderer's host parts: the camera matrices against the
oracle's float64 restatement of cgtkGLLookAt / cgtkGLPerspective, and the
PortablePixmap P3 layout of sph_image_save_ppm."""
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
