"""The drop-in C++ header runs the reference's main-loop calls on the GPU and
matches the Python binding of the same library, bit for bit."""
import os
import subprocess

import numpy as np
import pytest

from cudasphnew_gb300 import scenes

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_example01_through_the_cpp_header(sphlib, tmp_path):
    exe = tmp_path / "example01_driver"
    libdir = os.path.dirname(sphlib.LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "example01_driver.cpp"), "-o", str(exe),
                    "-L", libdir, "-lsph_gb300", f"-Wl,-rpath,{libdir}"], check=True)
    prefix = str(tmp_path / "ex")
    out = subprocess.run([str(exe), "2", prefix], capture_output=True, text=True, check=True).stdout
    assert "particles 39304 steps 2" in out

    sc = scenes.example01()
    with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options, sc.boundary) as sim:
        sim.Advance()
        sim.Advance()
        pos = sim.positions()
        sd = sim.read(sphlib.FIELD_SIMULATION_DATA)
        h, ids, start, end = sim.cells()
    rows = np.loadtxt(prefix + "_particles.txt", skiprows=1)
    assert rows.shape == (sc.n, 9)
    # the text dump prints 6 significant digits
    np.testing.assert_allclose(rows[:, 1:4], pos, rtol=6e-6, atol=1e-9)
    np.testing.assert_allclose(rows[:, 4], sd[:, 1], rtol=6e-6)
    np.testing.assert_allclose(rows[:, 6:9], sd[:, 3:6], rtol=6e-6, atol=1e-4)
    lines = open(prefix + "_table.txt").read().splitlines()[2:]
    assert len(lines) == len(start)
    got_ids = np.array([int(l[8:20]) for l in lines[: sc.n]])
    got_start = np.array([int(l[32:44]) if l[32:44].strip() else -1 for l in lines])
    np.testing.assert_array_equal(got_ids, ids)
    np.testing.assert_array_equal(got_start, start)
