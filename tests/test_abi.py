"""CPU tests of the C ABI: the shared library loads, exports every entry point
include/sph.h declares, and the ctypes structs match the header's layout."""
import ctypes
import os
import re
import subprocess
import tempfile

import pytest

from cudasphnew_gb300 import lib as sphmod
from cudasphnew_gb300 import params as P

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "sph.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sph_[a-z_]+)\s*\(", text)))


def test_header_declares_what_the_binding_binds():
    assert declared_functions() == sorted(sphmod.SIGNATURES)


def test_library_exports_every_declared_symbol(sphlib):
    L = ctypes.CDLL(sphlib.LIB_PATH)
    for name in declared_functions():
        assert hasattr(L, name), name


def _c_layout():
    src = r"""
#include <stdio.h>
#include <stddef.h>
#include "sph.h"
#define O(T, f) printf(#T "." #f " %zu\n", offsetof(T, f))
int main(void) {
    printf("SimulationParameters %zu\n", sizeof(SimulationParameters));
    printf("sph_options %zu\n", sizeof(sph_options));
    printf("sph_boundary_desc %zu\n", sizeof(sph_boundary_desc));
    printf("sph_counts %zu\n", sizeof(sph_counts));
    printf("sph_diagnostics %zu\n", sizeof(sph_diagnostics));
    O(sph_diagnostics, kineticEnergy); O(sph_diagnostics, densityMaxRelError);
    printf("sph_corrector_config %zu\n", sizeof(sph_corrector_config));
    printf("sph_corrector_report %zu\n", sizeof(sph_corrector_report));
    O(sph_corrector_config, seed); O(sph_corrector_config, densityTolerance);
    O(sph_corrector_report, trainMilliseconds); O(sph_corrector_report, maxAuditError);
    printf("SPH_CORRECTOR_FLOATS %d\n", SPH_CORRECTOR_FLOATS);
    printf("SPH_CORRECTOR_WEIGHTS %d\n", SPH_CORRECTOR_WEIGHTS);
    O(SimulationParameters, numParticles); O(SimulationParameters, timeStep);
    O(SimulationParameters, poly6); O(SimulationParameters, laplViscSub);
    O(SimulationParameters, boxDim); O(SimulationParameters, restitution);
    O(sph_options, splitMin); O(sph_options, splitMax);
    O(sph_boundary_desc, gridSpacing); O(sph_boundary_desc, numShapes); O(sph_boundary_desc, shapes);
    return 0;
}
"""
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "layout.c")
        exe = os.path.join(d, "layout")
        open(c, "w").write(src)
        subprocess.run(["gcc", "-std=c99", "-I", os.path.dirname(HEADER), c, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    return {k: int(v) for k, v in (line.split() for line in out.strip().splitlines())}


def test_struct_layouts_match_header():
    lay = _c_layout()
    assert lay["SimulationParameters"] == ctypes.sizeof(P.SimulationParameters)
    assert lay["sph_options"] == ctypes.sizeof(P.Options)
    assert lay["sph_boundary_desc"] == ctypes.sizeof(P.BoundaryDesc)
    assert lay["sph_counts"] == ctypes.sizeof(sphmod.Counts)
    assert lay["sph_diagnostics"] == ctypes.sizeof(sphmod.Diagnostics)
    assert lay["sph_corrector_config"] == ctypes.sizeof(sphmod.CorrectorConfig)
    assert lay["sph_corrector_report"] == ctypes.sizeof(sphmod.CorrectorReport)
    assert lay.pop("SPH_CORRECTOR_FLOATS") == sphmod.CORRECTOR_FLOATS
    assert lay.pop("SPH_CORRECTOR_WEIGHTS") == sphmod.CORRECTOR_WEIGHTS
    for key, v in lay.items():
        if "." not in key:
            continue
        t, f = key.split(".")
        cls = {"SimulationParameters": P.SimulationParameters, "sph_options": P.Options,
               "sph_boundary_desc": P.BoundaryDesc, "sph_diagnostics": sphmod.Diagnostics,
               "sph_corrector_config": sphmod.CorrectorConfig,
               "sph_corrector_report": sphmod.CorrectorReport}[t]
        assert getattr(cls, f).offset == v, key


def test_reference_struct_size():
    # particle_simulation.h:54-111: 45 four-byte scalars (arrays counted per element)
    assert ctypes.sizeof(P.SimulationParameters) == 45 * 4


def test_default_options_are_the_reference_values(sphlib):
    o = P.Options()
    sphlib.load().sph_default_options(ctypes.byref(o))
    assert o.gravityAxis == 1 and o.boxCollision == 0
    assert (o.splitMin[0], o.splitMax[0]) == pytest.approx((0.2, 0.5))
    # reused neighbour lists are on by default for plain steps; the Python scenes agree
    assert o.neighbourSkin == pytest.approx(0.1) == P.default_options().neighbourSkin


def test_neighbour_skin_range_without_gpu(sphlib):
    L = sphlib.load()
    p = P.dam_break_params((0, 0, 0), (1, 1, 1), 4)
    buf = (ctypes.c_float * 12)()
    h = ctypes.c_void_p()
    for bad in (-0.1, 0.41, float("nan")):
        o = P.default_options()
        o.neighbourSkin = bad
        st = L.sph_create(ctypes.byref(p), ctypes.byref(o), buf, None, None, ctypes.byref(h))
        assert st == 1 and h.value is None and b"neighbourSkin" in L.sph_last_error()


def test_status_strings_and_errors_without_gpu(sphlib):
    L = sphlib.load()
    assert L.sph_status_string(0) == b"ok"
    assert L.sph_status_string(4) == b"particle outside the cell grid"
    # invalid arguments are rejected before any device call
    h = ctypes.c_void_p()
    st = L.sph_create(None, None, None, None, None, ctypes.byref(h))
    assert st == 1 and h.value is None
    assert b"Exception thrown in FILE:" in L.sph_last_error()
    p = P.dam_break_params((0, 0, 0), (1, 1, 1), 4)
    p.compactSupport = 2 * p.gridSpacing
    buf = (ctypes.c_float * 12)()
    st = L.sph_create(ctypes.byref(p), None, buf, None, None, ctypes.byref(h))
    assert st == 1 and b"27-cell stencil" in L.sph_last_error()


def test_empty_and_oversized_inputs_are_refused_without_gpu(sphlib):
    """No particles, or more than the 2^30 the index types hold, are refused
    before any device call, and so is every call on no handle."""
    L = sphlib.load()
    buf = (ctypes.c_float * 12)()
    h = ctypes.c_void_p()
    for count in (0, (1 << 30) + 1):
        p = P.dam_break_params((0, 0, 0), (1, 1, 1), 4)
        p.numParticles = count
        st = L.sph_create(ctypes.byref(p), None, buf, None, None, ctypes.byref(h))
        assert st == 1 and h.value is None and b"numParticles" in L.sph_last_error()
    assert L.sph_step(None, 0) == 1
    assert L.sph_step_many(None, 0, 2) == 1
    assert L.sph_read(None, 0, buf, 48) == 1
    assert L.sph_read_async(None, 0, buf, 48) == 1
    assert L.sph_write(None, 0, buf, 48) == 1
    assert L.sph_synchronize(None) == 1
    assert L.sph_destroy(None) == 0


def test_boundary_dims_without_gpu(sphlib):
    import numpy as np
    p = P.example01_params()
    d = P.example01_boundary(p)
    dims = np.zeros(3, np.uint32)
    sphlib.check(sphlib.load().sph_boundary_dims(ctypes.byref(d), dims.ctypes.data_as(ctypes.c_void_p)))
    assert tuple(dims) == (259, 194, 130) == d.dims()


def test_missing_library_fails_loudly(tmp_path):
    with pytest.raises(RuntimeError, match="missing"):
        sphmod._lib_backup = sphmod._lib
        try:
            sphmod._lib = None
            sphmod.load(str(tmp_path / "nope.so"))
        finally:
            sphmod._lib = sphmod._lib_backup


def test_cpp_header_compiles_and_links(sphlib, tmp_path):
    """include/particle_simulation.h builds a program that links the library."""
    src = os.path.join(ROOT, "tests", "cpp", "example01_driver.cpp")
    exe = tmp_path / "example01_driver"
    libdir = os.path.dirname(sphlib.LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), src, "-o", str(exe),
                    "-L", libdir, "-lsph_gb300", f"-Wl,-rpath,{libdir}"], check=True)
    assert exe.exists()
