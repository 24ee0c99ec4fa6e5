"""The allocation-free neighbour-table entry point, sph_cell_tables_noalloc().

It serves callers that cannot allocate device memory where they need the cell
tables (a frame loop an allocation would stall, or an application whose device
memory belongs to its own allocator): inputs and outputs are the caller's
device buffers and the intermediate data sits in one fixed array inside the
library.  These tests compare its tables with the ones sph_step() builds for
the same positions -- bit for bit, the bar of every integer table here -- on
two calls in a row, so the second call also shows that nothing the first call
left in the shared array leaks into its result.
"""
import ctypes

import numpy as np
import pytest

from cudasphnew_gb300 import scenes

pytestmark = pytest.mark.gpu

MAX_PARTICLES = 65536


def call_noalloc(sphlib, params, positions):
    torch = pytest.importorskip("torch")
    n = len(positions)
    C = params.num_cells
    vd = torch.from_numpy(np.ascontiguousarray(positions, np.float32).reshape(-1)).cuda()
    outs = [torch.full((n,), -7, dtype=torch.int32, device="cuda") for _ in range(2)]
    outs += [torch.full((C,), -7, dtype=torch.int32, device="cuda") for _ in range(2)]
    torch.cuda.synchronize()
    status = sphlib.load().sph_cell_tables_noalloc(
        ctypes.byref(params), ctypes.c_void_p(vd.data_ptr()), n,
        *[ctypes.c_void_p(o.data_ptr()) for o in outs], None)
    sphlib.check(status)
    return [o.cpu().numpy() for o in outs]


def test_noalloc_tables_match_the_step_on_two_calls(sphlib):
    sc = scenes.config1()  # 16,384 particles, 44^3 cells
    with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options) as sim:
        for _ in range(2):
            x = sim.positions()  # the positions the next step hashes
            sim.Advance()
            expected = sim.cells()
            got = call_noalloc(sphlib, sc.params, x)
            for a, b in zip(expected, got):
                np.testing.assert_array_equal(a, b)


def test_noalloc_rejects_sizes_beyond_its_array(sphlib):
    torch = pytest.importorskip("torch")
    sc = scenes.config1()
    n = MAX_PARTICLES + 1
    buf = torch.zeros(3 * n, dtype=torch.float32, device="cuda")
    ints = torch.zeros(max(n, sc.params.num_cells), dtype=torch.int32, device="cuda")
    p = ctypes.c_void_p(ints.data_ptr())
    L = sphlib.load()
    status = L.sph_cell_tables_noalloc(ctypes.byref(sc.params), ctypes.c_void_p(buf.data_ptr()), n,
                                       p, p, p, p, None)
    assert status == 1
    assert b"SPH_NOALLOC_MAX_PARTICLES" in L.sph_last_error()


def raw_call(sphlib, params, positions, stream=None):
    """The entry point's status for `positions` (no raise), outputs discarded."""
    torch = pytest.importorskip("torch")
    n = len(positions)
    vd = torch.from_numpy(np.ascontiguousarray(positions, np.float32).reshape(-1)).cuda()
    ints = [torch.zeros(max(n, params.num_cells), dtype=torch.int32, device="cuda") for _ in range(4)]
    torch.cuda.synchronize()
    return sphlib.load().sph_cell_tables_noalloc(
        ctypes.byref(params), ctypes.c_void_p(vd.data_ptr()), n,
        *[ctypes.c_void_p(o.data_ptr()) for o in ints], ctypes.c_void_p(stream))


def test_noalloc_at_its_particle_limit(sphlib):
    # 64 x 32 x 32 = 65,536 particles, exactly SPH_NOALLOC_MAX_PARTICLES
    sc = scenes.dam_break(64, 32, 32, (0.0, 0.0, 0.0), (1.0, 0.5, 0.5), 11, "noalloc_max", 1)
    assert sc.n == MAX_PARTICLES
    with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options) as sim:
        for _ in range(2):
            x = sim.positions()
            sim.Advance()
            expected = sim.cells()
            got = call_noalloc(sphlib, sc.params, x)
            for a, b in zip(expected, got):
                np.testing.assert_array_equal(a, b)


def test_noalloc_at_its_cell_limit(sphlib):
    # the 16,384-particle scene on a 64^3 grid: 262,144 cells, exactly SPH_NOALLOC_MAX_CELLS
    sc = scenes.config1()
    p = type(sc.params).from_buffer_copy(bytes(sc.params))
    for a in range(3):
        p.gridDim[a] = 64
    assert p.num_cells == 262144
    with sphlib.ParticleSimulation(p, sc.positions, sc.velocities, sc.options) as sim:
        x = sim.positions()
        sim.Advance()
        expected = sim.cells()
    got = call_noalloc(sphlib, p, x)
    for a, b in zip(expected, got):
        np.testing.assert_array_equal(a, b)
    p.gridDim[0] = 65  # one plane of cells too many
    assert raw_call(sphlib, p, x) == 1
    assert b"SPH_NOALLOC_MAX_CELLS" in sphlib.load().sph_last_error()


def test_noalloc_flags_bad_positions_and_recovers(sphlib):
    sc = scenes.config1()
    good = sc.positions.copy()
    nan = good.copy()
    nan[100, 1] = np.nan
    assert raw_call(sphlib, sc.params, nan) == 7  # SPH_ERR_NON_FINITE
    far = good.copy()
    # far below the grid in z: the reference's hash wraps x and y within their
    # rows (C remainder), but a negative z plane makes the whole hash negative
    far[200] = (0.5, 0.5, -5.0)
    assert raw_call(sphlib, sc.params, far) == 4  # SPH_ERR_OUT_OF_DOMAIN
    # the flags word in the shared array is cleared by the next call
    with sphlib.ParticleSimulation(sc.params, good, sc.velocities, sc.options) as sim:
        sim.Advance()
        expected = sim.cells()
    got = call_noalloc(sphlib, sc.params, good)
    for a, b in zip(expected, got):
        np.testing.assert_array_equal(a, b)


def test_noalloc_refuses_a_capturing_stream(sphlib):
    torch = pytest.importorskip("torch")
    sc = scenes.config1()
    call_noalloc(sphlib, sc.params, sc.positions)  # the device's first call comes before any capture
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    vd = torch.from_numpy(np.ascontiguousarray(sc.positions, np.float32).reshape(-1)).cuda()
    ints = torch.zeros(4 * max(sc.n, sc.params.num_cells), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    with torch.cuda.graph(g, stream=s):
        status = sphlib.load().sph_cell_tables_noalloc(
            ctypes.byref(sc.params), ctypes.c_void_p(vd.data_ptr()), sc.n,
            *[ctypes.c_void_p(ints.data_ptr() + 4 * k * max(sc.n, sc.params.num_cells)) for k in range(4)],
            ctypes.c_void_p(s.cuda_stream))
    assert status == 6  # SPH_ERR_NOT_SUPPORTED, nothing enqueued
    torch.cuda.synchronize()
