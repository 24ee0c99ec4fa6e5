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
