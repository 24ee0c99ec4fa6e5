"""GPU checks of host I/O through the C ABI with page-locked and pageable
buffers (sph_write, sph_read).

A page-locked source is read by the unpacking kernel itself; a pageable one
goes through a device staging buffer.  Positions and velocities read back
into page-locked memory are written there by the packing kernel (16-byte
stores where the destination is 16-byte aligned, single floats where it is
not); other fields and pageable destinations are gathered into staging and
copied back by DMA.  Every route must move the same bits, and a step driven
from page-locked buffers must equal one driven from pageable ones.
"""
import ctypes

import numpy as np
import pytest

from cudasphnew_gb300 import scenes

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def pinned(a):
    t = torch.empty(a.shape, dtype=torch.float32, pin_memory=True)
    t.numpy()[:] = a
    return t


def test_write_and_read_routes_move_the_same_bits(sphlib):
    sc = scenes.config1()
    n = sc.n
    L = sphlib.load()
    rng = np.random.default_rng(5)
    x = (sc.positions + rng.uniform(-1e-4, 1e-4, sc.positions.shape)).astype(np.float32)
    v = rng.standard_normal((n, 3)).astype(np.float32)
    with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options, sc.boundary) as sim:
        px, pv = pinned(x), pinned(v)
        sphlib.check(L.sph_write(sim._h, sphlib.FIELD_VERTEX_DATA, ctypes.c_void_p(px.data_ptr()), n * 12))
        sphlib.check(L.sph_write(sim._h, sphlib.FIELD_VELOCITY, ctypes.c_void_p(pv.data_ptr()), n * 12))
        for field, want in ((sphlib.FIELD_VERTEX_DATA, x), (sphlib.FIELD_VELOCITY, v)):
            out = torch.zeros((n, 3), dtype=torch.float32, pin_memory=True)
            sphlib.check(L.sph_read(sim._h, field, ctypes.c_void_p(out.data_ptr()), n * 12))
            np.testing.assert_array_equal(out.numpy(), want)
            np.testing.assert_array_equal(sim.read(field), want)  # pageable destination
        # the handle keeps its own copy: the source may change after a sync
        sim.synchronize()
        px.numpy()[:] = 0.0
        np.testing.assert_array_equal(sim.positions(), x)


def test_step_from_pinned_equals_step_from_pageable(sphlib):
    sc = scenes.config1()
    n = sc.n
    L = sphlib.load()
    outs = []
    for route in ("pinned", "pageable"):
        with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options, sc.boundary) as sim:
            sim.step(count=3)
            x, v = sim.positions(), sim.velocities()
            res = []
            for _ in range(3):
                if route == "pinned":
                    px, pv = pinned(x), pinned(v)
                    sphlib.check(L.sph_write(sim._h, sphlib.FIELD_VERTEX_DATA, ctypes.c_void_p(px.data_ptr()),
                                             n * 12))
                    sphlib.check(L.sph_write(sim._h, sphlib.FIELD_VELOCITY, ctypes.c_void_p(pv.data_ptr()),
                                             n * 12))
                    sphlib.check(L.sph_step(sim._h, sphlib.SPH_STEP_PLAIN))
                    out = torch.zeros((n, 3), dtype=torch.float32, pin_memory=True)
                    sphlib.check(L.sph_read(sim._h, sphlib.FIELD_VERTEX_DATA, ctypes.c_void_p(out.data_ptr()),
                                            n * 12))
                    x = out.numpy().copy()
                else:
                    sim.write_state(x, v)
                    sim.Advance()
                    x = sim.positions()
                v = sim.velocities()
                res.append((x, v))
            outs.append(res)
    for (xa, va), (xb, vb) in zip(*outs):
        np.testing.assert_array_equal(xa, xb)
        np.testing.assert_array_equal(va, vb)


@pytest.mark.parametrize("shift", [0, 1, 3])
def test_read_into_page_locked_memory_at_any_alignment(sphlib, shift):
    # 693 particles: the last block of 256 is partial and 693 * 3 floats leave a
    # ragged tail of single floats after the 16-byte stores
    sc = scenes.dam_break(7, 9, 11, (0, 0, 0), (0.5, 0.5, 0.5), 3, "io_ragged", 0)
    n = sc.n
    assert n == 693
    L = sphlib.load()
    rng = np.random.default_rng(11)
    v = rng.standard_normal((n, 3)).astype(np.float32)
    with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options, sc.boundary) as sim:
        sim.write_state(sc.positions, v)
        sim.step(count=2)
        for field, want in ((sphlib.FIELD_VERTEX_DATA, sim.positions()), (sphlib.FIELD_VELOCITY, sim.velocities())):
            # a page-locked buffer entered `shift` floats after its start, with
            # guard values around the destination
            buf = torch.full((n * 3 + 8,), -7.0, dtype=torch.float32, pin_memory=True)
            dst = buf[shift:shift + n * 3]
            sphlib.check(L.sph_read(sim._h, field, ctypes.c_void_p(dst.data_ptr()), n * 12))
            np.testing.assert_array_equal(dst.numpy().reshape(n, 3), want)
            assert np.all(buf.numpy()[:shift] == -7.0) and np.all(buf.numpy()[shift + n * 3:] == -7.0)


def test_pipelined_loop_equals_the_blocking_loop(sphlib):
    """write (page-locked) + step + sph_read_async in a loop -- each step's
    uploads issued while the previous step and its read-back are still queued,
    so they take the overlapped path -- gives every step's result bit for bit
    as write + step + sph_read does."""
    sc = scenes.config1()
    n = sc.n
    L = sphlib.load()
    rng = np.random.default_rng(3)
    steps = 6
    xs = [pinned((sc.positions + rng.uniform(-2e-4, 2e-4, sc.positions.shape)).astype(np.float32))
          for _ in range(steps)]
    vs = [pinned(rng.uniform(-0.5, 0.5, (n, 3)).astype(np.float32)) for _ in range(steps)]
    results = {}
    for mode in ("blocking", "pipelined"):
        outs = [torch.zeros((n, 3), dtype=torch.float32, pin_memory=True) for _ in range(steps)]
        with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options, sc.boundary) as sim:
            sim.step(count=2)
            sim.synchronize()
            for k in range(steps):
                sphlib.check(L.sph_write(sim._h, sphlib.FIELD_VERTEX_DATA, ctypes.c_void_p(xs[k].data_ptr()), n * 12))
                sphlib.check(L.sph_write(sim._h, sphlib.FIELD_VELOCITY, ctypes.c_void_p(vs[k].data_ptr()), n * 12))
                sphlib.check(L.sph_step(sim._h, sphlib.SPH_STEP_PLAIN))
                read = L.sph_read if mode == "blocking" else L.sph_read_async
                sphlib.check(read(sim._h, sphlib.FIELD_VERTEX_DATA, ctypes.c_void_p(outs[k].data_ptr()), n * 12))
            sim.synchronize()
        results[mode] = [o.numpy().copy() for o in outs]
    for a, b in zip(results["blocking"], results["pipelined"]):
        np.testing.assert_array_equal(a, b)
    assert not np.array_equal(results["blocking"][0], results["blocking"][1])


def test_write_while_busy_is_ordered_before_later_work(sphlib):
    """A page-locked write issued while steps are still queued lands before
    anything enqueued after it: the next read returns the written state."""
    sc = scenes.config1()
    n = sc.n
    L = sphlib.load()
    rng = np.random.default_rng(9)
    x = pinned((sc.positions + rng.uniform(-1e-4, 1e-4, sc.positions.shape)).astype(np.float32))
    v = pinned(rng.standard_normal((n, 3)).astype(np.float32))
    with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options, sc.boundary) as sim:
        sim.step(count=2)
        sim.synchronize()
        sphlib.check(L.sph_step_many(sim._h, sphlib.SPH_STEP_PLAIN, 20))  # queued, not waited for
        sphlib.check(L.sph_write(sim._h, sphlib.FIELD_VERTEX_DATA, ctypes.c_void_p(x.data_ptr()), n * 12))
        sphlib.check(L.sph_write(sim._h, sphlib.FIELD_VELOCITY, ctypes.c_void_p(v.data_ptr()), n * 12))
        np.testing.assert_array_equal(sim.positions(), x.numpy())
        np.testing.assert_array_equal(sim.velocities(), v.numpy())


def test_read_async_refuses_host_side_fields(sphlib):
    sc = scenes.dam_break(8, 8, 8, (0, 0, 0), (0.5, 0.5, 0.5), 3, "io_tiny", 0)
    L = sphlib.load()
    with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options, sc.boundary) as sim:
        sim.step()
        buf = np.zeros(sc.n * 10, np.float32)
        for field in (sphlib.FIELD_SIMULATION_DATA, sphlib.FIELD_STATE):
            assert L.sph_read_async(sim._h, field, buf.ctypes.data, buf.nbytes) != 0


@pytest.mark.parametrize("pinned_dst", [True, False])
def test_read_async_fields_equal_blocking_reads(sphlib, pinned_dst):
    """Every field sph_read_async takes, into page-locked or pageable memory,
    holds after sph_synchronize what sph_read gives."""
    sc = scenes.config1()
    n = sc.n
    L = sphlib.load()
    fields = {sphlib.FIELD_VERTEX_DATA: 3, sphlib.FIELD_VELOCITY: 3, sphlib.FIELD_ACCELERATION: 3,
              sphlib.FIELD_DENSITY: 1, sphlib.FIELD_PRESSURE: 1}
    with sphlib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options, sc.boundary) as sim:
        sim.step(count=3)
        outs = {}
        for f, c in fields.items():
            if pinned_dst:
                buf = torch.zeros((n * c,), dtype=torch.float32, pin_memory=True)
                ptr, arr = buf.data_ptr(), buf.numpy()
            else:
                arr = np.zeros(n * c, np.float32)
                ptr = arr.ctypes.data
            sphlib.check(L.sph_read_async(sim._h, f, ctypes.c_void_p(ptr), n * c * 4))
            outs[f] = (arr, buf if pinned_dst else None)
        sim.synchronize()
        for f, (arr, _) in outs.items():
            np.testing.assert_array_equal(arr.reshape(sim.read(f).shape), sim.read(f))


def test_batch_writes_while_busy_keep_scene_lanes(sphlib):
    """A batched handle's page-locked writes issued behind queued steps land
    in order and keep each particle's scene."""
    scs = [scenes.batched_scene(k, f, 300 + i, f"io{i}") for i, (k, f) in enumerate(((1500, 0.05), (2500, 0.1)))]
    L = sphlib.load()
    with sphlib.ParticleSimulation.batch(scs, scs[0].options) as sim:
        n = sim.n
        sim.step(count=2)
        x, v = sim.positions(), sim.velocities()
        px, pv = pinned(x), pinned(v)
        sphlib.check(L.sph_step_many(sim._h, sphlib.SPH_STEP_PLAIN, 10))  # queued
        sphlib.check(L.sph_write(sim._h, sphlib.FIELD_VERTEX_DATA, ctypes.c_void_p(px.data_ptr()), n * 12))
        sphlib.check(L.sph_write(sim._h, sphlib.FIELD_VELOCITY, ctypes.c_void_p(pv.data_ptr()), n * 12))
        sim.step(count=3)
        got = sim.positions()
    with sphlib.ParticleSimulation.batch(scs, scs[0].options) as ref:
        ref.step(count=2)
        ref.step(count=3)
        np.testing.assert_array_equal(got, ref.positions())
