"""CPU checks of the synthetic scenes: the counter-based generator against
SplitMix64's published output, and the benchmark configurations' sizes,
lattice order and jitter bounds."""
import numpy as np

from cudasphnew_gb300 import params as P
from cudasphnew_gb300 import scenes


def test_splitmix64_published_sequence():
    # SplitMix64 seeded with 0 (Steele, Lea, Flood 2014): the first outputs
    # are the finaliser at 1, 2 and 3 times the golden gamma
    gold = int(scenes._GOLD)
    got = scenes.splitmix64(np.array([0, gold, (2 * gold) % 2**64], dtype=np.uint64))
    assert [int(v) for v in got] == [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F]


def test_uniform_range_and_resolution():
    u = scenes.uniform(7, np.arange(100000, dtype=np.uint64))
    assert u.min() >= 0.0 and u.max() < 1.0
    assert np.all(np.round(u * (1 << 24)) == u * (1 << 24))  # 24-bit values
    assert abs(u.mean() - 0.5) < 0.01
    # the seed selects a different stream
    assert not np.array_equal(u[:100], scenes.uniform(8, np.arange(100, dtype=np.uint64)))


def test_lattice_order_and_jitter():
    nx, ny, nz, s, j = 5, 4, 3, P.SPACING, 0.01 * P.H
    x = scenes.lattice_block(nx, ny, nz, (0.1, 0.2, 0.3), s, 1, j).astype(np.float64)
    assert x.shape == (nx * ny * nz, 3)
    k, jj, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    node = np.array([0.1, 0.2, 0.3]) + (np.stack([i.ravel(), jj.ravel(), k.ravel()], 1) + 0.5) * s
    assert np.abs(x - node).max() <= j * (1 + 1e-6)  # x fastest, then y, then z
    assert np.abs(x - node).max() > 0.5 * j  # the jitter is there


def test_benchmark_sizes():
    assert scenes.config1().n == 16384
    assert scenes.config3().n == 262144
    sc = scenes.config3()
    assert sc.options.childMode == 1
    f32 = lambda v: [float(np.float32(a)) for a in v]
    assert list(sc.options.splitMin) == f32([0.4] * 3) and list(sc.options.splitMax) == f32([0.6] * 3)


def test_batch_sizes_log_uniform():
    ns, fr = scenes.batch_sizes()
    assert len(ns) == 64
    assert min(ns) >= 4096 and max(ns) <= 262144
    assert 3.0e6 < sum(ns) < 5.5e6  # ~4M particles in all
    assert all(0.05 <= f <= 0.2 for f in fr)
    # log-uniform: the median count sits near the geometric mean of the range
    assert 0.4 * np.sqrt(4096 * 262144) < np.median(ns) < 2.5 * np.sqrt(4096 * 262144)
