"""CPU checks of the measurement arithmetic in bench.py: the interacting-pair
count behind the combined roofline, the roofline itself, the working-set
size that decides the L2 note, and where the HBM peak comes from."""
import json
import types

import numpy as np
import pytest

import bench


def test_pair_count_matches_brute_force():
    pytest.importorskip("scipy")
    rng = np.random.default_rng(11)
    pos = rng.uniform(0.0, 0.2, (600, 3)).astype(np.float32)
    h = 0.025
    x = pos.astype(np.float64)
    d2 = ((x[:, None, :] - x[None, :, :]) ** 2).sum(-1)
    want = int((d2 <= h * h).sum()) - len(pos)  # ordered pairs, i != j
    assert bench.pair_count(pos, h) == want
    assert want > 0


def fake_scene(num_cells, dims=None):
    params = types.SimpleNamespace(num_cells=num_cells)
    boundary = None if dims is None else types.SimpleNamespace(dims=lambda: dims)
    return types.SimpleNamespace(params=params, boundary=boundary)


@pytest.mark.parametrize("kernel", ["k_density", "k_force"])
def test_kernel_roofline_arithmetic(kernel):
    n, C, g3, pairs, t = 2000, 1000, 120, 30000, 10e-6
    fp32 = bench.fp32_peak(2, 1000.0)
    assert fp32 == 2 * 128 * 2 * 1000.0 * 1e6
    r = bench.kernel_roofline(kernel, n, C, g3, pairs, t, hbm_gbs=1000.0, fp32=fp32, traffic=123.0)
    if kernel == "k_density":
        assert r["algorithmic_bytes_per_launch"] == 24 * n
        assert r["flop_per_launch"] == 15 * (pairs + n)
    else:
        assert r["algorithmic_bytes_per_launch"] == 56 * n + 8 * C + 12 * g3
        assert r["flop_per_launch"] == 40 * pairs
    t_bytes = r["algorithmic_bytes_per_launch"] / 1e12
    t_flop = r["flop_per_launch"] / fp32
    assert r["achieved"] == pytest.approx(r["algorithmic_bytes_per_launch"] / t / 1e9)
    assert r["frac"] == pytest.approx(r["achieved"] / 1000.0)
    assert r["t_bytes_us"] == pytest.approx(t_bytes * 1e6)
    assert r["t_flop_us"] == pytest.approx(t_flop * 1e6)
    assert r["limiter"] == ("fp32" if t_flop >= t_bytes else "hbm")
    assert r["combined_frac"] == pytest.approx(max(t_bytes, t_flop) / t)
    assert r["traffic"] == 123.0 and r["bound"] == "hbm" and r["unit"] == "GB/s"


def test_kernel_roofline_picks_the_binding_resource():
    # no pairs: the bytes bind; many pairs on a tiny GPU: the flops bind
    assert bench.kernel_roofline("k_force", 100, 10, 0, 0, 1e-6, 1000.0, 1e9)["limiter"] == "hbm"
    assert bench.kernel_roofline("k_force", 100, 10, 0, 10**9, 1e-6, 1000.0, 1e9)["limiter"] == "fp32"


def test_profiled_traffic_only_for_the_current_sources(tmp_path, monkeypatch):
    sha = bench.kernel_sources_sha16()
    (tmp_path / "profiles").mkdir()
    (tmp_path / "profiles" / "traffic_w.md").write_text(
        "| kernel | dram bytes / launch | launches | kernel sources |\n|---|---:|---:|---|\n"
        f"| k_density | 1.5e8 | 2 | {sha} |\n| k_force | 2.5e8 | 2 | 0000000000000000 |\n")
    real = bench.kernel_sources_sha16
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    monkeypatch.setattr(bench, "kernel_sources_sha16", real)
    monkeypatch.setattr(bench, "KERNEL_SOURCES", [])
    assert bench.profiled_traffic("w") == {}  # the hash of no files differs
    monkeypatch.setattr(bench, "kernel_sources_sha16", lambda: sha)
    assert bench.profiled_traffic("w") == {"k_density": 1.5e8}  # the stale k_force row is dropped
    assert bench.profiled_traffic("missing") == {}


def test_cpu_model_is_named():
    assert isinstance(bench.cpu_model(), str) and bench.cpu_model()


def test_working_set_counts_state_tables_and_maps():
    sc = fake_scene(500, (8, 8, 8))
    sc.n = 1000
    assert bench.working_set_bytes(sc) == 1000 * (16 * 6 + 8 + 4 * 3) + 8 * 501 + 8 * 8 * 8 * 20


def test_peak_source(tmp_path, monkeypatch):
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    assert bench.load_peaks() == (6800.0, "fallback")
    (tmp_path / "MEASURED_PEAKS.json").write_text(json.dumps({"hbm_gbs": 6788.3}))
    assert bench.load_peaks() == (6788.3, "measured")


def test_kernel_hash_ignores_comments_only():
    src = 'int a = 1; // one\n/* block\n   comment */\nconst char* s = "//x /* y */";\n\nchar c = \'"\';\n'
    code = bench.code_of(src)
    assert code == 'int a = 1;\nconst char* s = "//x /* y */";\nchar c = \'"\';'
    assert bench.code_of(src.replace("one", "two").replace("block", "other")) == code
    assert bench.code_of(src.replace("a = 1", "a = 2")) != code


def test_clock_summary_reads_the_timed_region():
    def row(sm, reasons=("Not Active",) * 4):
        return ["0", str(sm), "2070", "900", "0x0", *reasons]
    c = bench.ClockSampler(0)
    c.samples = [(0.5, row(1000)), (1.0, row(2070)), (1.1, row(2060)),
                 (1.2, row(2070, ("Not Active", "Not Active", "Not Active", "Active"))), (3.0, row(900))]
    s = c.summary(0.9, 1.3)
    assert s["window"] == "timed_region" and s["samples"] == 3
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0 and s["reasons"] == ["sw_power_cap"]
    # fewer than two samples inside: the whole run's samples, and said so
    s = c.summary(2.9, 3.1)
    assert s["window"] == "warmup_and_timed_region" and s["samples"] == 5
    assert bench.ClockSampler(0).summary(0, 1)["samples"] == 0
