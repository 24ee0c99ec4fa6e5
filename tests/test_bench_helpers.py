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


def test_combined_roofline_arithmetic():
    sc = fake_scene(1000, (4, 5, 6))
    n, pairs, t = 2000, 30000, 10e-6
    r = bench.combined_roofline(sc, n, pairs, t, hbm_gbs=1000.0, sms=2, max_mhz=1000.0)
    assert r["bytes"] == 56 * n + 8 * 1000 + 12 * 120
    assert r["flop"] == 40.0 * pairs
    fp32 = 2 * 128 * 2 * 1000.0 * 1e6
    assert r["fp32_peak_tflops"] == pytest.approx(fp32 / 1e12)
    t_bytes = r["bytes"] / 1e12
    t_flop = r["flop"] / fp32
    assert r["t_bytes_us"] == pytest.approx(t_bytes * 1e6)
    assert r["t_flop_us"] == pytest.approx(t_flop * 1e6)
    assert r["bound"] == ("fp32" if t_flop >= t_bytes else "hbm")
    assert r["frac"] == pytest.approx(max(t_bytes, t_flop) / t)


def test_combined_roofline_picks_the_binding_resource():
    sc = fake_scene(10)
    # no pairs: the bytes bind
    assert bench.combined_roofline(sc, 100, 0, 1e-6, 1000.0, 1, 1000.0)["bound"] == "hbm"
    # many pairs on a tiny GPU: the flops bind
    assert bench.combined_roofline(sc, 100, 10**9, 1e-6, 1000.0, 1, 1000.0)["bound"] == "fp32"


def test_working_set_counts_state_tables_and_maps():
    sc = fake_scene(500, (8, 8, 8))
    sc.n = 1000
    assert bench.working_set_bytes(sc) == 1000 * (16 * 6 + 8 + 4 * 3) + 8 * 501 + 8 * 8 * 8 * 20


def test_peak_source(tmp_path, monkeypatch):
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    assert bench.load_peaks() == (6800.0, "fallback")
    (tmp_path / "MEASURED_PEAKS.json").write_text(json.dumps({"hbm_gbs": 6788.3}))
    assert bench.load_peaks() == (6788.3, "measured")
