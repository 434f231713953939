"""Autotuner: candidate selection, cache keys and cache file handling (CPU),
and tuning a real geometry (GPU)."""

from __future__ import annotations

import numpy as np
import pytest

from gratopy_gb300 import autotune as at


def test_select_fastest_and_ties_to_smaller_split():
    assert at.select({1: 3.0, 2: 1.0, 4: 2.0, 8: 1.5}) == 2
    assert at.select({8: 1.0, 4: 1.0, 2: 2.0}) == 4
    with pytest.raises(ValueError):
        at.select({})


def test_geometry_key_distinguishes_what_changes_the_launch():
    base = at.geometry_key("GB300", "fanbeam", np.float32, (512, 512), (768, 360), 1)
    assert base == "GB300|fanbeam|float32|512x512|768x360|z1"
    assert at.geometry_key("GB300", "fanbeam", np.float64, (512, 512), (768, 360), 1) != base
    assert at.geometry_key("GB300", "radon", np.float32, (512, 512), (768, 360), 1) != base
    assert at.geometry_key("GB300", "fanbeam", np.float32, (512, 512), (768, 361), 1) != base
    stacked = at.geometry_key("GB300", "fanbeam", np.float32, (512, 512), (768, 360), 16)
    assert stacked.endswith("zN")
    assert stacked == at.geometry_key("GB300", "fanbeam", np.float32, (512, 512), (768, 360), 4)


def test_cache_roundtrip_merges_entries(tmp_path, monkeypatch):
    path = tmp_path / "sub" / "tune.json"
    assert at.load_cache(path) == {}
    at.store_cache({"a": {"fwd_split": 8, "bwd_split": 1}}, path)
    at.store_cache({"b": {"fwd_split": 2, "bwd_split": 4}}, path)
    data = at.load_cache(path)
    assert data["a"]["fwd_split"] == 8 and data["b"]["bwd_split"] == 4
    path.write_text("not json")
    assert at.load_cache(path) == {}
    monkeypatch.setenv("GRATOPY_GB300_TUNE_CACHE", str(tmp_path / "env.json"))
    assert at.cache_path() == tmp_path / "env.json"


@pytest.mark.gpu
@pytest.mark.parametrize("geom", ["radon", "fan"])
def test_tune_applies_splits_and_keeps_results(cuda_device, tmp_path, geom):
    import torch

    import gratopy_gb300 as gg
    from tests.helpers import device_settings, rel_l2

    cfg = {
        "radon": dict(geometry="radon", img_shape=(96, 80), angles=60, n_detectors=128),
        "fan": dict(geometry="fanbeam", img_shape=(96, 96), angles=72, n_detectors=140,
                    detector_width=40.0, R=70.0, RE=30.0),
    }[geom]
    ps = device_settings(cfg, cuda_device)
    x = gg.core.empty(ps.img_shape, torch.float32, "F", cuda_device)
    x.copy_(torch.rand(ps.img_shape, device=cuda_device))
    y0 = gg.forwardprojection(x, ps)
    b0 = gg.backprojection(y0, ps)
    cache = tmp_path / "tune.json"
    res = at.tune(ps, np.float32, cache_file=cache, repeats=3)
    assert res["fwd_split"] in at.SPLITS and res["bwd_split"] in at.SPLITS
    assert not res["cached"] and set(res["timings"]["fwd"]) == set(at.SPLITS)
    g = ps.gr_geometry(np.float32)
    assert (g.fwd_split, g.bwd_split) == (res["fwd_split"], res["bwd_split"])
    y1 = gg.forwardprojection(x, ps)
    b1 = gg.backprojection(y0, ps)
    assert rel_l2(y1.cpu().numpy(), y0.cpu().numpy()) < 1e-6
    assert rel_l2(b1.cpu().numpy(), b0.cpu().numpy()) < 1e-6
    again = at.tune(ps, np.float32, cache_file=cache)
    assert again["cached"] and again["fwd_split"] == res["fwd_split"]
