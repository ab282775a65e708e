"""Host-side state on CPU: reconstruction checkpoints (written per generation, read back by
``load_checkpoint`` as the reference's prep_data.py:297-324 does) and the autotuner's
persistent cache (keyed by device, library version, transform and point-count bucket)."""
import json
import os

import numpy as np
import torch

from cmtip_gb300 import reconstruct, tune


def test_checkpoint_round_trip(tmp_path):
    ac = torch.arange(27, dtype=torch.float64).reshape(3, 3, 3)
    quats = np.random.default_rng(0).standard_normal((5, 4)).astype(np.float32)
    reconstruct._save(str(tmp_path), 4, {"generation": 4, "ac_phased": ac, "orientations": quats,
                                         "reciprocal_extent": 0.75, "support_": None})
    path = tmp_path / "checkpoint_g4.npz"
    assert path.exists()
    ck = reconstruct.load_checkpoint(str(path))
    assert ck["generation"] == 4
    assert np.array_equal(ck["ac_phased"], ac.numpy()) and ck["ac_phased"].dtype == np.float64
    assert np.array_equal(ck["orientations"], quats) and ck["orientations"].dtype == np.float32
    assert isinstance(ck["reciprocal_extent"], float) and ck["reciprocal_extent"] == 0.75
    assert "support_" not in ck  # None entries are not written


def test_load_checkpoint_without_file_starts_at_generation_zero():
    assert reconstruct.load_checkpoint() == {"generation": 0, "orientations": None}


def test_tune_cache_persists_and_survives_a_corrupt_file(tmp_path, monkeypatch):
    cache = tmp_path / "sub" / "tune.json"
    monkeypatch.setenv("CMT_TUNE_CACHE", str(cache))
    assert tune._load_file() == {}
    tune._store_file("a", {"bin_size": 5, "maxsub": 16384})
    tune._store_file("b", {"bin_size": 8, "maxsub": 8192})
    assert json.loads(cache.read_text()) == {"a": {"bin_size": 5, "maxsub": 16384},
                                             "b": {"bin_size": 8, "maxsub": 8192}}
    assert not os.path.exists(str(cache) + ".tmp")  # written through a rename
    cache.write_text("{not json")
    assert tune._load_file() == {}
    tune._store_file("c", {"bin_size": 4, "maxsub": 2048})
    assert tune._load_file() == {"c": {"bin_size": 4, "maxsub": 2048}}


def test_tune_signature_buckets_point_counts_by_power_of_two():
    s = lambda n, **kw: tune.signature(1, 81, 32, 1e-6, n, **kw)
    assert s(2 ** 30) == s(2 ** 31 - 1) != s(2 ** 31)
    assert "|N2^30|" in s(1_310_720_000)
    assert s(1000) != tune.signature(2, 81, 32, 1e-6, 1000)
    assert s(1000) != tune.signature(1, 81, 64, 1e-6, 1000)
    assert s(1000, tag="x") != s(1000)
