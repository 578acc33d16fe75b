"""Autotuner table logic (no GPU): keys, buckets, the JSON round trip and the
default for untuned workloads."""
import numpy as np

from thejoker_gb300 import autotune as at


def test_table_round_trip_and_lookup(tmp_path):
    path = str(tmp_path / "tune.json")
    assert at.load(path) == {}
    assert at.chunk_for(2, "applied", "mixed", [40], path=path) == at.DEFAULT_CHUNK
    k = at.key_for(2, "applied", "mixed", [40, 41, 39])
    assert "L=2" in k and "jitter=applied" in k and "N<=64" in k
    at.save({k: {"chunk": 2048, "ms": {"1024": 1.0, "2048": 0.9}}}, path)
    assert at.chunk_for(2, "applied", "mixed", [30, 50], path=path) == 2048
    # another bucket, precision or jitter mode is a different entry
    assert at.chunk_for(2, "applied", "mixed", [200], path=path) == at.DEFAULT_CHUNK
    assert at.chunk_for(2, "reference", "mixed", [40], path=path) == at.DEFAULT_CHUNK
    assert at.chunk_for(2, "applied", "fp64", [40], path=path) == at.DEFAULT_CHUNK


def test_epoch_buckets():
    assert at._epoch_bucket(np.array([3, 5, 16])) == "<=16"
    assert at._epoch_bucket([17, 64]) == "<=64"
    assert at._epoch_bucket([100]) == "<=256"
    assert at._epoch_bucket([300, 400]) == ">256"
    assert at._epoch_bucket(None) == "any"
