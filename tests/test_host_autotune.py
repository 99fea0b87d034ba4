"""The batched autotuner's host side on the CPU: the distribution signature
that keys its cache, the cache file's round trip, and that a cached schedule
is returned without touching the device (the role of the preferences
LinearSolve's autotuner writes and src/preferences.jl reads back).  The
search itself times the device and runs in the GPU bench."""
from importlib import import_module

import numpy as np
import pytest


def test_signature_keys_the_distribution(pkg):
    at = import_module(pkg.__name__ + ".autotune")
    rng = np.random.default_rng(0)
    s1 = rng.integers(8, 257, size=20000)
    s2 = rng.permutation(s1)
    assert at.signature(s1, "fp32") == at.signature(s2, "fp32")  # order does not matter
    assert at.signature(s1, "fp32") != at.signature(s1, "fp64")
    assert at.signature(s1, "fp32") != at.signature(np.full(20000, 32), "fp32")
    assert at.signature(s1, "fp32") != at.signature(s1[:5000], "fp32")  # count in thousands


def test_cached_schedule_needs_no_device(pkg, tmp_path, monkeypatch):
    at = import_module(pkg.__name__ + ".autotune")
    monkeypatch.setenv("GBLU_AUTOTUNE_FILE", str(tmp_path / "tune.json"))
    sizes = np.arange(8, 257, dtype=np.int64)
    sig = at.signature(sizes, "fp64")
    sched = {"upper": [64, 256], "threads": [128, 256], "panel": [8, 16], "ctas": [0, 304],
             "ms": 1.5, "signature": sig, "precision": "fp64", "count": len(sizes), "trials": 9}
    at._store_cache({sig: sched})
    assert at._load_cache() == {sig: sched}

    class NoDevice:
        @property
        def lib(self):
            raise AssertionError("the device was touched")

    assert at.tune(NoDevice(), sizes, precision="fp64") == sched
    with pytest.raises(AssertionError):  # a new distribution is searched (on the device)
        at.tune(NoDevice(), sizes[:10], precision="fp64")


def test_unreadable_cache_is_empty(pkg, tmp_path, monkeypatch):
    at = import_module(pkg.__name__ + ".autotune")
    p = tmp_path / "tune.json"
    p.write_text("{not json")
    monkeypatch.setenv("GBLU_AUTOTUNE_FILE", str(p))
    assert at._load_cache() == {}
    monkeypatch.setenv("GBLU_AUTOTUNE_FILE", str(tmp_path / "missing" / "tune.json"))
    assert at._load_cache() == {}
