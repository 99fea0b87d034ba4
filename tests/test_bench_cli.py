"""The bench contract's CPU reference arm runs and prints one well-formed JSON
line (small sizes; the GPU arm is exercised on the GPU)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_contract_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--n", "256",
                          "--nrhs", "2", "--steps", "1", "--warmup", "1"],
                         capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["cpu_baseline"]["kind"] in ("port", "reference")


def test_serving_workload_shape(pkg):
    """The served stream the bench times (here 40 keys and 150 requests of
    the bench's 300 and 1000): keys with their own sizes, log-uniform in
    [64, 4096], a warm request per key, and a stream of about 30 % new
    matrices whose Aeff is the key's matrix at that point (what the results
    are checked against)."""
    sys.path.insert(0, ROOT)
    import bench
    import numpy as np
    sizes, warm, reqs = bench.serving_workload(pkg, 40, 150, seed=0)
    assert len(sizes) == 40 and 64 <= sizes.min() and sizes.max() <= 4096
    assert len(np.unique(sizes)) > 30
    assert [r["key"] for r in warm] == list(range(40)) and all(r["A"] is not None for r in warm)
    assert len(reqs) == 150 and 0.15 < np.mean([r["A"] is not None for r in reqs]) < 0.45
    cur = {r["key"]: r["A"] for r in warm}
    for r in reqs:
        n = int(sizes[r["key"]])
        assert r["b"].shape == (n,)
        if r["A"] is not None:
            assert r["A"].shape == (n, n) and r["A"].flags.f_contiguous
            cur[r["key"]] = r["A"]
        assert r["Aeff"] is cur[r["key"]]
    again = bench.serving_workload(pkg, 40, 150, seed=0)
    assert np.array_equal(again[0], sizes) and np.array_equal(again[2][17]["b"], reqs[17]["b"])
