"""The serving client's host logic (serving.run_stream / latency_summary) on
the CPU, against a stand-in server (test infrastructure only) that answers
like gblu_serve_*: a solve-only request on an evicted key completes with
GBLU_ENOTFACTORED, which the client sends again with the matrix it was
meant for under a one-off key, never under the key itself (a newer matrix
of that key may be queued behind it).  The device server is covered by
test_gpu_serving.py."""
import threading
from importlib import import_module

import numpy as np


class _Server:
    def __init__(self, evicted):
        self.evicted = set(evicted)
        self.submitted = []
        self.out = []
        self.mu = threading.Lock()
        self.mats = {}

    def submit(self, tag, key, b, A=None):
        with self.mu:
            self.submitted.append((tag, key, A is not None))
            if A is not None:
                self.mats[key] = A
                self.evicted.discard(key)
            if A is None and key in self.evicted:
                self.out.append({"tag": tag, "status": 5, "latency_us": 10.0, "x": None})
                return
            x = np.linalg.solve(self.mats[key], b)
            self.out.append({"tag": tag, "status": 0, "latency_us": 1000.0 * (1 + tag), "x": x})

    def poll(self, max_n, wait_ms=0):
        with self.mu:
            got, self.out = self.out[:max_n], self.out[max_n:]
        return got


def test_resubmits_evicted_solves_under_one_off_keys(pkg):
    serving = import_module(pkg.__name__ + ".serving")
    rng = np.random.default_rng(0)
    n = 5
    A0 = rng.standard_normal((n, n)) + n * np.eye(n)
    A1 = rng.standard_normal((n, n)) + n * np.eye(n)
    srv = _Server(evicted=[])
    srv.mats[7] = A0
    srv.evicted.add(7)  # key 7's factors were evicted before the stream
    reqs = [
        {"key": 7, "A": None, "b": rng.standard_normal(n), "Aeff": A0},  # meant for A0: resent
        {"key": 7, "A": A1, "b": rng.standard_normal(n), "Aeff": A1},    # a newer matrix of key 7
        {"key": 7, "A": None, "b": rng.standard_normal(n), "Aeff": A1},
    ]
    done, wall = serving.run_stream(srv, reqs, rate_hz=0.0, timeout_s=10.0, resubmit_missing=True)
    by_tag = {d["tag"]: d for d in done}
    assert sorted(by_tag) == [0, 1, 2] and all(d["status"] == 0 for d in done)
    # request 0 went out twice: under key 7, then under the one-off key with its own matrix
    assert srv.submitted.count((0, 7, False)) == 1
    assert (0, serving.ONE_OFF_KEY + 0, True) in srv.submitted
    assert all(key != 7 or tag != 0 or not has_a for tag, key, has_a in srv.submitted)
    assert by_tag[0]["resubmitted"] == 1 and by_tag[1]["resubmitted"] == 0
    assert by_tag[0]["client_latency_us"] is not None
    for i, r in enumerate(reqs):
        assert np.allclose(r["Aeff"] @ by_tag[i]["x"], r["b"])
    assert np.array_equal(srv.mats[7], A1)  # the key keeps its newest matrix
    s = serving.latency_summary(done, wall)
    assert s["completed"] == 3 and s["failed"] == 0 and s["resubmitted"] == 1
    assert s["p50_ms"] == 2.0  # latencies 1, 2, 3 ms


def test_without_resubmission_failures_are_reported(pkg):
    serving = import_module(pkg.__name__ + ".serving")
    n = 3
    srv = _Server(evicted=[1])
    srv.mats[1] = np.eye(n)
    reqs = [{"key": 1, "A": None, "b": np.ones(n)}, {"key": 2, "A": 2 * np.eye(n), "b": np.ones(n)}]
    done, wall = serving.run_stream(srv, reqs, rate_hz=0.0, timeout_s=10.0)
    st = {d["tag"]: d["status"] for d in done}
    assert st == {0: 5, 1: 0}
    s = serving.latency_summary(done, wall)
    assert s["completed"] == 1 and s["failed"] == 1
