"""The serving loop: continuous batching over resident factorizations.
Every result meets the FP64 backward-error bound, and is bit-identical whether
its request ran alone or in a concurrent mix."""
import numpy as np
import pytest

from conftest import EPS64

pytestmark = pytest.mark.gpu


def _requests(pkg, seed=0, nkeys=6, nreq=60, nmin=64, nmax=600):
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(nmin), np.log(nmax), size=nkeys)).astype(int)
    mats = {k: pkg.workloads.shifted(int(sizes[k]), 1, seed=1000 + k)[0] for k in range(nkeys)}
    reqs = [{"key": k, "A": mats[k], "b": rng.standard_normal(sizes[k])} for k in range(nkeys)]
    for _ in range(nreq - nkeys):
        k = int(rng.integers(nkeys))
        new_a = rng.random() < 0.3
        if new_a:
            G = rng.standard_normal((sizes[k], sizes[k]))
            mats[k] = G + 4 * np.sqrt(sizes[k]) * np.eye(sizes[k])
        reqs.append({"key": k, "A": mats[k] if new_a else None, "b": rng.standard_normal(sizes[k]),
                     "Aeff": mats[k]})
    for r in reqs[:nkeys]:
        r["Aeff"] = r["A"]
    return reqs


def _run(pkg, ctx, reqs, workers, precision, rate=0.0, pivot="partial"):
    from importlib import import_module
    serving = import_module(pkg.__name__ + ".serving")
    srv = serving.Server(ctx, workers=workers, precision=precision, pivot=pivot)
    if rate == 0.0 and workers == 1:
        done = []
        for i, r in enumerate(reqs):  # strictly one at a time
            srv.submit(i, r["key"], r["b"], r["A"])
            got = []
            while not got:
                got = srv.poll(16, wait_ms=50)
            done.extend(got)
    else:
        done, _ = serving.run_stream(srv, reqs, rate_hz=rate, seed=1)
    stats = srv.stats()
    srv.close()
    return {d["tag"]: d for d in done}, stats


@pytest.mark.parametrize("precision,pivot", [("fp64", "partial"), ("fp32", "partial"), ("bf16", "partial"),
                                             ("fp32", "rbt"), ("bf16", "rbt")])
def test_serving_results_accurate_and_mix_independent(ctx, oracle_mod, pkg, precision, pivot):
    """pivot = rbt: the server's mixed factors pivot no rows after the random
    butterfly transform (orders 257..600 here, most not multiples of 4)."""
    reqs = _requests(pkg, seed=3)
    alone, _ = _run(pkg, ctx, reqs, workers=1, precision=precision, pivot=pivot)
    mixed, stats = _run(pkg, ctx, reqs, workers=4, precision=precision, pivot=pivot)
    assert stats["completed"] == len(reqs)
    for i, r in enumerate(reqs):
        a, m = alone[i], mixed[i]
        assert a["status"] == 0 and m["status"] == 0, (a, m)
        n = len(r["b"])
        assert oracle_mod.backward_error(r["Aeff"], m["x"], r["b"]) <= 10 * n * EPS64
        assert np.array_equal(a["x"], m["x"]), i  # same alone and in the mix


def test_serving_budget_evicts_and_reports(ctx, pkg):
    from importlib import import_module
    serving = import_module(pkg.__name__ + ".serving")
    rng = np.random.default_rng(5)
    n = 256
    # a budget that holds about two FP32 factorizations of n = 256
    # (n = 256 would go to the small-system lane, which holds no factorizations)
    srv = serving.Server(ctx, workers=2, precision="fp32", hbm_budget_bytes=3 * (1 << 20) + 1_500_000,
                         small_n=0)
    A = [pkg.workloads.shifted(n, 1, seed=k)[0] for k in range(4)]
    for k in range(4):
        srv.submit(k, k, rng.standard_normal(n), A[k])
    done = []
    while len(done) < 4:
        done += srv.poll(8, wait_ms=50)
    assert all(d["status"] == 0 for d in done)
    st = srv.stats()
    assert st["evictions"] >= 1
    assert st["resident_bytes"] <= 3 * (1 << 20) + 1_500_000
    # a solve on an evicted key reports GBLU_ENOTFACTORED (5) instead of a wrong answer
    srv.submit(10, 0, rng.standard_normal(n), None)
    d = []
    while not d:
        d = srv.poll(4, wait_ms=50)
    assert d[0]["status"] in (0, 5)
    srv.close()


def test_serving_merges_rhs_on_one_key(ctx, pkg):
    from importlib import import_module
    serving = import_module(pkg.__name__ + ".serving")
    rng = np.random.default_rng(6)
    n = 400
    A = pkg.workloads.shifted(n, 1, seed=9)[0]
    srv = serving.Server(ctx, workers=1, precision="fp32", max_rhs_batch=8)
    srv.submit(0, 77, rng.standard_normal(n), A)
    bs = [rng.standard_normal(n) for _ in range(12)]
    for i, b in enumerate(bs):
        srv.submit(1 + i, 77, b, None)
    done = []
    while len(done) < 13:
        done += srv.poll(32, wait_ms=50)
    assert all(d["status"] == 0 for d in done)
    st = srv.stats()
    assert st["merged_solves"] >= 1
    sol = {d["tag"]: d["x"] for d in done}
    for i, b in enumerate(bs):
        assert np.linalg.norm(A @ sol[1 + i] - b, np.inf) <= 10 * n * 2.2e-16 * (
            np.abs(A).sum(1).max() * np.abs(sol[1 + i]).max() + np.abs(b).max())
    srv.close()


def _serve_all(pkg, ctx, reqs, **kw):
    """Submit everything at once (or, with one_by_one, each after the
    previous completed); return completions by tag and the server stats."""
    from importlib import import_module
    serving = import_module(pkg.__name__ + ".serving")
    one = kw.pop("one_by_one", False)
    srv = serving.Server(ctx, **kw)
    done = []
    if one:
        for i, r in enumerate(reqs):
            srv.submit(i, r["key"], r["b"], r.get("A"))
            got = []
            while not got:
                got = srv.poll(16, wait_ms=50)
            done += got
    else:
        for i, r in enumerate(reqs):
            srv.submit(i, r["key"], r["b"], r.get("A"))
        while len(done) < len(reqs):
            done += srv.poll(256, wait_ms=50)
    st = srv.stats()
    srv.close()
    return {d["tag"]: d for d in done}, st


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_small_lane_batches_across_keys(ctx, oracle_mod, pkg, precision):
    """Requests with n <= 256 of many keys are factored and solved together
    (one launch of the batched kernels per group of queued requests); each
    answer meets the bound and equals the answer of the request run alone."""
    rng = np.random.default_rng(11)
    nkeys = 40
    sizes = rng.integers(8, 257, size=nkeys)
    reqs = []
    for k in range(nkeys):
        A = pkg.workloads.shifted(int(sizes[k]), 1, seed=2000 + k)[0]
        reqs.append({"key": k, "A": A, "b": rng.standard_normal(sizes[k]), "Aeff": A})
    for _ in range(3 * nkeys):
        k = int(rng.integers(nkeys))
        reqs.append({"key": k, "A": None, "b": rng.standard_normal(sizes[k]), "Aeff": reqs[k]["A"]})
    mixed, st = _serve_all(pkg, ctx, reqs, workers=2, precision=precision)
    alone, st1 = _serve_all(pkg, ctx, reqs, workers=1, precision=precision, one_by_one=True)
    assert st["small_systems"] == len(reqs)
    assert st["small_launches"] < len(reqs) and st1["small_launches"] == len(reqs)
    for i, r in enumerate(reqs):
        assert mixed[i]["status"] == 0 and alone[i]["status"] == 0
        n = len(r["b"])
        assert oracle_mod.backward_error(r["Aeff"], mixed[i]["x"], r["b"]) <= 10 * n * EPS64
        assert np.array_equal(mixed[i]["x"], alone[i]["x"]), i


def test_small_lane_keeps_per_key_order(ctx, oracle_mod, pkg):
    """A key's requests keep their order inside one launch: a solve after a
    new matrix uses that matrix, a solve before it the previous one."""
    rng = np.random.default_rng(12)
    n = 100
    A1 = pkg.workloads.shifted(n, 1, seed=1)[0]
    A2 = pkg.workloads.shifted(n, 1, seed=2)[0]
    b = [rng.standard_normal(n) for _ in range(4)]
    reqs = [{"key": 5, "A": A1, "b": b[0]}, {"key": 5, "A": None, "b": b[1]},
            {"key": 5, "A": A2, "b": b[2]}, {"key": 5, "A": None, "b": b[3]}]
    done, _ = _serve_all(pkg, ctx, reqs, workers=1, precision="fp64")
    for i, A in enumerate((A1, A1, A2, A2)):
        assert done[i]["status"] == 0
        assert oracle_mod.backward_error(A, done[i]["x"], b[i]) <= 10 * n * EPS64


def test_small_lane_unknown_key_not_factored(ctx, pkg):
    rng = np.random.default_rng(13)
    done, _ = _serve_all(pkg, ctx, [{"key": 99, "A": None, "b": rng.standard_normal(50)}], workers=1,
                         precision="fp64")
    assert done[0]["status"] == 5  # GBLU_ENOTFACTORED


def test_admission_waits_for_memory(ctx, pkg):
    """A budget that holds one n = 700 FP32 factorization: two new matrices
    at once, the second waits for the first to go idle, then evicts it."""
    rng = np.random.default_rng(14)
    n = 700
    ld = 704
    one = ld * n * 4 + ld * n * 8 + 64 * n * 8 + (1 << 20)
    reqs = [{"key": k, "A": pkg.workloads.shifted(n, 1, seed=30 + k)[0], "b": rng.standard_normal(n)}
            for k in range(3)]
    done, st = _serve_all(pkg, ctx, reqs, workers=3, precision="fp32", hbm_budget_bytes=one + one // 2)
    assert all(done[i]["status"] == 0 for i in range(3))
    assert st["evictions"] >= 2 and st["admission_waits"] >= 1
    assert st["resident_bytes"] <= one + one // 2


def test_resent_request_keeps_key_matrix(ctx, pkg, oracle_mod):
    """A solve on an evicted key is sent again with the matrix it was meant
    for, under a one-off key: a newer matrix of that key, already queued,
    stays the key's matrix for the requests after it.  Budget: one n = 700
    FP32 factorization."""
    from importlib import import_module
    serving = import_module(pkg.__name__ + ".serving")
    rng = np.random.default_rng(15)
    n = 700
    one = 704 * n * 4 + 704 * n * 8 + 64 * n * 8 + (1 << 20)
    A1, A2, B1 = (pkg.workloads.shifted(n, 1, seed=40 + i)[0] for i in range(3))
    plan = [(0, A1, A1), (1, B1, B1), (0, None, A1), (0, A2, A2), (0, None, A2), (0, None, A2)]
    reqs = [{"key": k, "A": A, "b": rng.standard_normal(n), "Aeff": Ae} for k, A, Ae in plan]
    srv = serving.Server(ctx, workers=1, precision="fp32", hbm_budget_bytes=one + one // 2)
    done, _ = serving.run_stream(srv, reqs, rate_hz=0.0, resubmit_missing=True, timeout_s=120)
    srv.close()
    assert len(done) == len(reqs)
    for d in done:
        assert d["status"] == 0, d
        r = reqs[d["tag"]]
        assert oracle_mod.backward_error(r["Aeff"], d["x"], r["b"]) <= 10 * n * EPS64, d["tag"]
