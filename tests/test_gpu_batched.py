"""Batched uneven LU (one persistent kernel per size bucket in one CUDA graph)
against the oracle's per-system getrf + getrs."""
import ctypes

import numpy as np
import pytest

from conftest import EPS64

pytestmark = pytest.mark.gpu


class Batch:
    def __init__(self, ctx, sizes, precision):
        self.ctx, self.lib = ctx, ctx.lib
        self.sizes = np.ascontiguousarray(sizes, dtype=np.int64)
        h = ctypes.c_void_p()
        st = self.lib.gblu_batch_create(ctx.handle, len(self.sizes), self.sizes.ctypes.data,
                                        precision, ctypes.byref(h))
        assert st == 0, self.lib.gblu_last_error(ctx.handle)
        self.h = h

    def schedule(self, upper, threads, panel):
        u = np.array(upper, dtype=np.int32)
        t = np.array(threads, dtype=np.int32)
        p = np.array(panel, dtype=np.int32)
        return self.lib.gblu_batch_schedule(self.ctx.handle, self.h, len(u), u.ctypes.data,
                                            t.ctypes.data, p.ctypes.data, None)

    def solve(self, A, b):
        X = np.array(b, dtype=np.float64, copy=True)
        info = np.zeros(len(self.sizes), dtype=np.int64)
        st = self.lib.gblu_batch_solve(self.ctx.handle, self.h, np.ascontiguousarray(A).ctypes.data,
                                       X.ctypes.data, 0, info.ctypes.data)
        assert st == 0, self.lib.gblu_last_error(self.ctx.handle)
        return X, info

    def close(self):
        self.lib.gblu_batch_destroy(self.ctx.handle, self.h)


def test_fp64_batch_bit_exact(ctx, oracle_mod, pkg):
    sizes, A, b, _ = pkg.workloads.batch(300, seed=1)
    bt = Batch(ctx, sizes, 0)
    X, info = bt.solve(A, b)
    Aref, Xref, info_ref = oracle_mod.gesv_batched(sizes, A, b)
    assert np.array_equal(info, info_ref)
    assert np.array_equal(X, Xref)
    bt.close()


@pytest.mark.parametrize("sched", [([256], [256], [16]), ([32, 96, 256], [128, 256, 512], [8, 16, 16]),
                                   ([64, 128, 256], [128, 128, 256], [16, 8, 8]),
                                   ([48, 256], [64, 64], [8, 8])])
def test_fp64_batch_schedules(ctx, oracle_mod, pkg, sched):
    sizes, A, b, _ = pkg.workloads.batch(200, seed=2)
    bt = Batch(ctx, sizes, 0)
    assert bt.schedule(*sched) == 0
    X, info = bt.solve(A, b)
    _, Xref, info_ref = oracle_mod.gesv_batched(sizes, A, b)
    assert np.array_equal(X, Xref)
    bt.close()


def test_fp64_batch_edge_sizes(ctx, oracle_mod, pkg):
    rng = np.random.default_rng(3)
    sizes = np.array([1, 2, 7, 8, 9, 15, 16, 17, 31, 32, 33, 64, 65, 127, 128, 129, 255, 256, 256, 1],
                     dtype=np.int64)
    A = np.concatenate([rng.standard_normal(n * n) for n in sizes])
    b = rng.standard_normal(int(sizes.sum()))
    bt = Batch(ctx, sizes, 0)
    X, info = bt.solve(A, b)
    _, Xref, info_ref = oracle_mod.gesv_batched(sizes, A, b)
    assert np.array_equal(info, info_ref)
    assert np.array_equal(X, Xref)
    bt.close()


def test_batch_singular_system_reported(ctx, oracle_mod, pkg):
    sizes, A, b, _ = pkg.workloads.batch(20, seed=4)
    a_off, _ = pkg.workloads.offsets(sizes)
    k = 5
    n = int(sizes[k])
    Ak = A[a_off[k]:a_off[k] + n * n].reshape(n, n, order="F")
    Ak[:, 0] = 0.0
    A[a_off[k]:a_off[k] + n * n] = Ak.ravel(order="F")
    for prec in (0, 1):
        bt = Batch(ctx, sizes, prec)
        X, info = bt.solve(A, b)
        assert info[k] == 1
        assert all(info[i] == 0 for i in range(len(sizes)) if i != k)
        bt.close()


def test_mixed_batch_reaches_fp64(ctx, oracle_mod, pkg):
    sizes, A, b, _ = pkg.workloads.batch(400, seed=5)
    bt = Batch(ctx, sizes, 1)
    X, info = bt.solve(A, b)
    assert (info == 0).all()
    a_off, b_off = pkg.workloads.offsets(sizes)
    worst = 0.0
    for i, n in enumerate(sizes):
        n = int(n)
        Ai = A[a_off[i]:a_off[i] + n * n].reshape(n, n, order="F")
        be = oracle_mod.backward_error(Ai, X[b_off[i]:b_off[i] + n], b[b_off[i]:b_off[i] + n])
        worst = max(worst, be / (n * EPS64))
    assert worst <= 10.0, worst
    bt.close()


def test_mixed_batch_result_independent_of_neighbours(ctx, pkg):
    """A system's result is the same alone and inside a batch (fixed-order
    arithmetic, one CTA per system)."""
    sizes, A, b, _ = pkg.workloads.batch(60, seed=6)
    a_off, b_off = pkg.workloads.offsets(sizes)
    bt = Batch(ctx, sizes, 1)
    X, _ = bt.solve(A, b)
    bt.close()
    for i in (0, 17, 59):
        n = int(sizes[i])
        one = Batch(ctx, np.array([n]), 1)
        Xi, _ = one.solve(A[a_off[i]:a_off[i] + n * n], b[b_off[i]:b_off[i] + n])
        assert np.array_equal(Xi, X[b_off[i]:b_off[i] + n])
        one.close()


def test_batch_rejects_oversize(ctx):
    h = ctypes.c_void_p()
    sizes = np.array([10, 257], dtype=np.int64)
    st = ctx.lib.gblu_batch_create(ctx.handle, 2, sizes.ctypes.data, 0, ctypes.byref(h))
    assert st == 7


def test_autotuner_finds_valid_schedule(ctx, oracle_mod, pkg, tmp_path, monkeypatch):
    monkeypatch.setenv("GBLU_AUTOTUNE_FILE", str(tmp_path / "autotune.json"))
    from importlib import import_module
    at = import_module(pkg.__name__ + ".autotune")
    sizes, A, b, _ = pkg.workloads.batch(300, seed=8)
    sched = at.tune(ctx, sizes, "fp64", A=A, b=b, budget_s=5.0)
    assert sched["upper"][-1] == 256 and sched["ms"] > 0
    assert (tmp_path / "autotune.json").exists()
    again = at.tune(ctx, sizes, "fp64", A=A, b=b)  # served from the cache
    assert again["signature"] == sched["signature"]
    bt = Batch(ctx, sizes, 0)
    at.apply(ctx, bt.h, sched)
    X, info = bt.solve(A, b)
    _, Xref, _ = oracle_mod.gesv_batched(sizes, A, b)
    assert np.array_equal(X, Xref)
    bt.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_full_batch_every_system_within_bound(ctx, oracle_mod, pkg, precision):
    """The bench's whole workload (20,000 systems, n uniform in [8, 256]):
    every system's backward error within 10 n eps64, FP64 and FP32 + IR (the
    bench itself samples 200 of them)."""
    sizes, A, b, _ = pkg.workloads.batch(20000, seed=0)
    bt = Batch(ctx, sizes, precision)
    X, info = bt.solve(A, b)
    assert (info == 0).all()
    a_off, b_off = pkg.workloads.offsets(sizes)
    worst = 0.0
    for i, n in enumerate(sizes):
        n = int(n)
        Ai = A[a_off[i]:a_off[i] + n * n].reshape(n, n, order="F")
        x = X[b_off[i]:b_off[i] + n]
        bi = b[b_off[i]:b_off[i] + n]
        r = bi - Ai @ x
        be = np.abs(r).max() / (np.abs(Ai).sum(axis=1).max() * np.abs(x).max() + np.abs(bi).max())
        worst = max(worst, be / (n * EPS64))
    assert worst <= 10.0, worst
    bt.close()
