"""The sharded batched solve with the library's batched kernels on each
rank: world size 2 over gloo, each rank on GPU (rank % device count).  The
ranks' kernels never wait on one another (each solves its own shard; the
gather is on the host), so two ranks may share one GPU.  Every system's
FP64 solution is bit-identical to the oracle's per-system getrf + getrs."""
import os
import socket

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import __graft_entry__ as ge
    import oracle
    pkg = ge.load_package()
    from importlib import import_module
    sh = import_module(pkg.__name__ + ".sharding")
    ctx = pkg.Context(rank % max(1, torch.cuda.device_count()))
    sizes, A, b, _ = pkg.workloads.batch(300, seed=19)
    x = sh.solve_distributed(sizes, A, b, rank, world, sh.gpu_solve_fn(ctx, "fp64"))
    _, Xref, _ = oracle.gesv_batched(sizes, A, b)
    q.put((rank, bool(np.array_equal(x, Xref))))
    ctx.close()
    dist.destroy_process_group()


def test_two_rank_batched_gpu_solve_matches_oracle():
    import multiprocessing as mp
    mctx = mp.get_context("spawn")
    q = mctx.Queue()
    port = _free_port()
    procs = [mctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=300) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert sorted(res) == [(0, True), (1, True)]

