"""The multi-rank reduction of bench.py (catana_gb300.shards) on CPU: two gloo
ranks each decompose half of a catalog with the oracle, combine with one
all-reduce, and match the oracle on the whole catalog."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, weighted, q):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    sys.path.insert(0, os.path.join(root, "tests"))
    # the shard helper has no dependency on the CUDA library
    import importlib.util
    spec = importlib.util.spec_from_file_location("shards", os.path.join(root, "catana_gb300", "shards.py"))
    shards = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(shards)
    from oracle import oracle as O
    from conftest import uniform_ball
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    pts = uniform_ball(700, 300.0, seed=8)
    w = np.random.default_rng(8).uniform(0.5, 1.5, 700) if weighted else None
    cut = [0, 300, 700]
    sl = slice(cut[rank], cut[rank + 1])
    k, c, f = O.sfb_raw(pts[sl], 6, 5, 300.0, interpolated=False, weights=None if w is None else w[sl], nthreads=1)
    flat = np.concatenate([x.ravel() for x in f])
    ft = torch.from_numpy(np.stack([flat.real, flat.imag], axis=1).ravel().copy())
    wl = (cut[rank + 1] - cut[rank]) if w is None else float(w[sl].sum())
    ft, total = shards.combine_flmn(ft, wl, dist.all_reduce)
    cl = shards.cln_from_flmn(ft, 6, 5)
    if rank == 0:
        k0, c0, f0 = O.sfb_raw(pts, 6, 5, 300.0, interpolated=False, weights=w, nthreads=1)
        fz = ft.view(-1, 2).numpy()
        fz = fz[:, 0] + 1j * fz[:, 1]
        ref = np.concatenate([x.ravel() for x in f0])
        q.put((float(np.abs(fz - ref).max() / np.abs(ref).max()), float(np.max(np.abs(cl.numpy() - c0) / c0))))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("weighted", [False, True])
def test_two_rank_reduction(weighted):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, weighted, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    ef, ec = q.get(timeout=5)
    assert ef < 1e-12 and ec < 1e-11
