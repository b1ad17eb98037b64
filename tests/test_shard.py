"""Row-band sharding (fringe_gb300/shard.py) on two CPU ranks over gloo: each
rank phase-links its band from its own rows (the oracle stands in for the
GPU), the bands are gathered, and the result equals the whole scene."""
import os
import socket

import numpy as np
import pytest

from fringe_gb300 import synth
from fringe_gb300.shard import row_bands


def test_bands_cover_rows_once_with_aprons():
    for rows, world, ny in [(2048, 4, 5), (45, 2, 3), (7, 3, 2), (100, 8, 10)]:
        bands = row_bands(rows, world, ny)
        covered = np.zeros(rows, int)
        for b in bands:
            covered[b.r0:b.r1] += 1
            if b.r1 > b.r0:
                assert b.s0 <= max(0, b.r0 - ny) and b.s0 % 8 == 0
                assert b.s1 >= min(rows, b.r1 + ny)
        assert (covered == 1).all()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, q):
    import torch
    import torch.distributed as dist
    import oracle
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    stack, nmap = synth.scene("voronoi", 37, 24, 10, 3, 4, seed=77)
    band = row_bands(37, world, 3)[rank]
    o = oracle.run(stack[:, band.s0:band.s1], nmap[band.s0:band.s1], 3, 4, method="MLE",
                   rows=band.local_rows)
    lr0, lr1 = band.local_rows
    mine = torch.from_numpy(np.ascontiguousarray(o["tcorr"][lr0:lr1]))
    ph = torch.from_numpy(np.ascontiguousarray(o["phase"][:, lr0:lr1]).view(np.float32))
    sizes = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(sizes, torch.tensor([mine.shape[0]]))
    n = int(max(s.item() for s in sizes))
    pad_t = torch.zeros((n, 24))
    pad_t[:mine.shape[0]] = mine
    pad_p = torch.zeros((10, n, 48))
    pad_p[:, :mine.shape[0]] = ph
    gt = [torch.zeros_like(pad_t) for _ in range(world)]
    gp = [torch.zeros_like(pad_p) for _ in range(world)]
    dist.all_gather(gt, pad_t)
    dist.all_gather(gp, pad_p)
    if rank == 0:
        tc = np.concatenate([g[:int(s.item())].numpy() for g, s in zip(gt, sizes)])
        phs = np.concatenate([g[:, :int(s.item())].numpy() for g, s in zip(gp, sizes)], axis=1)
        whole = oracle.run(stack, nmap, 3, 4, method="MLE")
        ok = (np.array_equal(tc, whole["tcorr"], equal_nan=True) and
              np.array_equal(phs.view(np.complex64), whole["phase"]))
        q.put(bool(ok))
    dist.destroy_process_group()


def test_two_rank_gloo_bands_equal_whole_scene():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    assert q.get(timeout=10)
