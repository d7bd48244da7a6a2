"""Query-row sharding of the brute kNN across ranks (gloo, world_size 2, CPU).

Rows are independent: each rank computes its contiguous block of query rows
against all points and one all-gather rebuilds the full neighbour table, which
must equal the single-process result. This is the only exchange the stage has
(the assembly then runs on the gathered table)."""
import os
import socket

import numpy as np
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, out_path):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle import oracle
    from tapkee_gb300 import datasets
    from tapkee_gb300.sharding import shard_rows

    X = datasets.swiss_roll(600, seed=4)
    k = 8
    lo, hi = shard_rows(len(X), rank, world)
    local = oracle.knn_brute_rows(X, k, np.arange(lo, hi), nthreads=1)
    # pad to the largest shard for the all-gather
    cap = shard_rows(len(X), 0, world)[1]
    buf = torch.full((cap, k), -1, dtype=torch.int32)
    buf[: hi - lo] = torch.from_numpy(local)
    parts = [torch.empty_like(buf) for _ in range(world)]
    dist.all_gather(parts, buf)
    if rank == 0:
        rows = []
        for r in range(world):
            a, b = shard_rows(len(X), r, world)
            rows.append(parts[r][: b - a].numpy())
        np.save(out_path, np.concatenate(rows))
    dist.barrier()
    dist.destroy_process_group()


def test_row_sharded_knn_equals_single_rank(tmp_path):
    out = str(tmp_path / "gathered.npy")
    mp.spawn(_rank_main, args=(2, _free_port(), out), nprocs=2, join=True)
    from oracle import oracle
    from tapkee_gb300 import datasets
    X = datasets.swiss_roll(600, seed=4)
    ref, _, _ = oracle.knn_brute(X, 8, nthreads=1)
    got = np.load(out)
    assert got.shape == ref.shape
    assert all(set(a) == set(b) for a, b in zip(got, ref))
