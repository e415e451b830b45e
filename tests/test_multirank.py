"""Two-rank (gloo, CPU) test of spectrum sharding and the result gather.

Each rank searches its shard with the CPU oracle standing in for its GPU;
rank 0's gathered results must equal one single-process search.
"""
import os
import pickle
import socket
import tempfile

import numpy as np
import pytest
import torch.multiprocessing as mp

from hicops_gb300.shard import shard_bounds


def test_shard_bounds_cover_batch():
    for n in (0, 1, 7, 100, 101):
        for w in (1, 2, 3, 8):
            b = [shard_bounds(n, r, w) for r in range(w)]
            assert b[0][0] == 0 and b[-1][1] == n
            assert all(b[i][1] == b[i + 1][0] for i in range(w - 1))
            assert max(e - s for s, e in b) - min(e - s for s, e in b) <= 1


class _OracleRank:
    def __init__(self, db, p):
        from oracle import oracle as O
        self.oi = O.OracleIndex(db, p)

    def query(self, q, want_hist=False):
        return self.oi.query(q, tie_rule=1, threads=2, want_hist=want_hist)


def _worker(rank, world, port, path):
    import torch.distributed as dist
    from hicops_gb300 import synthetic as S
    from hicops_gb300.shard import sharded_query
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    p = S.SearchParams(maxz=2, dF=2, dM=100.0, threads=2)
    db = S.make_database(600, 41, p)
    q = S.make_queries(db, 61, 42, p)
    r, h = sharded_query(_OracleRank(db, p), q, dist, want_hist=True)
    if rank == 0:
        with open(path, "wb") as f:
            pickle.dump((r, h), f)
    dist.barrier()
    dist.destroy_process_group()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def test_two_rank_gather_equals_single_process():
    from hicops_gb300 import synthetic as S
    path = os.path.join(tempfile.mkdtemp(), "r.pkl")
    mp.start_processes(_worker, args=(2, _free_port(), path), nprocs=2, start_method="spawn")
    with open(path, "rb") as f:
        r, h = pickle.load(f)
    p = S.SearchParams(maxz=2, dF=2, dM=100.0, threads=2)
    db = S.make_database(600, 41, p)
    q = S.make_queries(db, 61, 42, p)
    r1, h1 = _OracleRank(db, p).query(q, want_hist=True)
    assert np.array_equal(r, r1) and np.array_equal(h, h1)
