"""CPU tests of the row-sharded product (pml_gb300.shard) with two gloo ranks on
127.0.0.1: the row partition, each rank's block, and the all-gather that
reassembles C, against the oracle's product of the whole matrices.  The
per-rank product is the oracle's here (there is no GPU in this test); on GPUs
it is the CUDA product on the rank's device."""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from conftest import ROOT


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_row_partition():
    from pml_gb300.shard import row_partition
    assert row_partition(64, 2) == [(0, 32), (32, 64)]
    assert row_partition(5, 2) == [(0, 3), (3, 5)]
    assert row_partition(10, 4) == [(0, 3), (3, 6), (6, 8), (8, 10)]
    assert row_partition(1, 3) == [(0, 1), (1, 1), (1, 1)]
    assert row_partition(0, 2) == [(0, 0), (0, 0)]
    for r in range(0, 40):
        for w in range(1, 9):
            parts = row_partition(r, w)
            assert parts[0][0] == 0 and parts[-1][1] == r
            assert all(a[1] == b[0] for a, b in zip(parts, parts[1:]))
            sizes = [b - a for a, b in parts]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        row_partition(3, 0)


def _worker(rank: int, world: int, port: int, cases, out):
    import sys
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch
    import torch.distributed as dist
    import oracle
    from pml_gb300.shard import poly_mat_mul_sharded

    def mul(X, Y, p):   # stands in for the GPU product of one rank's rows
        Xn = X.numpy().view(np.uint64)
        Yn = Y.numpy().view(np.uint64)
        return torch.from_numpy(oracle.poly_mat_mul(Xn, Yn, p).view(np.int64))

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        res = []
        for (r, k, c, l1, l2, p) in cases:
            A = torch.from_numpy(oracle.rand_poly_mat(r, k, l1, p, 1).view(np.int64))
            B = torch.from_numpy(oracle.rand_poly_mat(k, c, l2, p, 2).view(np.int64))
            C = poly_mat_mul_sharded(A, B, p, mul=mul)
            blk, (r0, r1) = poly_mat_mul_sharded(A, B, p, mul=mul, gather=False)
            res.append((C.numpy().view(np.uint64).copy(), blk.numpy().view(np.uint64).copy(), r0, r1))
        out.put((rank, res))
    finally:
        dist.destroy_process_group()


def test_two_ranks_reassemble_the_product():
    import oracle
    cases = [(6, 3, 4, 9, 7, 998244353), (5, 2, 3, 4, 6, 576460752303423619), (1, 2, 2, 3, 3, 7),
             (64, 2, 3, 5, 5, 998244353)]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, cases, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=180) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for idx, (r, k, c, l1, l2, p) in enumerate(cases):
        ref = oracle.poly_mat_mul(oracle.rand_poly_mat(r, k, l1, p, 1), oracle.rand_poly_mat(k, c, l2, p, 2), p)
        for rank in (0, 1):
            C, blk, r0, r1 = got[rank][idx]
            assert np.array_equal(C, ref)
            assert np.array_equal(blk, ref[r0:r1])
        # the two blocks cover the rows once, in order
        assert got[0][idx][2] == 0 and got[0][idx][3] == got[1][idx][2] and got[1][idx][3] == r
