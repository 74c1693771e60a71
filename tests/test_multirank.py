"""Multi-rank host logic on CPU (gloo, world size 2): ring sharding balanced by
bead count and the one gather of per-lambda partial sums (through the
caller's communicator) reproduce the single-process reduction and assembly."""
import os
import socket

import numpy as np

import sharding


def test_shard_rings_covers_and_balances():
    P = np.random.RandomState(11).choice([64, 128, 256, 512], size=4096)
    for ws in (1, 2, 3, 4, 8):
        blocks = [sharding.shard_rings(P, ws, r) for r in range(ws)]
        assert blocks[0][0] == 0 and blocks[-1][1] == len(P)
        for (a, b), (c, d) in zip(blocks, blocks[1:]):
            assert b == c
        loads = [P[a:b].sum() for a, b in blocks]
        assert max(loads) - min(loads) <= 2 * 512


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, ws, port, integrands, lam, nl, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    a, b = sharding.shard_rings(np.ones(len(lam)), ws, rank)
    part = sharding.lambda_partials(integrands[a:b], lam[a:b], nl)

    def allgather(arr):  # the caller's communicator (here a gloo group)
        out = [None] * ws
        dist.all_gather_object(out, arr)
        return out

    tot = sharding.combine_partials(part, allgather)
    q.put((rank, tot))
    dist.destroy_process_group()


def test_two_rank_gloo_reduction_matches_single_process():
    import multiprocessing as mp
    rs = np.random.RandomState(3)
    nl, nrep = 5, 37
    lam = np.repeat(np.arange(nl), nrep)
    integrands = rs.randn(nl * nrep) * 3 + lam
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, integrands, lam, nl, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    ref = sharding.lambda_partials(integrands, lam, nl)
    for _, tot in res:
        np.testing.assert_allclose(tot, ref, rtol=1e-13)
    np.testing.assert_array_equal(res[0][1], res[1][1])  # every rank gets the same bits
    mean, var = sharding.mean_var(res[0][1])
    m2 = integrands.reshape(nl, nrep).mean(1)
    np.testing.assert_allclose(mean, m2, rtol=1e-13)
    np.testing.assert_allclose(var, (integrands.reshape(nl, nrep) ** 2).mean(1) - m2 ** 2, rtol=1e-10)
