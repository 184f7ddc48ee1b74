"""Multi-process host logic with the gloo backend on CPU (world size 2):
replica timing and rate, structure sharding and the one collective of the
sharded fitting loss (a sum over ranks), against the serial results."""

import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from atomistica_gb300 import distributed as D  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ws, r, _ = D.dist_info()
        assert (ws, r) == (world, rank)
        # replicas: the slowest rank's time, the whole-job rate
        t = 1.0 + rank
        tmax = D.max_over_ranks(t)
        rate = D.replica_rate(1000, tmax, ws)
        # sharded fitting loss: per-structure synthetic results, seeded
        rng = np.random.default_rng(0)
        nat = rng.integers(8, 20, size=11)
        e, et = rng.normal(size=11), rng.normal(size=11)
        off = np.concatenate([[0], np.cumsum(nat)])
        f, ft = rng.normal(size=(off[-1], 3)), rng.normal(size=(off[-1], 3))
        lo, hi = D.shard_range(11, rank, ws)
        sums = D.sharded_fitting_sums(e[lo:hi], et[lo:hi], nat[lo:hi],
                                      f[off[lo]:off[hi]], ft[off[lo]:off[hi]])
        tot = D.allreduce_sum(sums)
        loss = tot[0] / tot[2] + 0.1 * tot[1] / tot[3]
        out[rank] = (tmax, rate, loss, lo, hi)
    finally:
        dist.destroy_process_group()


def test_two_rank_host_logic():
    world = 2
    port = _free_port()
    out = mp.Manager().dict()
    mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
    rng = np.random.default_rng(0)
    nat = rng.integers(8, 20, size=11)
    e, et = rng.normal(size=11), rng.normal(size=11)
    off = np.concatenate([[0], np.cumsum(nat)])
    f, ft = rng.normal(size=(off[-1], 3)), rng.normal(size=(off[-1], 3))
    serial = np.mean(((e - et) / nat) ** 2) + 0.1 * np.mean(np.sum((f - ft) ** 2, axis=1))
    for rank in range(world):
        tmax, rate, loss, lo, hi = out[rank]
        assert tmax == 2.0
        assert rate == pytest.approx(2 * 1000 / 2.0)
        assert loss == pytest.approx(serial, rel=1e-14)
    # the shards tile the structures
    assert out[0][3] == 0 and out[0][4] == out[1][3] and out[1][4] == 11


def test_shard_range_single_process():
    for n in (0, 1, 7, 2048):
        for w in (1, 2, 3, 8):
            spans = [D.shard_range(n, r, w) for r in range(w)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
            sizes = [hi - lo for lo, hi in spans]
            assert max(sizes) - min(sizes) <= 1
    assert D.max_over_ranks(3.5) == 3.5
    assert np.array_equal(D.allreduce_sum([1.0, 2.0]), [1.0, 2.0])
