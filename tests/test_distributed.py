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


# ---------------------------------------------------------------------------
# Sharded fitting gradient: each rank evaluates its slice of the structures;
# here on the host, the oracle's energies and forces with derivatives by
# central differences (the GPU path uses fitting.TersoffBatch).

def _fit_set():
    from atomistica_gb300 import fitting
    from atomistica_gb300 import structures as S
    structs = S.si_fit_set(5, seed=61)[:5]
    theta, m = fitting.single_element_parameters()
    rng = np.random.default_rng(62)
    theta_t = theta * (1.0 + rng.uniform(-0.02, 0.02, size=14))
    return structs, theta, theta_t, m


class OracleShard:
    """evaluate / adjoint of fitting.TersoffBatch for a list of structures,
    from the oracle (reference algorithm) with central differences."""

    def __init__(self, structs, m):
        self.structs, self.m = structs, m

    def _ef(self, theta, structs=None):
        import oracle
        from atomistica_gb300 import fitting
        p = fitting.parameter_dict(theta, self.m)
        # one thread: a fixed summation order in every process
        out = [oracle.bop("tersoff", p, s, per_at=False, nthreads=1)
               for s in (structs or self.structs)]
        return np.array([o["epot"] for o in out]), np.concatenate([o["f"] for o in out])

    def evaluate(self, theta):
        e, f = self._ef(theta)
        return e, None, f, None

    def adjoint(self, theta, v):
        e, f = self._ef(theta)
        ns = len(self.structs)
        off = np.concatenate([[0], np.cumsum([len(s) for s in self.structs])])
        v = np.zeros_like(f) if v is None else v
        g, gd = np.zeros((ns, 14)), np.zeros((ns, 14))
        for k in range(14):
            h = 1e-6 * abs(theta[k]) if theta[k] != 0 else 1e-6
            u = np.zeros(14)
            u[k] = h
            ep, fp = self._ef(theta + u)
            em, fm = self._ef(theta - u)
            g[:, k] = (ep - em) / (2 * h)
            vf = [np.sum(v[off[q]:off[q + 1]] * (fp - fm)[off[q]:off[q + 1]]) / (2 * h)
                  for q in range(ns)]
            gd[:, k] = -np.array(vf)  # D_v dE/dtheta = -d(v . F)/dtheta
        eps = 1e-5
        moved = []
        for sg in (1, -1):
            ss = []
            for q, s in enumerate(self.structs):
                t = s.copy()
                t.positions = s.positions + sg * eps * v[off[q]:off[q + 1]]
                ss.append(t)
            moved.append(self._ef(theta, ss)[1])
        hv = (moved[0] - moved[1]) / (2 * eps)
        return e, f, hv, g, gd


def _fit_worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from atomistica_gb300 import fitting
        structs, theta, theta_t, m = _fit_set()
        lo, hi = D.shard_range(len(structs), rank, world)
        mine = structs[lo:hi]
        et, _, ft, _ = OracleShard(mine, m).evaluate(theta_t)
        loss, g, gp = fitting.sharded_loss_and_gradient(
            theta, OracleShard(mine, m), [len(s) for s in mine], et, ft)
        out[rank] = (loss, g, gp, lo, hi)
    finally:
        dist.destroy_process_group()


def test_sharded_fitting_gradient_two_ranks():
    from atomistica_gb300 import fitting
    world = 2
    port = _free_port()
    out = mp.Manager().dict()
    mp.spawn(_fit_worker, args=(world, port, out), nprocs=world, join=True)
    structs, theta, theta_t, m = _fit_set()
    sh = OracleShard(structs, m)
    et, _, ft, _ = sh.evaluate(theta_t)
    loss, g, gp = fitting.sharded_loss_and_gradient(theta, sh, [len(s) for s in structs],
                                                    et, ft)
    assert np.max(np.abs(g)) > 0
    gps = []
    for rank in range(world):
        l_r, g_r, gp_r, lo, hi = out[rank]
        assert l_r == pytest.approx(loss, rel=1e-13)
        assert np.all(np.abs(g_r - g) <= 1e-12 * np.abs(g) + 1e-300)
        gps.append(gp_r)
    assert np.max(np.abs(np.concatenate(gps) - gp)) <= 1e-12 * np.max(np.abs(gp))
    # the serial result is the loss's own derivative (central differences)
    k = 0
    h = 1e-6 * theta[k]

    def lossv(th):
        e, _, f, _ = sh.evaluate(th)
        nat = np.array([len(s) for s in structs], float)
        return np.mean(((e - et) / nat) ** 2) + 0.1 * np.mean(np.sum((f - ft) ** 2, axis=1))
    u = np.zeros(14)
    u[k] = h
    fd = (lossv(theta + u) - lossv(theta - u)) / (2 * h)
    assert abs(g[k] - fd) <= 1e-5 * abs(fd)
