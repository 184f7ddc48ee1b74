"""Velocity Verlet on the GPU (gb_batch_md_*, verlet.f90:100-235) against the
same integrator on the host with the oracle's forces; CUDA-graph steps equal
eager steps bitwise; total energy is conserved."""

import numpy as np
import pytest

import oracle

from helpers import TERSOFF, rattled_diamond

pytestmark = pytest.mark.gpu

M_SI = 28.0855  # amu; with eV and A the time unit is 10.18 fs
DT = 0.1


def _system(seed):
    structs = [rattled_diamond("Si", 5.431, (2, 2, 2), 0.1, seed),
               rattled_diamond("Si", 5.431, (2, 2, 3), 0.1, seed + 1)]
    n = sum(len(s) for s in structs)
    rng = np.random.default_rng(seed + 2)
    v = rng.normal(0.0, 0.02, (n, 3))  # ~ a few hundred K
    m = np.full(n, M_SI)
    return structs, v, m


def _cpu_verlet(s, v, m, nsteps):
    s = s.copy()
    v = v.copy()
    f = oracle.bop("tersoff", TERSOFF, s, per_at=False)["f"]
    for _ in range(nsteps):
        v = v + 0.5 * f / m[:, None] * DT
        s.positions = s.positions + v * DT
        f = oracle.bop("tersoff", TERSOFF, s, per_at=False)["f"]
        v = v + 0.5 * f / m[:, None] * DT
    return s.positions, v, f


def test_md_matches_host_verlet(gpu):
    from atomistica_gb300 import native
    structs, v, m = _system(61)
    b = native.Batch(structs)
    b.md_set_state(v, m)
    pot = native.Tersoff()
    b.md_run(pot, DT, 20)
    r, vg, f = b.md_get_state()
    for q, s in enumerate(structs):
        sl = slice(b.offsets[q], b.offsets[q + 1])
        rr, vv, ff = _cpu_verlet(s, v[sl], m[sl], 20)
        assert np.max(np.abs(r[sl] - rr)) < 1e-9
        assert np.max(np.abs(vg[sl] - vv)) < 1e-9
        assert np.max(np.abs(f[sl] - ff)) < 1e-8


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_md_graph_equals_eager(gpu, prec):
    from atomistica_gb300 import native
    structs, v, m = _system(62)
    pot = native.Tersoff(precision=prec)
    out = []
    for graph in (False, True):
        b = native.Batch(structs)
        b.set_options(graph=graph)
        b.md_set_state(v, m)
        e, w = b.md_run(pot, DT, 30)
        info = b.last_info()
        if graph:
            assert info["replayed"] and info["graph_kernels"] > 0
        out.append((e, w) + b.md_get_state())
    for x, y in zip(out[0], out[1]):
        assert np.array_equal(x, y)


def test_md_energy_conservation(gpu):
    from atomistica_gb300 import native
    structs, v, m = _system(63)
    b = native.Batch(structs)
    b.set_options(graph=True)
    b.md_set_state(v, m)
    pot = native.Tersoff()
    dt = DT / 2  # Verlet's energy error scales as dt^2
    e0, _ = b.md_run(pot, dt, 1)
    _, v0, _ = b.md_get_state()
    k0 = 0.5 * np.sum(m[:, None] * v0 ** 2)
    e1, _ = b.md_run(pot, dt, 800)
    _, v1, _ = b.md_get_state()
    k1 = 0.5 * np.sum(m[:, None] * v1 ** 2)
    n = len(m)
    drift = abs((e1.sum() + k1) - (e0.sum() + k0)) / n
    assert drift < 1e-4, drift
    assert abs(k1 - k0) / n > 1e-6  # the system did move


def _md_states(structs, v, m, prec, graph, plan):
    from atomistica_gb300 import native
    b = native.Batch(structs)
    b.set_options(graph=graph)
    b.md_set_state(v, m)
    pot = native.Tersoff(precision=prec)
    for item in plan:
        if isinstance(item, int):
            e, w = b.md_run(pot, DT, item)
        else:
            b.set_positions(item)
    return (e, w) + b.md_get_state()


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_md_overflow_falls_back(gpu, prec):
    # A captured step that outgrows the captured list capacity leaves the
    # second half kick undone and is redone eagerly.  Two ways to get there:
    # positions compressed between runs (the first replayed step overflows),
    # and a cluster driven inward so that its coordination grows during the
    # run.  Either way the trajectory equals the eager one bitwise.
    structs, v, m = _system(64)
    r0 = np.concatenate([s.positions for s in structs])
    dense = r0.copy()
    n0 = len(structs[0])
    c = dense[:n0].mean(axis=0)
    dense[:n0] = c + 0.75 * (dense[:n0] - c)
    plan = [12, dense, 21]
    a = _md_states(structs, v, m, prec, False, plan)
    g = _md_states(structs, v, m, prec, True, plan)
    for x, y in zip(a, g):
        assert np.array_equal(x, y)

    cl = rattled_diamond("Si", 5.431 * 1.15, (2, 2, 2), 0.05, 65)
    cl.cell = cl.cell * 2.0  # a cluster in vacuum
    cl.positions = cl.positions + 0.25 * np.diag(cl.cell)
    centre = cl.positions.mean(axis=0)
    vin = -0.35 * (cl.positions - centre)
    mc = np.full(len(cl), M_SI)
    a = _md_states([cl], vin, mc, prec, False, [40])
    g = _md_states([cl], vin, mc, prec, True, [40])
    for x, y in zip(a, g):
        assert np.array_equal(x, y)
    assert np.all(np.isfinite(g[2]))
