"""CUDA-graph replay of whole single-structure evaluations
(gb_potential_set_graph): replays equal the eager path bit for bit, follow new
positions, fall back to the eager path when the captured list capacity or
tile plan is exceeded (outputs untouched by the failed replay), keep the
accumulate / set semantics of the force argument, and are not used when
per-atom outputs or a mask are requested."""

import numpy as np
import pytest

from atomistica_gb300 import structures as S

from helpers import rattled_diamond

pytestmark = pytest.mark.gpu


def _setup(s, cls, precision, graph):
    from atomistica_gb300 import native
    p = native.from_atoms(s)
    nl = native.Neighbors(100)
    pot = getattr(native, cls)(precision=precision)
    pot.bind_to(p, nl)
    if graph:
        pot.set_graph(True)
    return p, nl, pot


def _eval(p, nl, pot, r, f):
    """set_positions + energy_and_forces accumulating into the device array f."""
    f.zero_()
    p.set_positions(r)
    e, _, w = pot.energy_and_forces(p, nl, forces=f)
    return e, f.cpu().numpy().copy(), np.array(w)


@pytest.mark.parametrize("cls,precision", [("Tersoff", "mixed"), ("Tersoff", "fp64"),
                                           ("Kumagai", "fp64"), ("Brenner", "mixed")])
def test_replay_equals_eager(gpu, cls, precision):
    import torch
    s = S.tersoff_si_4096(seed=11) if cls != "Brenner" else \
        rattled_diamond("Si", 5.431, (4, 4, 4), 0.15, 12)
    if cls == "Kumagai":
        s = rattled_diamond("Si", 5.429, (4, 4, 4), 0.2, 13)
    dev = torch.device("cuda", 0)
    r0 = torch.tensor(s.positions, dtype=torch.float64, device=dev)
    f = torch.zeros((len(s), 3), dtype=torch.float64, device=dev)
    eager = _setup(s, cls, precision, False)
    graph = _setup(s, cls, precision, True)
    rng = np.random.default_rng(14)
    replays = 0
    for step in range(5):
        r = r0 + torch.tensor(rng.uniform(-0.03, 0.03, (len(s), 3)), device=dev)
        e0, f0, w0 = _eval(*eager, r, f)
        e1, f1, w1 = _eval(*graph, r, f)
        replays += graph[2].last_replayed()
        assert e1 == e0 and np.array_equal(f1, f0) and np.array_equal(w1, w0), step
    assert replays >= 3  # calls after the first (eager + capture) replay


def test_overflow_falls_back_and_recaptures(gpu):
    import torch
    s = rattled_diamond("Si", 5.431, (3, 3, 3), 0.1, 15)
    dev = torch.device("cuda", 0)
    r0 = torch.tensor(s.positions, dtype=torch.float64, device=dev)
    f = torch.zeros((len(s), 3), dtype=torch.float64, device=dev)
    eager = _setup(s, "Tersoff", "mixed", False)
    graph = _setup(s, "Tersoff", "mixed", True)
    for _ in range(2):
        _eval(*graph, r0, f)
    assert graph[2].last_replayed()
    # a compressed region: more neighbours per atom than the captured capacity
    dense = r0.clone()
    c = dense[:40].mean(dim=0)
    dense[:40] = c + 0.55 * (dense[:40] - c)
    e0, f0, w0 = _eval(*eager, dense, f)
    e1, f1, w1 = _eval(*graph, dense, f)
    assert not graph[2].last_replayed()
    assert e1 == e0 and np.array_equal(f1, f0) and np.array_equal(w1, w0)
    # captured again with the new capacity: the next call replays
    e2, f2, w2 = _eval(*graph, dense, f)
    assert graph[2].last_replayed()
    assert e2 == e0 and np.array_equal(f2, f0) and np.array_equal(w2, w0)


def test_failed_replay_leaves_accumulated_forces(gpu):
    # accumulate mode: a replay that overflowed must not have added anything;
    # the eager redo adds the forces once
    import torch
    s = rattled_diamond("Si", 5.431, (3, 3, 3), 0.1, 16)
    dev = torch.device("cuda", 0)
    r0 = torch.tensor(s.positions, dtype=torch.float64, device=dev)
    graph = _setup(s, "Tersoff", "mixed", True)
    eager = _setup(s, "Tersoff", "mixed", False)
    f = torch.zeros((len(s), 3), dtype=torch.float64, device=dev)
    for _ in range(2):
        _eval(*graph, r0, f)
    dense = r0.clone()
    c = dense[:40].mean(dim=0)
    dense[:40] = c + 0.55 * (dense[:40] - c)
    _, fe, _ = _eval(*eager, dense, f)
    base = torch.ones((len(s), 3), dtype=torch.float64, device=dev)
    p, nl, pot = graph
    p.set_positions(dense)
    pot.energy_and_forces(p, nl, forces=base)
    assert not pot.last_replayed()
    assert np.array_equal(base.cpu().numpy(), fe + 1.0)


def test_host_forces_accumulate_and_set(gpu):
    s = rattled_diamond("Si", 5.431, (3, 3, 3), 0.1, 17)
    eager = _setup(s, "Tersoff", "mixed", False)
    graph = _setup(s, "Tersoff", "mixed", True)
    for accumulate in (True, False):
        fe = np.full((len(s), 3), 2.0)
        p, nl, pot = eager
        pot.energy_and_forces(p, nl, forces=fe, accumulate=accumulate)
        p, nl, pot = graph
        for _ in range(3):
            fg = np.full((len(s), 3), 2.0)
            pot.energy_and_forces(p, nl, forces=fg, accumulate=accumulate)
            assert np.array_equal(fg, fe)
        assert pot.last_replayed()


def test_per_atom_outputs_stay_eager(gpu):
    s = rattled_diamond("Si", 5.431, (3, 3, 3), 0.1, 18)
    p, nl, pot = _setup(s, "Tersoff", "fp64", True)
    for _ in range(3):
        out = pot.energy_and_forces(p, nl, epot_per_at=True)
        assert not pot.last_replayed()
    mask = np.ones(len(s), dtype=np.int32)
    for _ in range(2):
        pot.energy_and_forces(p, nl, mask=mask)
        assert not pot.last_replayed()
    assert np.isfinite(out[0])


def test_nonfinite_position_after_replays(gpu):
    from atomistica_gb300._lib import AtomisticaError
    s = rattled_diamond("Si", 5.431, (3, 3, 3), 0.1, 19)
    p, nl, pot = _setup(s, "Tersoff", "mixed", True)
    for _ in range(3):
        pot.energy_and_forces(p, nl)
    assert pot.last_replayed()
    r = s.positions.copy()
    r[5, 1] = np.nan
    p.set_positions(r)
    with pytest.raises(AtomisticaError, match="Non-finite particle position"):
        pot.energy_and_forces(p, nl)


def test_eam_replay_equals_eager(gpu, tmp_path):
    import torch
    from atomistica_gb300 import io as gio
    from atomistica_gb300 import native
    fn = gio.analytic_alloy_setfl(str(tmp_path / "a.setfl"), ["Cu", "Ag"], seed=3)
    s = S.fcc("Cu", 3.7, (5, 5, 5))
    rng = np.random.default_rng(20)
    s.numbers = np.array(rng.choice([29, 47], len(s)), dtype=np.int32)
    dev = torch.device("cuda", 0)
    r0 = torch.tensor(s.positions, dtype=torch.float64, device=dev)
    f = torch.zeros((len(s), 3), dtype=torch.float64, device=dev)
    runs = []
    for graph in (False, True):
        p = native.from_atoms(s)
        nl = native.Neighbors(100)
        pot = native.TabulatedAlloyEAM(fn)
        pot.bind_to(p, nl)
        if graph:
            pot.set_graph(True)
        runs.append((p, nl, pot))
    replays = 0
    for step in range(4):
        r = r0 + torch.tensor(rng.normal(0, 0.05, (len(s), 3)), device=dev)
        e0, f0, w0 = _eval(*runs[0], r, f)
        e1, f1, w1 = _eval(*runs[1], r, f)
        replays += runs[1][2].last_replayed()
        assert e1 == e0 and np.array_equal(f1, f0) and np.array_equal(w1, w0), step
    assert replays >= 2


def test_cell_change_recaptures(gpu):
    # a new cell (strain) changes the binning baked into the graph: that call
    # runs eagerly and captures again; the results equal the eager path's
    import torch
    s = rattled_diamond("Si", 5.431, (3, 3, 3), 0.1, 21)
    dev = torch.device("cuda", 0)
    r0 = torch.tensor(s.positions, dtype=torch.float64, device=dev)
    f = torch.zeros((len(s), 3), dtype=torch.float64, device=dev)
    eager = _setup(s, "Tersoff", "mixed", False)
    graph = _setup(s, "Tersoff", "mixed", True)
    for _ in range(2):
        _eval(*graph, r0, f)
    assert graph[2].last_replayed()
    strain = np.diag([1.01, 0.99, 1.02])
    cell = s.cell @ strain
    r1 = torch.tensor(s.positions @ strain, dtype=torch.float64, device=dev)
    for p, _, _ in (eager, graph):
        p.set_cell(cell, True)
    for call in range(3):
        e0, f0, w0 = _eval(*eager, r1, f)
        e1, f1, w1 = _eval(*graph, r1, f)
        assert graph[2].last_replayed() == (call > 0)
        assert e1 == e0 and np.array_equal(f1, f0) and np.array_equal(w1, w0), call


def test_new_force_array_every_call_stays_eager(gpu):
    # a new device force array every call never matches the captured one:
    # after a few captures the potential stops capturing; results stay exact
    import torch
    s = rattled_diamond("Si", 5.431, (3, 3, 3), 0.1, 22)
    dev = torch.device("cuda", 0)
    p, nl, pot = _setup(s, "Tersoff", "mixed", True)
    pe, nle, pote = _setup(s, "Tersoff", "mixed", False)
    fe = torch.zeros((len(s), 3), dtype=torch.float64, device=dev)
    e0, _, _ = pote.energy_and_forces(pe, nle, forces=fe)
    for _ in range(6):
        f = torch.zeros((len(s), 3), dtype=torch.float64, device=dev)
        e, _, _ = pot.energy_and_forces(p, nl, forces=f)
        assert not pot.last_replayed()
        assert e == e0 and torch.equal(f, fe)


@pytest.mark.parametrize("graph", [False, True])
def test_pinned_host_forces_written_directly(gpu, graph):
    # forces written (not accumulated) into page-locked host memory go there
    # straight from the gather; equal to the device-array result, also after
    # the array held other values
    import torch
    s = rattled_diamond("Si", 5.431, (3, 3, 3), 0.1, 23)
    dev = torch.device("cuda", 0)
    pe, nle, pote = _setup(s, "Tersoff", "mixed", False)
    fe = torch.zeros((len(s), 3), dtype=torch.float64, device=dev)
    e0, _, w0 = pote.energy_and_forces(pe, nle, forces=fe)
    p, nl, pot = _setup(s, "Tersoff", "mixed", graph)
    fh = torch.full((len(s), 3), 7.0, dtype=torch.float64).pin_memory()
    fn = fh.numpy()
    for call in range(3):
        fn[...] = 7.0
        e, _, w = pot.energy_and_forces(p, nl, forces=fn, accumulate=False)
        assert e == e0 and np.array_equal(fn, fe.cpu().numpy()), call
        assert np.array_equal(np.asarray(w), np.asarray(w0))
    assert pot.last_replayed() == graph


def test_eam_forces_written_for_skipped_atoms(gpu, tmp_path):
    # store mode: atoms of elements the potential skips get zero forces even
    # when the array held other values
    import torch
    from atomistica_gb300 import io as gio
    from atomistica_gb300 import native
    fn_ = gio.analytic_alloy_setfl(str(tmp_path / "a.setfl"), ["Cu", "Ag"], seed=4)
    s = S.fcc("Cu", 3.7, (3, 3, 3))
    s.numbers[::5] = 14  # not in the file
    p = native.from_atoms(s)
    nl = native.Neighbors(100)
    pot = native.TabulatedAlloyEAM(fn_)
    pot.bind_to(p, nl)
    dev = torch.device("cuda", 0)
    f0 = torch.zeros((len(s), 3), dtype=torch.float64, device=dev)
    pot.energy_and_forces(p, nl, forces=f0)
    f1 = torch.full((len(s), 3), 3.0, dtype=torch.float64, device=dev)
    pot.energy_and_forces(p, nl, forces=f1, accumulate=False)
    assert torch.equal(f1, f0)
    assert torch.all(f1[::5] == 0)
