"""Batched evaluation (many structures, one neighbour build and one tile
launch) against per-structure evaluations: the FP64 oracle, and the single-
structure GPU path of the same library (identical forces, energies and
virials to rounding of the tile sums)."""

import numpy as np
import pytest

import oracle
from atomistica_gb300 import structures as S

from helpers import KUMAGAI, MIXED_F_TOL, TERSOFF, gpu_bop, rattled_diamond, triclinic_si

pytestmark = pytest.mark.gpu


def _mixed_set(seed=0):
    """Uneven structures: 8-atom triclinic cells (several images of each
    atom within the cutoff), rattled diamond supercells, a non-periodic
    cluster and a slab."""
    out = [triclinic_si(8, seed=seed + 1), triclinic_si(24, seed=seed + 2),
           rattled_diamond(size=(2, 2, 2), amp=0.3, seed=seed + 3),
           triclinic_si(100, seed=seed + 4),
           rattled_diamond(size=(1, 1, 1), amp=0.2, seed=seed + 5),
           S.tersoff_si_4096(seed=seed + 6)]
    slab = rattled_diamond(size=(2, 2, 3), amp=0.2, seed=seed + 7)
    slab.pbc = np.array([True, True, False])
    out.append(slab)
    cluster = rattled_diamond(size=(2, 2, 2), amp=0.2, seed=seed + 8)
    cluster.pbc = np.array([False, False, False])
    out.append(cluster)
    return out


def _run_batch(structs, kind="tersoff", precision="fp64", params=None):
    from atomistica_gb300 import native
    b = native.Batch(structs)
    cls = native.Tersoff if kind == "tersoff" else native.Kumagai
    pot = cls(precision=precision, **(params or {}))
    e, f, w = b.energy_and_forces(pot)
    return b, e, f, w


@pytest.mark.parametrize("kind", ["tersoff", "kumagai"])
def test_batch_matches_oracle_fp64(gpu, kind):
    structs = _mixed_set(10 if kind == "tersoff" else 20)
    params = TERSOFF if kind == "tersoff" else KUMAGAI
    b, e, f, w = _run_batch(structs, kind)
    for q, s in enumerate(structs):
        ref = oracle.bop(kind, params, s, per_at=False)
        n = len(s)
        fq = f[b.offsets[q]:b.offsets[q + 1]]
        assert abs(e[q] - ref["epot"]) / n < 1e-10, (q, e[q], ref["epot"])
        assert np.max(np.abs(fq - ref["f"])) < 1e-9, q
        assert np.max(np.abs(w[q] - ref["wpot"])) < 1e-9 * max(n, 1), q


def test_batch_equals_single_structure_path(gpu):
    structs = _mixed_set(30)
    b, e, f, w = _run_batch(structs)
    for q, s in enumerate(structs):
        one = gpu_bop("tersoff", s, per_at=False)
        fq = f[b.offsets[q]:b.offsets[q + 1]]
        assert np.array_equal(fq, one["f"]), q  # same list order, same per-bond sums
        assert abs(e[q] - one["epot"]) <= 1e-12 * max(1.0, abs(one["epot"]))
        assert np.max(np.abs(w[q] - one["wpot"])) <= 1e-12 * max(1.0, np.max(np.abs(w[q])))


def test_batch_mixed_precision(gpu):
    structs = S.si_batch(48, seed=41)
    b, e, f, w = _run_batch(structs, precision="mixed")
    for q, s in enumerate(structs):
        ref = oracle.bop("tersoff", TERSOFF, s, per_at=False)
        fq = f[b.offsets[q]:b.offsets[q + 1]]
        assert np.max(np.abs(fq - ref["f"])) <= MIXED_F_TOL, q
        assert abs(e[q] - ref["epot"]) / len(s) < 1e-6, q


def test_batch_deterministic_and_accumulating(gpu):
    structs = S.si_batch(32, seed=42)
    from atomistica_gb300 import native
    b = native.Batch(structs)
    pot = native.Tersoff(precision="mixed")
    e1, f1, w1 = b.energy_and_forces(pot)
    e2, f2, w2 = b.energy_and_forces(pot)
    assert np.array_equal(e1, e2) and np.array_equal(f1, f2) and np.array_equal(w1, w2)
    # forces are accumulated into a caller array, energies set
    f0 = np.ones_like(f1)
    e3, f3, _ = b.energy_and_forces(pot, forces=f0)
    assert np.array_equal(e3, e1)
    assert np.array_equal(f3, f1 + 1.0)
    # new positions rebuild the list
    r = np.concatenate([s.positions for s in structs]) + 0.01
    b.set_positions(r)
    e4, f4, _ = b.energy_and_forces(pot)
    assert not np.array_equal(f4, f1)


def test_batch_c4_sample_fp64(gpu):
    # a sample of the 2048-structure batch workload (N in [8, 512], strained
    # triclinic cells, 2.0 A minimum separation)
    structs = S.si_batch(64, seed=4)
    b, e, f, w = _run_batch(structs)
    worst = 0.0
    for q, s in enumerate(structs):
        ref = oracle.bop("tersoff", TERSOFF, s, per_at=False)
        fq = f[b.offsets[q]:b.offsets[q + 1]]
        worst = max(worst, float(np.max(np.abs(fq - ref["f"]))))
        assert abs(e[q] - ref["epot"]) / len(s) < 1e-10, q
    assert worst < 1e-9, worst


def test_batch_graph_replay_and_fallback(gpu):
    from atomistica_gb300 import native
    structs = S.si_batch(24, seed=43)
    r0 = np.concatenate([s.positions for s in structs])
    for prec in ("fp64", "mixed"):
        pot = native.Tersoff(precision=prec)
        eager = native.Batch(structs)
        graph = native.Batch(structs)
        graph.set_options(graph=True)
        e0, f0, w0 = eager.energy_and_forces(pot)
        e1, f1, w1 = graph.energy_and_forces(pot)    # eager, then captured
        info = graph.last_info()
        assert not info["replayed"] and info["graph_kernels"] > 0
        e2, f2, w2 = graph.energy_and_forces(pot)    # replay
        assert graph.last_info()["replayed"]
        for e, f, w in ((e1, f1, w1), (e2, f2, w2)):
            assert np.array_equal(f, f0) and np.array_equal(e, e0) and np.array_equal(w, w0)
        # new positions: the replay rebuilds the list on the device
        r1 = r0 + np.random.default_rng(3).uniform(-0.05, 0.05, r0.shape)
        eager.set_positions(r1)
        graph.set_positions(r1)
        e0, f0, _ = eager.energy_and_forces(pot)
        e3, f3, _ = graph.energy_and_forces(pot)
        assert graph.last_info()["replayed"]
        assert np.array_equal(f3, f0) and np.array_equal(e3, e0)
        # a denser configuration overflows the captured list capacity: the
        # replay is discarded and the evaluation redone eagerly
        dense = r0.copy()
        sl = slice(int(graph.offsets[0]), int(graph.offsets[1]))
        c = dense[sl].mean(axis=0)
        dense[sl] = c + 0.6 * (dense[sl] - c)
        eager.set_positions(dense)
        graph.set_positions(dense)
        e0, f0, _ = eager.energy_and_forces(pot)
        e4, f4, _ = graph.energy_and_forces(pot)
        assert not graph.last_info()["replayed"]
        assert np.array_equal(f4, f0) and np.array_equal(e4, e0)


def test_batch_autotune(gpu):
    from atomistica_gb300 import native
    structs = S.si_batch(16, seed=44)
    pot = native.Tersoff()
    plain = native.Batch(structs)
    tuned = native.Batch(structs)
    tuned.set_options(autotune=True)
    e0, f0, _ = plain.energy_and_forces(pot)
    e1, f1, _ = tuned.energy_and_forces(pot)
    info = tuned.last_info()
    assert info["tuned_candidates"] >= 1 and info["tile_bonds"] in (128, 192, 256)
    assert np.array_equal(f1, f0)  # per-bond sums do not depend on the tiles
    assert np.max(np.abs(e1 - e0)) <= 1e-12 * np.max(np.abs(e0))


def test_batch_eager_after_capture_same_positions(gpu):
    # the capture sizes the list arrays for its capacity; an eager call on
    # unchanged positions afterwards must not use a list lost by that
    from atomistica_gb300 import native
    structs = S.si_batch(24, seed=45)
    pot = native.Tersoff(precision="mixed")
    b = native.Batch(structs)
    b.set_options(graph=True)
    e1, f1, w1 = b.energy_and_forces(pot)   # eager, then captured
    b.set_options(graph=False)
    e2, f2, w2 = b.energy_and_forces(pot)   # eager on the same positions
    assert np.array_equal(f2, f1) and np.array_equal(e2, e1) and np.array_equal(w2, w1)


def test_batch_graph_device_arrays(gpu):
    # Device force arrays: the graph captured for the caller's array adds into
    # it directly (no staging copies); energies and virials are written on the
    # device.  An overflowed replay must leave the array untouched before the
    # eager redo, and another array must not be written through the old graph.
    import torch
    from atomistica_gb300 import native
    structs = S.si_batch(24, seed=46)
    r0 = np.concatenate([s.positions for s in structs])
    nat = len(r0)
    pot = native.Tersoff(precision="mixed")

    def reference(r):
        ref = native.Batch(structs)
        ref.set_positions(r)
        fr = torch.full((nat, 3), 0.5, dtype=torch.float64, device="cuda")
        e, _, w = ref.energy_and_forces(pot, forces=fr)
        return e.cpu().numpy(), fr.cpu().numpy(), w.cpu().numpy()

    def call(b, f):
        f.fill_(0.5)
        e, _, w = b.energy_and_forces(pot, forces=f)
        return e.cpu().numpy(), f.cpu().numpy(), w.cpu().numpy(), b.last_info()["replayed"]

    e0, f0, w0 = reference(r0)
    b = native.Batch(structs)
    b.set_options(graph=True)
    f = torch.zeros((nat, 3), dtype=torch.float64, device="cuda")
    for k in range(3):  # eager (then captured), then replays into the same array
        e, fg, w, rep = call(b, f)
        assert rep == (k > 0)
        assert np.array_equal(fg, f0) and np.array_equal(e, e0) and np.array_equal(w, w0)
    dense = r0.copy()
    sl = slice(int(b.offsets[0]), int(b.offsets[1]))
    c = dense[sl].mean(axis=0)
    dense[sl] = c + 0.6 * (dense[sl] - c)
    ed, fd, wd = reference(dense)
    b.set_positions(dense)
    e, fg, w, rep = call(b, f)
    assert not rep
    assert np.array_equal(fg, fd) and np.array_equal(e, ed) and np.array_equal(w, wd)
    # (the dense configuration re-cut the tiles: from here on the energies and
    # virials may differ from the reference by the rounding of the tile sums;
    # the forces do not depend on the tiles)
    b.set_positions(r0)
    call(b, f)
    e, fg, w, rep = call(b, f)
    assert rep and np.array_equal(fg, f0)
    f2 = torch.zeros((nat, 3), dtype=torch.float64, device="cuda")
    e, fg, w, rep = call(b, f2)  # another array: not through the old graph
    assert not rep and np.array_equal(fg, f0)
    # (the mixed form adds virials in FP32 per tile)
    assert np.allclose(e, e0, rtol=1e-12, atol=0)
    assert np.max(np.abs(w - w0)) <= 1e-5 * np.max(np.abs(w0))
    for arr in (f2, f, f2):  # later graphs stage through their own buffer
        e1, fg, w1, rep = call(b, arr)
        assert rep and np.array_equal(fg, f0)
        assert np.array_equal(e1, e) and np.array_equal(w1, w)
