"""GPU parity: the CUDA path through the C-ABI against the C++ FP64 oracle on
the same seeded inputs.  Neighbour pair sets must be bit-exact (and in the
reference's per-atom order); energies within 1e-10 eV/atom, forces and
virials within 1e-9 eV/A (per atom); the mixed form within 1e-5 eV/A."""

import numpy as np
import pytest

import oracle
from atomistica_gb300 import parameters as P
from atomistica_gb300 import structures as S

from helpers import (KUMAGAI, MIXED_F_TOL, TERSOFF, compare, gpu_bop, gpu_eam, random_carbon,
                     rattled_diamond, sorted_triples, triclinic_si)

pytestmark = pytest.mark.gpu


def _nl_check(s, cutoff, got):
    ref = oracle.neighbors(s, cutoff)
    seed, j, dc = got
    assert np.array_equal(seed, ref.seed), "per-atom neighbour counts differ"
    # identical order (reference per-atom order) implies identical sets
    assert np.array_equal(j, ref.nbr)
    assert np.array_equal(dc, ref.dc)
    assert np.array_equal(sorted_triples(seed, j, dc), ref.triples())


def _strained(s, eps):
    s = s.copy()
    F = np.eye(3) + np.asarray(eps)
    s.positions = s.positions @ F.T
    s.cell = s.cell @ F.T
    return s


# Structures above the small-structure size of the pair search (one thread,
# or one warp-flattened walk, per atom): cubic boxes (rows and cells beyond
# the cutoff skipped), a slab, a sheared box and atoms outside the box.
LARGE_NL = {
    "amorphous_65536": lambda: S.tersoff_si_amorphous(65536, seed=5),
    "amorphous_262144": lambda: S.tersoff_si_amorphous(262144, seed=6, sigma=0.4),
    "slab_65536": lambda: _nopbc(S.tersoff_si_amorphous(65536, seed=7), [True, True, False]),
    "sheared_65536": lambda: _strained(S.tersoff_si_amorphous(65536, seed=8),
                                       [[0, 0.03, 0], [0, 0, 0], [0.02, 0, 0]]),
    "outside_65536": lambda: _rattle(S.tersoff_si_amorphous(65536, seed=9), 2.0, 10),
}


@pytest.mark.parametrize("name", sorted(LARGE_NL))
def test_neighbour_list_large(gpu, name):
    # First build (count and fill passes), then a rebuild on moved positions
    # (single pass with staged entries): both bit-exact and in the
    # reference's per-atom order.
    from atomistica_gb300 import native
    s = LARGE_NL[name]()
    p = native.from_atoms(s)
    nl = native.Neighbors(100)
    nl.request_interaction_range(3.0)
    _nl_check(s, 3.0, nl.get_list(p))
    s2 = _rattle(s.copy(), 0.05, 11)
    p.coordinates[:] = s2.positions
    p.I_changed_positions()
    _nl_check(s2, 3.0, nl.get_list(p))


CASES = {
    "si_4096": lambda: S.tersoff_si_4096(),
    "si_rattled": lambda: rattled_diamond(amp=0.4, seed=1),
    "si_small_cell": lambda: rattled_diamond(size=(1, 1, 1), amp=0.2, seed=2),
    "si_triclinic_8": lambda: triclinic_si(8, seed=3),
    "si_triclinic_24": lambda: triclinic_si(24, seed=4),
    "si_triclinic_100": lambda: triclinic_si(100, seed=5),
    "carbon": lambda: random_carbon(96, seed=6),
    "sic": lambda: _rattle(S.b3(("Si", "C"), 4.3596, (2, 2, 2)), 0.3, 7),
}


def _rattle(s, amp, seed):
    s.positions += np.random.default_rng(seed).uniform(-amp, amp, s.positions.shape)
    return s


def _nopbc(s, pbc):
    s = s.copy()
    s.pbc = np.array(pbc)
    return s


@pytest.mark.parametrize("name", sorted(CASES))
def test_tersoff_fp64(gpu, name):
    s = CASES[name]()
    got = gpu_bop("tersoff", s)
    ref = oracle.bop("tersoff", TERSOFF, s)
    _nl_check(s, oracle.bop_cutoff("tersoff", TERSOFF, s), got["nl"])
    compare(ref, got, len(s))


@pytest.mark.parametrize("pbc", [(True, True, False), (False, False, False),
                                 (True, False, False)])
def test_tersoff_partial_pbc(gpu, pbc):
    s = _nopbc(rattled_diamond(size=(2, 2, 2), amp=0.2, seed=11), pbc)
    got = gpu_bop("tersoff", s)
    ref = oracle.bop("tersoff", TERSOFF, s)
    compare(ref, got, len(s))
    _nl_check(s, 3.0, got["nl"])


def test_tersoff_atoms_outside_cell(gpu):
    # positions far outside the box (shifted by lattice vectors, and non-pbc
    # clamping): python_neighbors.f90:645-659.
    s = rattled_diamond(size=(2, 2, 2), amp=0.2, seed=12)
    s.positions[5] += 3 * s.cell[0] - 2 * s.cell[2]
    s.positions[9] -= 4 * s.cell[1]
    got = gpu_bop("tersoff", s)
    ref = oracle.bop("tersoff", TERSOFF, s)
    compare(ref, got, len(s))
    _nl_check(s, 3.0, got["nl"])
    t = _nopbc(s, (False, True, True))
    t.cell = t.cell * 0.9
    got = gpu_bop("tersoff", t)
    ref = oracle.bop("tersoff", TERSOFF, t)
    compare(ref, got, len(t))


def test_floating_point_issue(gpu):
    # test_neighbor_list.py:155-175: coordination 4 with a -4.4e-52 coordinate.
    pos = np.array([[-4.41173839e-52, 0.0, 0.0], [-4.41173839e-52, 2.26371743, 2.26371743],
                    [2.26371743, 0.0, 2.26371743], [2.26371743, 2.26371743, 0.0],
                    [1.13185872, 1.13185872, 1.13185872], [1.13185872, 3.39557615, 3.39557615],
                    [3.39557615, 1.13185872, 3.39557615], [3.39557615, 3.39557615, 1.13185872]])
    s = S.Structure(pos, np.eye(3) * 4.527434867899659, np.array([True] * 3),
                    np.array([14] * 4 + [6] * 4, dtype=np.int32))
    got = gpu_bop("tersoff", s)
    ref = oracle.bop("tersoff", TERSOFF, s)
    compare(ref, got, len(s))
    seed, j, dc = got["nl"]
    i = np.repeat(np.arange(8), np.diff(seed))
    dr = pos[i] - pos[j] + dc @ s.cell
    r = np.sqrt((dr ** 2).sum(1))
    assert np.all(np.bincount(i[r < 3.0], minlength=8) == 4)


@pytest.mark.parametrize("seed", [0, 1])
def test_kumagai_fp64(gpu, seed):
    s = rattled_diamond(a=5.429, size=(2, 2, 2), amp=0.3, seed=20 + seed)
    got = gpu_bop("kumagai", s)
    ref = oracle.bop("kumagai", KUMAGAI, s)
    compare(ref, got, len(s))
    s = triclinic_si(40, seed=30 + seed)
    got = gpu_bop("kumagai", s)
    ref = oracle.bop("kumagai", KUMAGAI, s)
    compare(ref, got, len(s))


@pytest.mark.parametrize("kind", ["tersoff", "kumagai"])
def test_mask(gpu, kind):
    s = random_carbon(96, seed=40) if kind == "tersoff" else rattled_diamond(seed=41)
    params = TERSOFF if kind == "tersoff" else KUMAGAI
    mask = np.random.default_rng(42).integers(0, 2, len(s)).astype(bool)
    got = gpu_bop(kind, s, mask=mask)
    ref = oracle.bop(kind, params, s, mask=mask)
    compare(ref, got, len(s))
    # mask decomposition (test_mask.py:38-85)
    g2 = gpu_bop(kind, s, mask=~mask)
    g0 = gpu_bop(kind, s)
    assert abs(g0["epot"] - got["epot"] - g2["epot"]) < 1e-6
    assert np.max(np.abs(g0["f"] - got["f"] - g2["f"])) < 1e-6
    assert np.max(np.abs(g0["wpot"] - got["wpot"] - g2["wpot"])) < 1e-6


def test_per_bond(gpu):
    s = rattled_diamond(size=(2, 2, 2), amp=0.3, seed=50)
    got = gpu_bop("tersoff", s, per_bond=True)
    ref = oracle.bop("tersoff", TERSOFF, s, per_bond=True)
    assert np.max(np.abs(got["epot_per_bond"] - ref["epot_per_bond"])) < 1e-10
    assert np.max(np.abs(got["f_per_bond"] - ref["f_per_bond"])) < 1e-9
    # wpot_per_bond: reference buffer is Fortran (3,3,n), viewed (n,3,3) C-order
    wref = np.transpose(ref["wpot_per_bond"], (0, 2, 1))
    assert np.max(np.abs(got["wpot_per_bond"] - wref)) < 1e-9
    assert abs(got["epot_per_bond"].sum() - got["epot"]) < 1e-9


def test_unknown_elements_and_isolated(gpu):
    # atoms unknown to the potential are skipped as i and j (bop_kernel.f90:569,588)
    s = rattled_diamond(size=(2, 2, 2), amp=0.2, seed=60)
    s.numbers[::7] = 29
    got = gpu_bop("tersoff", s)
    ref = oracle.bop("tersoff", TERSOFF, s)
    compare(ref, got, len(s))
    # isolated dimer: zeta = 0 -> b = 1 (tersoff_func.f90:140-158)
    d = S.Structure(np.array([[5.0, 5.0, 5.0], [7.3, 5.0, 5.0]]), np.eye(3) * 20.0,
                    np.array([False] * 3), np.array([14, 14], dtype=np.int32))
    got = gpu_bop("tersoff", d)
    ref = oracle.bop("tersoff", TERSOFF, d)
    compare(ref, got, 2)
    # single atom and empty neighbourhood
    one = S.Structure(np.array([[1.0, 1.0, 1.0]]), np.eye(3) * 10.0, np.array([True] * 3),
                      np.array([14], dtype=np.int32))
    got = gpu_bop("tersoff", one)
    assert got["epot"] == 0.0 and np.all(got["f"] == 0.0)


def test_deterministic(gpu):
    s = S.tersoff_si_4096(seed=9)
    a = gpu_bop("tersoff", s)
    b = gpu_bop("tersoff", s)
    assert a["epot"] == b["epot"]
    assert np.array_equal(a["f"], b["f"]) and np.array_equal(a["wpot"], b["wpot"])
    am = gpu_bop("tersoff", s, precision="mixed")
    bm = gpu_bop("tersoff", s, precision="mixed")
    assert np.array_equal(am["f"], bm["f"]) and am["epot"] == bm["epot"]


@pytest.mark.parametrize("kind", ["tersoff", "kumagai"])
def test_mixed_precision(gpu, kind):
    s = S.tersoff_si_4096(seed=13) if kind == "tersoff" else rattled_diamond(
        a=5.429, size=(6, 6, 6), amp=0.2, seed=14)
    params = TERSOFF if kind == "tersoff" else KUMAGAI
    ref = oracle.bop(kind, params, s)
    got = gpu_bop(kind, s, precision="mixed")
    df = np.max(np.abs(got["f"] - ref["f"]))
    de = abs(got["epot"] - ref["epot"]) / len(s)
    assert df <= MIXED_F_TOL, df
    assert de < 1e-6, de
    assert np.max(np.abs(got["wpot"] - ref["wpot"])) < 1e-5 * len(s)


def _cu_setfl(tmp_path, **kw):
    from atomistica_gb300 import io as gio
    fn = str(tmp_path / "cu.setfl")
    gio.cu_analytic_setfl(fn, **kw)
    return fn


def test_eam_tables_bit_identical(gpu, tmp_path):
    from atomistica_gb300 import native
    fn = _cu_setfl(tmp_path, nr=1000, nrho=1000)
    pot = native.TabulatedAlloyEAM(fn)
    e = oracle.EAM(fn)
    for which, idx in ((0, 0), (1, 0), (2, 0)):
        xg, cg = pot.table(which, idx)
        xr, cr = e.table(which, idx)
        assert np.array_equal(xg, xr) and np.array_equal(cg, cr)


@pytest.mark.parametrize("size,sigma", [((3, 3, 3), 0.05), ((6, 6, 6), 0.1)])
def test_eam_fp64(gpu, tmp_path, size, sigma):
    fn = _cu_setfl(tmp_path, nr=2000, nrho=2000)
    rng = np.random.default_rng(70)
    s = S.fcc("Cu", 3.615, size)
    s.positions += rng.normal(0, sigma, s.positions.shape)
    got = gpu_eam(fn, s)
    ref = oracle.EAM(fn).compute(s)
    compare(ref, got, len(s))
    _nl_check(s, 5.0, got["nl"])


def test_derived_sqrt_is_correctly_rounded(gpu):
    # The EAM density pass derives r from its refined 1/sqrt(r^2) (one FMA
    # residual correction) instead of a separate square root; near a setfl
    # table's zero padding the interval coordinate needs r rounded exactly as
    # the correctly rounded sqrt.  2^27 arguments per range: the squared
    # distances of the tables and a wider range.
    import ctypes
    from atomistica_gb300 import _lib
    L = _lib.load()
    for lo, hi in ((1e-2, 1.0), (1.0, 100.0), (1e-6, 1e6)):
        bad = ctypes.c_int64(-1)
        assert L.gb_diag_sqrt_check(1 << 27, lo, hi, ctypes.byref(bad)) == 0
        assert bad.value == 0, (lo, hi, bad.value)


def test_eam_mask(gpu, tmp_path):
    fn = _cu_setfl(tmp_path, nr=2000, nrho=2000)
    rng = np.random.default_rng(71)
    s = S.fcc("Cu", 3.615, (3, 3, 3))
    s.positions += rng.normal(0, 0.05, s.positions.shape)
    mask = rng.integers(0, 2, len(s)).astype(bool)
    got = gpu_eam(fn, s, mask=mask)
    ref = oracle.EAM(fn).compute(s, mask=mask)
    compare(ref, got, len(s))
    g2 = gpu_eam(fn, s, mask=~mask)
    g0 = gpu_eam(fn, s)
    assert abs(g0["epot"] - got["epot"] - g2["epot"]) < 1e-6
    assert np.max(np.abs(g0["f"] - got["f"] - g2["f"])) < 1e-6


@pytest.mark.parametrize("natoms", [65536, 1048576])
def test_mixed_precision_amorphous_workload(gpu, natoms):
    # The bench workload (2.33 g/cm^3, sigma = 0.25 A, close contacts down to
    # ~0.5 A with forces of several hundred eV/A): the mixed form must stay
    # within 1e-5 eV/A of the FP64 oracle; the FP64 drop-in within 1e-9.
    s = S.tersoff_si_amorphous(natoms, seed=3)
    ref = oracle.bop_compute("tersoff", TERSOFF, s)
    g64 = gpu_bop("tersoff", s, per_at=False)
    gmx = gpu_bop("tersoff", s, precision="mixed", per_at=False)
    _nl_check(s, 3.0, g64["nl"])  # the full pair set, in the reference's order
    assert np.max(np.abs(g64["f"] - ref["f"])) < 1e-9
    assert abs(g64["epot"] - ref["epot"]) / natoms < 1e-10
    dfm = np.max(np.abs(gmx["f"] - ref["f"]))
    assert dfm <= MIXED_F_TOL, dfm
    assert abs(gmx["epot"] - ref["epot"]) / natoms < 1e-6
    # size-independent properties: no net force (translation invariance)
    assert np.max(np.abs(gmx["f"].sum(axis=0))) < 1e-6 * natoms ** 0.5
    assert np.max(np.abs(g64["f"].sum(axis=0))) < 1e-9 * natoms ** 0.5


def test_forces_set_instead_of_accumulated(gpu):
    from atomistica_gb300 import native
    s = rattled_diamond("Si", 5.431, (2, 2, 2), 0.2, 71)
    p = native.from_atoms(s)
    nl = native.Neighbors(100)
    pot = native.Tersoff()
    pot.bind_to(p, nl)
    e0, f0, w0 = pot.energy_and_forces(p, nl)
    f1 = np.full((len(s), 3), 7.0)
    e1, f1, w1 = pot.energy_and_forces(p, nl, forces=f1, accumulate=False)
    assert np.array_equal(f1, f0) and e1 == e0 and np.array_equal(w1, w0)
    f2 = np.full((len(s), 3), 7.0)
    _, f2, _ = pot.energy_and_forces(p, nl, forces=f2)
    assert np.max(np.abs(f2 - (f0 + 7.0))) < 1e-12


@pytest.mark.parametrize("size", [(3, 3, 3), (5, 5, 5)])
def test_funcfl_eam_fp64(gpu, tmp_path, size):
    # TabulatedEAM (single-element funcfl) against the oracle's restatement
    from atomistica_gb300 import io as gio
    from atomistica_gb300 import native
    from atomistica_gb300 import structures as S
    fn = gio.cu_analytic_funcfl(str(tmp_path / "cu.eam"))
    s = S.fcc("Cu", 3.615, size)
    s.positions += np.random.default_rng(8).normal(0, 0.08, s.positions.shape)
    ref = oracle.FuncflEAM(fn).compute(s)
    p = native.from_atoms(s)
    nl = native.Neighbors(100)
    pot = native.TabulatedEAM(fn)
    pot.bind_to(p, nl)
    e, f, w, epa, wpa = pot.energy_and_forces(p, nl, epot_per_at=True, wpot_per_at=True)
    n = len(s)
    assert abs(e - ref["epot"]) / n < 1e-10
    assert np.max(np.abs(f - ref["f"])) < 1e-9
    assert np.max(np.abs(w - ref["wpot"])) < 1e-9 * n
    assert np.max(np.abs(epa - ref["epot_per_at"])) < 1e-9
    assert not np.any(wpa)  # the reference kernel leaves the per-atom virial alone
    with pytest.raises(Exception):
        pot.energy_and_forces(p, nl, mask=np.ones(n, dtype=bool))
