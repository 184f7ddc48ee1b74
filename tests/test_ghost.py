"""The LAMMPS ghost-atom contract (gb_potential_energy_and_forces_ghost):
a periodic structure is given as its atoms plus explicit ghost images out to
twice the cutoff (the ghost width the reference requests for LAMMPS,
default_bind_to_func.f90:137-139) with a full, shift-free list over all of
them; bonds are computed for the local atoms only and the forces on ghosts
are summed back onto their owners, as LAMMPS does.  The result must equal the
periodic evaluation of the oracle."""

import numpy as np
import pytest

import oracle

from helpers import (KUMAGAI, TERSOFF, TERSOFF_SCR, MIXED_F_TOL, fold, ghost_system,
                     random_carbon, rattled_diamond)

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["tersoff", "kumagai", "tersoff_scr", "tersoff_mixed"])
def test_ghost_contract_equals_periodic(gpu, case):
    from atomistica_gb300 import native
    if case == "kumagai":
        s, kind, params = rattled_diamond("Si", 5.429, (3, 3, 3), 0.3, 41), "kumagai", KUMAGAI
        pot = native.Kumagai()
    elif case == "tersoff_scr":
        s, kind, params = random_carbon(64, seed=42), "tersoff_scr", TERSOFF_SCR
        pot = native.TersoffScr()
    else:
        s, kind, params = rattled_diamond("Si", 5.431, (3, 3, 3), 0.3, 43), "tersoff", TERSOFF
        pot = native.Tersoff(precision="mixed" if case == "tersoff_mixed" else "fp64")
    ref = oracle.bop(kind, params, s)
    cutoff = pot.get_cutoff()
    r_all, Z, owner, seed, nbr = ghost_system(s, cutoff)
    n = len(s)
    epot, f, wpot, epa, wpa = pot.energy_and_forces_ghost(r_all, Z, seed, nbr, n,
                                                          epot_per_at=True, wpot_per_at=True)
    if case == "tersoff_scr":
        # the screened loops stop early in list order, so the reference
        # itself depends on the list's order: compare with the oracle on the
        # same ghost list (and the periodic result to 1e-6 below)
        g = oracle.bop_ghost(kind, params, r_all, Z, seed, nbr, n)
        assert abs(epot - g["epot"]) / n < 1e-10
        assert np.max(np.abs(f - g["f"])) < 1e-9
        assert np.max(np.abs(wpot - g["wpot"])) < 1e-9 * n
        assert np.max(np.abs(epa - g["epot_per_at"])) < 1e-9
        assert np.max(np.abs(wpa - g["wpot_per_at"])) < 1e-9
        assert abs(epot - ref["epot"]) / n < 1e-6
        return
    ff = fold(owner, f, n)
    ftol = MIXED_F_TOL if case == "tersoff_mixed" else 1e-9
    etol = 1e-6 if case == "tersoff_mixed" else 1e-10
    assert abs(epot - ref["epot"]) / n < etol
    assert np.max(np.abs(ff - ref["f"])) < ftol
    if case != "tersoff_mixed":
        assert np.max(np.abs(wpot - ref["wpot"])) < 1e-9 * n
        assert np.max(np.abs(fold(owner, epa, n) - ref["epot_per_at"])) < 1e-9
        assert np.max(np.abs(fold(owner, wpa, n) - ref["wpot_per_at"])) < 1e-9


def test_ghost_arguments(gpu):
    from atomistica_gb300 import native
    from atomistica_gb300._lib import AtomisticaError
    pot = native.Tersoff()
    r = np.zeros((2, 3))
    r[1, 0] = 2.3
    # natloc > nat is rejected; a dimer with no ghosts works
    with pytest.raises(AtomisticaError):
        pot.energy_and_forces_ghost(r, [14, 14], [0, 1, 2], [1, 0], 3)
    e, f, w = pot.energy_and_forces_ghost(r, [14, 14], [0, 1, 2], [1, 0], 2)
    assert np.isfinite(e) and abs(f[0, 0] + f[1, 0]) < 1e-12


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_lammps_per_atom_virial_layout(gpu, precision):
    # lammps_<mod>_energy_and_forces takes wpot_per_at as Fortran (6,nat) and
    # accumulates -w11, -w22, -w33, -w21, -w31, -w32 into it (SUM_VIRIAL
    # under LAMMPS, macros.inc:202; bop_kernel.f90:1514-1517)
    from atomistica_gb300 import native
    s = rattled_diamond("Si", 5.431, (2, 2, 2), 0.3, 44)
    pot = native.Tersoff(precision=precision)
    r_all, Z, owner, seed, nbr = ghost_system(s, pot.get_cutoff())
    n, nall = len(s), len(r_all)
    e0, f0, w0, wpa = pot.energy_and_forces_ghost(r_all, Z, seed, nbr, n, wpot_per_at=True)
    vatom0 = np.random.default_rng(5).normal(size=(nall, 6))
    vatom = vatom0.copy()
    e1, f1, w1 = pot.energy_and_forces_ghost(r_all, Z, seed, nbr, n, vatom=vatom)
    assert e1 == e0 and np.array_equal(f1, f0) and np.array_equal(w1, w0)
    # numpy wpa[i, c, a] is Fortran element (a, c, i)
    comp = np.stack([wpa[:, 0, 0], wpa[:, 1, 1], wpa[:, 2, 2],
                     wpa[:, 0, 1], wpa[:, 0, 2], wpa[:, 1, 2]], axis=1)
    assert np.array_equal(vatom, vatom0 - comp)
    # summed over owners: the periodic oracle's per-atom virial, and over all
    # atoms minus the Voigt form of the total virial (wpot[a, c] = (a, c))
    ref = oracle.bop("tersoff", TERSOFF, s)
    rw = ref["wpot_per_at"]
    ref_comp = -np.stack([rw[:, 0, 0], rw[:, 1, 1], rw[:, 2, 2],
                          rw[:, 0, 1], rw[:, 0, 2], rw[:, 1, 2]], axis=1)
    tol = 1e-4 if precision == "mixed" else 1e-9
    assert np.max(np.abs(fold(owner, vatom - vatom0, n) - ref_comp)) < tol
    tot = -np.array([w1[0, 0], w1[1, 1], w1[2, 2], w1[1, 0], w1[2, 0], w1[2, 1]])
    wtol = 1e-6 * np.max(np.abs(tot)) if precision == "mixed" else 1e-9 * nall
    assert np.max(np.abs((vatom - vatom0).sum(axis=0) - tot)) < wtol
    with pytest.raises(ValueError):
        pot.energy_and_forces_ghost(r_all, Z, seed, nbr, n, vatom=np.zeros((nall, 9)))
