"""Host-side logic on CPU: workload generators, file formats, parameter
conversion and the Python front-end's behaviour without a GPU."""

import numpy as np
import pytest

import oracle
from atomistica_gb300 import io as gio
from atomistica_gb300 import parameters as P
from atomistica_gb300 import structures as S


def test_workload_sizes_and_density():
    s = S.tersoff_si_4096()
    assert len(s) == 4096 and np.allclose(np.diag(s.cell), 8 * 5.431)
    assert np.max(np.abs(s.positions - S.diamond("Si", 5.431, (8, 8, 8)).positions)) <= 0.1
    c = S.tersoff_si_amorphous(natoms=4096, seed=3)
    assert len(c) == 4096
    rho = len(c) * S.MASS_SI / S.AVOGADRO / c.get_volume() * 1e24
    assert abs(rho - 2.33) < 1e-9


def test_full_size_amorphous_construction():
    c = S.tersoff_si_amorphous()
    assert len(c) == 1048576
    assert c.info["sites"] == 8 * 51 ** 3 and c.info["deleted"] == 12632
    assert abs(c.info["a"] - 5.4086) < 1e-3


def test_batch_and_fit_sets():
    b = S.si_batch(nstruct=6, seed=1)
    for s in b:
        assert 8 <= len(s) <= 512
        d = s.positions[:, None, :] - s.positions[None, :, :]
        frac = d @ np.linalg.inv(s.cell)
        frac -= np.round(frac)
        r = np.sqrt(((frac @ s.cell) ** 2).sum(-1)) + np.eye(len(s)) * 10
        assert r.min() >= 2.0 - 1e-9
    f = S.si_fit_set(nstruct=10)
    assert all(len(s) in (64, 96, 144, 216) for s in f)


def test_setfl_round_trip(tmp_path):
    fn = gio.cu_analytic_setfl(str(tmp_path / "cu.setfl"), nr=500, nrho=400)
    e = oracle.EAM(fn)
    assert e.nel == 1 and abs(e.cutoff - 5.0) < 1e-15
    x, c = e.table(1, 0)
    r = np.arange(502) * x[1]
    expect = np.exp(-3.0 * (r[:500] / 2.556 - 1.0))
    assert np.allclose(c[0, :500], expect, rtol=0, atol=1e-15)
    assert c[0, 500] == 0 and c[0, 501] == 0  # two zero pads (tabulated_alloy_eam.f90:222)
    x, c = e.table(2, 0)
    rr = np.arange(500) * x[1]
    phi = 0.35 * (np.exp(-2.8 * (rr - 2.556)) - 2 * np.exp(-1.4 * (rr - 2.556)))
    assert np.allclose(c[0, :500], 0.5 * rr * phi, atol=1e-14)  # r*phi scaled by 1/2


def test_parameter_conversion():
    from atomistica_gb300 import _lib, native
    p = native.tersoff_params(P.Tersoff_PRB_39_5566_Si_C)
    assert p.nel == 2 and list(p.Z)[:2] == [6, 14]
    assert p.A[2] == 1.8308e3 and p.r2[2] == 3.0 and p.lambda_[1] == (3.4879 + 2.4799) / 2
    q = native.kumagai_params(P.Kumagai_CompMaterSci_39_457_Si)
    assert q.Z[0] == 14 and q.beta[0] == 1 and q.r2[0] == 3.3
    si = P.tersoff_single_element(P.Tersoff_PRB_39_5566_Si_C, "Si")
    assert si["A"] == [1.8308e3] and si["n"] == [7.8734e-1]
    assert isinstance(p, _lib.TersoffParams)


def test_brenner_parameters_and_checks():
    # brenner_module.f90:200-210: d = 0 and S <= 1 are rejected at set-up
    from atomistica_gb300 import _lib, native
    p = native.brenner_params(P.Erhart_PRB_71_035211_SiC)
    assert p.nel == 2 and list(p.Z)[:2] == [6, 14] and p.c[1] == 273987.0 and p.m[2] == 1
    with pytest.raises(ValueError):
        native.brenner_params(dict(P.Erhart_PRB_71_035211_SiC, D0=[6.0]))
    native.Brenner(**P.Erhart_PRB_71_035211_SiC)
    native.BrennerScr(**P.Erhart_PRB_71_035211_SiC__Scr)
    for bad in (dict(S=[2.167, 1.0, 1.842]), dict(d=[6.28433, 0.0, 0.81472]),
                dict(r2=[1.0, 2.6, 2.96])):
        with pytest.raises(_lib.AtomisticaError):
            native.Brenner(**dict(P.Erhart_PRB_71_035211_SiC, **bad))


@pytest.mark.parametrize("kind", ["brenner", "brenner_scr"])
def test_brenner_interaction_range(kind):
    # Brenner requests r2 of each present pair; BrennerScr sqrt(C_dr_cut)
    # max(r2, or2, bor2) of the pair itself (brenner_module.f90:229-243)
    import oracle
    prm = P.Erhart_PRB_71_035211_SiC__Scr if kind == "brenner_scr" else \
        P.Erhart_PRB_71_035211_SiC
    si = S.diamond("Si", 5.43)
    c = S.diamond("C", 3.57)
    if kind == "brenner":
        assert oracle.bop_cutoff(kind, prm, si) == 2.96
        assert oracle.bop_cutoff(kind, prm, c) == 2.15
    else:
        x = np.sqrt(9.0 / 8.0)
        assert abs(oracle.bop_cutoff(kind, prm, si) - x * 6.0) < 1e-12
        assert abs(oracle.bop_cutoff(kind, prm, c) - x * 4.0) < 1e-12


def test_pair_index_matches_reference_table():
    # src/macros.inc:110-123 table for maxval=4 (1-based): row i, col j>=i
    expect = {(1, 1): 1, (1, 2): 2, (1, 3): 3, (1, 4): 4, (2, 2): 5, (2, 3): 6, (2, 4): 7,
              (3, 3): 8, (3, 4): 9, (4, 4): 10}
    for (i, j), v in expect.items():
        assert P.pair_index(i - 1, j - 1, 4) + 1 == v
        assert P.pair_index(j - 1, i - 1, 4) + 1 == v


def test_cfg_reader(reference_tests_dir):
    import os
    s = gio.read_cfg(os.path.join(reference_tests_dir, "aC_small.cfg"))
    assert len(s) == 128 and np.all(s.numbers == 6)
    assert np.allclose(np.diag(s.cell), 9.584001)


def test_frontend_fails_loudly_without_gpu():
    from atomistica_gb300 import _lib, native
    _lib.load()
    if _lib.device_count() > 0:
        pytest.skip("a GPU is present")
    with pytest.raises(_lib.AtomisticaError):
        native.from_atoms(S.diamond("Si", 5.431))


def test_random_packing_generator():
    # grid path (large cell) and all-images path (thin triclinic cell)
    for nat, cell in ((200, np.diag([14.0, 15.0, 16.0])),
                      (12, np.array([[5.0, 0.0, 0.0], [2.6, 4.9, 0.0], [1.0, 1.2, 6.0]]))):
        a = S._random_packing(np.random.default_rng(5), nat, cell, 2.0)
        b = S._random_packing(np.random.default_rng(5), nat, cell, 2.0)
        assert np.array_equal(a, b)
        fr = a @ np.linalg.inv(cell)
        assert np.all((fr > -1e-12) & (fr < 1 + 1e-12))
        shifts = np.array([[i, j, k] for i in (-1, 0, 1) for j in (-1, 0, 1)
                           for k in (-1, 0, 1)], dtype=float) @ cell
        d = a[:, None, None, :] - a[None, :, None, :] + shifts[None, None, :, :]
        r2 = np.einsum("ijsk,ijsk->ijs", d, d)
        r2[np.arange(nat), np.arange(nat), 13] = np.inf  # self, zero shift
        assert np.sqrt(r2.min()) >= 2.0


@pytest.mark.parametrize("kind", ["tersoff", "kumagai", "tersoff_scr"])
def test_oracle_ghost_contract(kind):
    # bonds of the local atoms with explicit ghost images (the LAMMPS build)
    # equal the periodic evaluation; the screened loops depend on the list
    # order (early exit), so there the agreement is to 1e-6 eV
    import oracle
    from helpers import KUMAGAI, TERSOFF, TERSOFF_SCR, fold, ghost_system, rattled_diamond
    params = {"tersoff": TERSOFF, "kumagai": KUMAGAI, "tersoff_scr": TERSOFF_SCR}[kind]
    s = rattled_diamond("Si", 5.431, (2, 2, 2), 0.25, 51)
    ref = oracle.bop(kind, params, s)
    cut = oracle.bop_cutoff(kind, params, s)
    r, Z, owner, seed, nbr = ghost_system(s, cut)
    g = oracle.bop_ghost(kind, params, r, Z, seed, nbr, len(s))
    n = len(s)
    tol = 1e-6 if kind == "tersoff_scr" else 1e-10
    assert abs(g["epot"] - ref["epot"]) < tol * n
    assert np.max(np.abs(fold(owner, g["f"], n) - ref["f"])) < (1e-5 if kind == "tersoff_scr"
                                                                 else 1e-9)
    assert np.max(np.abs(fold(owner, g["epot_per_at"], n) - ref["epot_per_at"])) < \
        (1e-5 if kind == "tersoff_scr" else 1e-9)
