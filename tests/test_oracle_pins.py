"""Pins of the C++ FP64 oracle against the reference's own known-answer tests,
re-expressed without ASE (CPU only).  The reference ships no golden
energy/force vectors and cannot be compiled here, so these are what anchor the
oracle:

  * Si(100) unrelaxed surface energy 2.309 J/m^2 and bit-equal energies for
    "pbc z off" vs "z doubled" (tests/test_pbc.py:42-59);
  * Ec, a0 and elastic constants within 5 % (tests/test_bulk_properties.py,
    check logic src/python/atomistica/tests.py:335-415);
  * finite-difference forces and virial (src/python/atomistica/tests.py:44-119,
    tests/test_forces_and_virial.py);
  * mask additivity (tests/test_mask.py:38-85);
  * neighbour-list geometry and pbc counts (tests/test_neighbor_list.py);
  * EAM special cases (tests/test_eam_special_cases.py);
  * dimer continuity (tests/test_dimers.py:109-136).

The screened variants (TersoffScr, KumagaiScr) are pinned by the same tests
the reference runs for them: bulk properties, FD forces and virials, mask
additivity and the Kumagai dimer.  The Brenner form (Erhart-Albe Si-C and
BrennerScr, Brenner's carbon potential II, Henriksson Fe-C with masks,
Kioseoglou Al-N with n != 1) likewise: tests/test_bulk_properties.py:67-94 and
tests/test_forces_and_virial.py:91-114.
"""

import os

import numpy as np
import pytest

import oracle
from atomistica_gb300 import io as gio
from atomistica_gb300 import structures as S

from atomistica_gb300 import parameters as P

from helpers import KUMAGAI, TERSOFF, random_carbon, random_wch, rattled_diamond

TERSOFF_SCR = P.Tersoff_PRB_39_5566_Si_C__Scr
KUMAGAI_SCR = P.Kumagai_CompMaterSci_39_457_Si__Scr
BRENNER = P.Erhart_PRB_71_035211_SiC
BRENNER_SCR = P.Erhart_PRB_71_035211_SiC__Scr
JUSLIN = P.Juslin_JAP_98_123520_WCH
JUSLIN_SCR = P.Juslin_JAP_98_123520_WCH__Scr
PARAMS = {"tersoff": TERSOFF, "kumagai": KUMAGAI, "tersoff_scr": TERSOFF_SCR,
          "kumagai_scr": KUMAGAI_SCR, "brenner": BRENNER, "brenner_scr": BRENNER_SCR,
          "juslin": JUSLIN, "juslin_scr": JUSLIN_SCR}

GPA = 160.21766208  # eV/A^3 -> GPa
JM2 = 16.02176634  # eV/A^2 -> J/m^2


def energy(kind, s, params=None, mask=None):
    if kind == "eam":
        return params.compute(s, mask=mask, per_at=False)
    return oracle.bop(kind, params, s, mask=mask, per_at=False)


def stress(kind, s, params):
    w = energy(kind, s, params)["wpot"]
    return np.array([w[0, 0], w[1, 1], w[2, 2], (w[1, 2] + w[2, 1]) / 2,
                     (w[0, 2] + w[2, 0]) / 2, (w[0, 1] + w[1, 0]) / 2]) / s.get_volume()


def lattice_minimum(kind, builder, params, a_lo, a_hi):
    """Golden-section search of E(a)/N for a perfect cubic crystal."""
    g = (np.sqrt(5) - 1) / 2
    f = lambda a: energy(kind, builder(a), params)["epot"] / len(builder(a))  # noqa: E731
    x1, x2 = a_hi - g * (a_hi - a_lo), a_lo + g * (a_hi - a_lo)
    f1, f2 = f(x1), f(x2)
    for _ in range(60):
        if f1 < f2:
            a_hi, x2, f2 = x2, x1, f1
            x1 = a_hi - g * (a_hi - a_lo)
            f1 = f(x1)
        else:
            a_lo, x1, f1 = x1, x2, f2
            x2 = a_lo + g * (a_hi - a_lo)
            f2 = f(x2)
    a0 = 0.5 * (a_lo + a_hi)
    return a0, f(a0)


def strained(s, T):
    t = s.copy()
    t.set_cell(np.dot(np.eye(3) + T, s.cell.T).T, scale_atoms=True)
    return t


def relax_positions(kind, s, params):
    from scipy.optimize import minimize
    x0 = s.positions.ravel().copy()

    def fun(x):
        t = s.copy()
        t.positions = x.reshape(-1, 3)
        o = energy(kind, t, params)
        return o["epot"], -o["f"].ravel()

    r = minimize(fun, x0, jac=True, method="L-BFGS-B", options={"gtol": 1e-10, "ftol": 1e-15,
                                                                "maxiter": 2000})
    t = s.copy()
    t.positions = r.x.reshape(-1, 3)
    return t


def cubic_elastic_constants(kind, s, params, eps=1e-6, relax=False):
    """Unrelaxed (or position-relaxed) C11, C12, C44 in GPa
    (cubic_elastic_constants, src/python/atomistica/tests.py:143-183)."""
    s0 = stress(kind, s, params)
    rl = (lambda t: relax_positions(kind, t, params)) if relax else (lambda t: t)
    a = stress(kind, rl(strained(s, np.diag([eps, 0, 0]))), params)
    C11 = (a[0] - s0[0]) / eps
    b = stress(kind, rl(strained(s, np.diag([eps, -eps / 2, -eps / 2]))), params)
    Cp = ((b[0] - s0[0]) - (b[1] - s0[1])) / (3 * eps)
    C12 = C11 - 2 * Cp
    T = np.array([[0, .5, .5], [.5, 0, .5], [.5, .5, 0]]) * eps
    c = stress(kind, rl(strained(s, T)), params)
    C44 = (c[3] + c[4] + c[5] - s0[3] - s0[4] - s0[5]) / (3 * eps)
    return C11 * GPA, C12 * GPA, C44 * GPA


def within(x, target, pct=5.0):
    return abs(x - target) * 100.0 / abs(target) < pct


# ---------------------------------------------------------------------------


def test_surface_energy_and_pbc_bit_equality():
    a = S.diamond("Si", 5.432, (2, 2, 2))
    sx, sy, sz = np.diag(a.cell)
    e1 = energy("tersoff", a, TERSOFF)["epot"]
    b = a.copy()
    b.pbc = np.array([True, True, False])
    e2 = energy("tersoff", b, TERSOFF)["epot"]
    c = a.copy()
    c.cell = np.diag([sx, sy, 2 * sz])
    e3 = energy("tersoff", c, TERSOFF)["epot"]
    assert e2 == e3
    esurf = (e2 - e1) / (2 * sx * sy) * JM2
    assert abs(esurf - 2.309) < 0.001, esurf


@pytest.mark.parametrize("case", [
    # name, kind, builder, Ec, a0, C11, C12, C44 unrelaxed (C440)
    ("tersoff dia-Si", "tersoff", lambda a: S.diamond("Si", a), 4.63, 5.432, 143, 75, 119),
    ("tersoff dia-C", "tersoff", lambda a: S.diamond("C", a), 7.396 - 0.0250, 3.566, 1067, 104,
     671),
    ("tersoff B3-SiC", "tersoff", lambda a: S.b3(("Si", "C"), a), 6.165, 4.321, 437, 118, 311),
    ("kumagai dia-Si", "kumagai", lambda a: S.diamond("Si", a), 4.630, 5.429, 166.4, 65.3,
     120.9),
    # screened variants: the same targets (tests/test_bulk_properties.py:122-160)
    ("tersoff_scr dia-Si", "tersoff_scr", lambda a: S.diamond("Si", a), 4.63, 5.432, 143, 75,
     119),
    ("tersoff_scr dia-C", "tersoff_scr", lambda a: S.diamond("C", a), 7.396 - 0.0250, 3.566,
     1067, 104, 671),
    ("tersoff_scr B3-SiC", "tersoff_scr", lambda a: S.b3(("Si", "C"), a), 6.165, 4.321, 437,
     118, 311),
    ("kumagai_scr dia-Si", "kumagai_scr", lambda a: S.diamond("Si", a), 4.630, 5.429, 166.4,
     65.3, 120.9),
])
def test_bulk_properties_bop(case):
    name, kind, builder, Ec, a0, C11, C12, C440 = case
    params = PARAMS[kind]
    a_min, e_min = lattice_minimum(kind, builder, params, 0.9 * a0, 1.1 * a0)
    assert within(-e_min, Ec), (name, e_min)
    assert within(a_min, a0), (name, a_min)
    c11, c12, c44 = cubic_elastic_constants(kind, builder(a_min), params)
    assert within(c11, C11), (name, c11)
    assert within(c12, C12), (name, c12)
    assert within(c44, C440), (name, c44)


@pytest.mark.parametrize("case", [
    # tests/test_bulk_properties.py:67-94: name, kind, params, builder, Ec, a0, C11, C12,
    # unrelaxed C44 (C440), relaxed C44 (C44r), B = (C11 + 2 C12)/3
    ("erhart dia-C", "brenner", BRENNER, lambda a: S.diamond("C", a), 7.3731, 3.566, 1082, 127,
     None, 673, 445),
    ("erhart dia-Si", "brenner", BRENNER, lambda a: S.diamond("Si", a), 4.63, 5.429, 167, 65,
     105, None, 99),
    ("erhart B3-SiC", "brenner", BRENNER, lambda a: S.b3(("Si", "C"), a), 6.340, 4.359, 382,
     145, 305, None, 224),
    ("erhart_scr dia-C", "brenner_scr", BRENNER_SCR, lambda a: S.diamond("C", a), 7.3731, 3.566,
     1082, 127, None, 673, 445),
    ("erhart_scr dia-Si", "brenner_scr", BRENNER_SCR, lambda a: S.diamond("Si", a), 4.63, 5.429,
     167, 65, 105, None, 99),
    ("erhart_scr B3-SiC", "brenner_scr", BRENNER_SCR, lambda a: S.b3(("Si", "C"), a), 6.340,
     4.359, 382, 145, 305, None, 224),
    ("brenner II dia-C", "brenner", P.Brenner_PRB_42_9458_C_II, lambda a: S.diamond("C", a),
     7.376 - 0.0524, 3.558, 621, 415, None, 383, 484),
])
def test_bulk_properties_brenner(case):
    name, kind, params, builder, Ec, a0, C11, C12, C440, C44r, B = case
    a_min, e_min = lattice_minimum(kind, builder, params, 0.9 * a0, 1.1 * a0)
    assert within(-e_min, Ec), (name, e_min)
    assert within(a_min, a0), (name, a_min)
    c11, c12, c44 = cubic_elastic_constants(kind, builder(a_min), params)
    assert within(c11, C11), (name, c11)
    assert within(c12, C12), (name, c12)
    assert within((c11 + 2 * c12) / 3, B), (name, c11, c12)
    if C440 is not None:
        assert within(c44, C440), (name, c44)
    if C44r is not None:
        _, _, c44r = cubic_elastic_constants(kind, builder(a_min), params, eps=1e-3, relax=True)
        assert within(c44r, C44r), (name, c44r)


@pytest.mark.parametrize("case", [
    # tests/test_bulk_properties.py:95-117 (Juslin, Juslin_JAP_98_123520_WCH):
    # name, builder, Ec, a0, C11, C12, C44 (bcc: no internal relaxation), B.
    # The reference's sc-W cell is 2x2x2 simple-cubic cells, so its a0 is
    # twice the lattice constant of the one-atom cell built here.
    ("bcc-W", lambda a: S.bcc("W", a), 8.89, 3.165, 542, 191, 162, 308),
    ("fcc-W", lambda a: S.fcc("W", a), 8.89 - 0.346, 4.005, None, None, None, None),
    ("sc-W", lambda a: S.sc("W", a), 8.89 - 1.614, 2.671, None, None, None, None),
    ("dia-C", lambda a: S.diamond("C", a), 7.376 - 0.0524, 3.558, 621, 415, None, 484),
    ("B1-W-C", lambda a: S.b1(("W", "C"), a), (16.68 - 0.98) / 2, 4.380, None, None, None, 433),
    ("B2-W-C", lambda a: S.b2(("W", "C"), a), (16.68 - 2.32) / 2, 2.704, None, None, None, 411),
    ("B3-W-C", lambda a: S.b3(("W", "C"), a), (16.68 - 2.12) / 2, 4.679, None, None, None, 511),
])
def test_bulk_properties_juslin(case):
    name, builder, Ec, a0, C11, C12, C44, B = case
    a_min, e_min = lattice_minimum("juslin", builder, JUSLIN, 0.9 * a0, 1.1 * a0)
    assert within(-e_min, Ec), (name, e_min)
    assert within(a_min, a0), (name, a_min)
    if C11 is None and B is None:
        return
    c11, c12, c44 = cubic_elastic_constants("juslin", builder(a_min), JUSLIN)
    if C11 is not None:
        assert within(c11, C11), (name, c11)
        assert within(c12, C12), (name, c12)
    if C44 is not None:
        assert within(c44, C44), (name, c44)
    assert within((c11 + 2 * c12) / 3, B), (name, c11, c12)


def test_relaxed_c44_tersoff_si():
    a_min, _ = lattice_minimum("tersoff", lambda a: S.diamond("Si", a), TERSOFF, 5.3, 5.6)
    s = S.diamond("Si", a_min)
    s.positions += 0.1
    _, _, c44 = cubic_elastic_constants("tersoff", s, TERSOFF, eps=1e-3, relax=True)
    assert within(c44, 69), c44


def test_bulk_properties_eam_au(reference_tests_dir):
    e = oracle.EAM(os.path.join(reference_tests_dir, "Au-Grochola-JCP05.eam.alloy"))
    builder = lambda a: S.fcc("Au", a)  # noqa: E731
    a_min, e_min = lattice_minimum("eam", builder, e, 3.9, 4.2)
    assert within(-e_min, 3.924) and within(a_min, 4.070)
    c11, c12, c44 = cubic_elastic_constants("eam", builder(a_min), e)
    assert within(c11, 202) and within(c12, 170) and within(c44, 46), (c11, c12, c44)


class _Funcfl:
    """funcfl oracle behind the EAM interface of these helpers (no masks)."""

    def __init__(self, fn):
        self.e = oracle.FuncflEAM(fn)

    def compute(self, s, mask=None, per_at=False):
        assert mask is None
        return self.e.compute(s, per_at=per_at)


def test_bulk_properties_funcfl_au(reference_tests_dir):
    # TabulatedEAM Au_u3.eam (tests/test_bulk_properties.py:133-136)
    e = _Funcfl(os.path.join(reference_tests_dir, "Au_u3.eam"))
    builder = lambda a: S.fcc("Au", a)  # noqa: E731
    a_min, e_min = lattice_minimum("eam", builder, e, 3.9, 4.2)
    assert within(-e_min, 3.93) and within(a_min, 4.08), (e_min, a_min)
    c11, c12, c44 = cubic_elastic_constants("eam", builder(a_min), e)
    assert within(c11, 183) and within(c12, 159) and within(c44, 45), (c11, c12, c44)
    assert within((c11 + 2 * c12) / 3, 167)


def test_fd_forces_virial_funcfl(tmp_path):
    e = _Funcfl(gio.cu_analytic_funcfl(str(tmp_path / "cu.eam")))
    s = S.fcc("Cu", 3.615, (3, 3, 3))
    s.positions += np.random.default_rng(7).normal(0, 0.05, s.positions.shape)
    ferr, werr = fd_check("eam", s, e, natoms=8)
    assert ferr < 1e-6 and werr < 1e-5, (ferr, werr)


def fd_check(kind, s, params, dx=1e-6, natoms=None, mask=None):
    o = energy(kind, s, params, mask=mask)
    err = 0.0
    for a in range(len(s) if natoms is None else min(natoms, len(s))):
        for c in range(3):
            sp, sm = s.copy(), s.copy()
            sp.positions[a, c] += dx
            sm.positions[a, c] -= dx
            ffd = -(energy(kind, sp, params, mask)["epot"] - energy(kind, sm, params, mask)["epot"])
            err = max(err, abs(ffd / (2 * dx) - o["f"][a, c]))
    W = np.zeros((3, 3))
    for i in range(3):
        for j in range(3):
            E = []
            for sg in (-1, 1):
                T = np.zeros((3, 3))
                T[i, j] = sg * dx
                t = s.copy()
                t.set_cell(s.cell @ (np.eye(3) + T), scale_atoms=True)
                E.append(energy(kind, t, params, mask)["epot"])
            W[i, j] = (E[1] - E[0]) / (2 * dx)
    return err, np.max(np.abs(W - o["wpot"]))


@pytest.mark.parametrize("scr", [False, True])
@pytest.mark.parametrize("name", ["dia-Si", "dia-C", "B3-SiC", "a-C", "kumagai"])
def test_fd_forces_virial_bop(name, scr):
    # tests/test_forces_and_virial.py:115-140 (Tersoff, TersoffScr, Kumagai,
    # KumagaiScr on dia-C, a-C, dia-Si, B3-SiC)
    if name == "dia-Si":
        kind, s = "tersoff", rattled_diamond("Si", 5.431, (2, 2, 2), 0.5, 1)
    elif name == "dia-C":
        kind, s = "tersoff", rattled_diamond("C", 3.566, (2, 2, 2), 0.3, 2)
    elif name == "B3-SiC":
        s = S.b3(("Si", "C"), 4.3596, (2, 2, 2))
        s.positions += np.random.default_rng(3).uniform(-0.4, 0.4, s.positions.shape)
        kind = "tersoff"
    elif name == "a-C":
        kind, s = "tersoff", random_carbon(64, seed=4)
    else:
        kind, s = "kumagai", rattled_diamond("Si", 5.429, (2, 2, 2), 0.4, 5)
    if scr:
        kind += "_scr"
    ferr, werr = fd_check(kind, s, PARAMS[kind], natoms=12)
    assert ferr < 1e-5 and werr < 1e-4, (ferr, werr)


@pytest.mark.parametrize("scr", [False, True])
@pytest.mark.parametrize("name", ["dia-C", "dia-Si", "B3-SiC", "a-C"])
def test_fd_forces_virial_brenner(name, scr):
    # tests/test_forces_and_virial.py:91-102 (Brenner, BrennerScr with
    # Erhart_PRB_71_035211_SiC on dia-C, a-C, dia-Si, B3-SiC)
    if name == "dia-C":
        s = rattled_diamond("C", 3.566, (2, 2, 2), 0.3, 21)
    elif name == "dia-Si":
        s = rattled_diamond("Si", 5.429, (2, 2, 2), 0.5, 22)
    elif name == "B3-SiC":
        s = S.b3(("Si", "C"), 4.3596, (2, 2, 2))
        s.positions += np.random.default_rng(23).uniform(-0.4, 0.4, s.positions.shape)
    else:
        s = random_carbon(64, seed=24)
    kind = "brenner_scr" if scr else "brenner"
    # dx = 1e-5: the reference form of g, 1 + c^2/d^2 - c^2/(d^2 + (h + cos)^2),
    # cancels ~6 digits for the Si-C pair (c^2/d^2 = 2.3e6), so the energy
    # carries ~1e-11 eV of rounding noise that a 1e-6 step turns into 3e-5 eV/A
    ferr, werr = fd_check(kind, s, PARAMS[kind], dx=1e-5, natoms=12)
    assert ferr < 1e-5 and werr < 1e-4, (ferr, werr)


@pytest.mark.parametrize("params", ["WCH", "FeCH"])
@pytest.mark.parametrize("scr", [False, True])
@pytest.mark.parametrize("name", ["bcc-W", "B1-W-C", "W-C-H"])
def test_fd_forces_virial_juslin(name, scr, params):
    # Juslin / JuslinScr (W-C-H and Kuopanportti Fe-C-H sets): rattled W and
    # WC crystals and a random W-C-H packing in which every triplet type of
    # h = omega exp(alpha dr) occurs, with and without masks
    rng = np.random.default_rng(91)
    metal = "W" if params == "WCH" else "Fe"
    if name == "bcc-W":
        s = S.bcc(metal, 3.165 if metal == "W" else 2.87, (3, 3, 3))
        s.positions += rng.uniform(-0.15, 0.15, s.positions.shape)
    elif name == "B1-W-C":
        s = S.b1((metal, "C"), 4.38, (2, 2, 2))
        s.positions += rng.uniform(-0.15, 0.15, s.positions.shape)
    else:
        s = random_wch(64, seed=92)
        s.numbers[s.numbers == 74] = 74 if metal == "W" else 26
    base = {"WCH": (JUSLIN, JUSLIN_SCR),
            "FeCH": (P.Kuopanportti_CMS_111_525_FeCH,
                     P.Kuopanportti_CMS_111_525_FeCH__Scr)}[params]
    kind = "juslin_scr" if scr else "juslin"
    mask = rng.integers(0, 2, len(s)).astype(bool) if name == "W-C-H" else None
    ferr, werr = fd_check(kind, s, base[1] if scr else base[0], natoms=10, mask=mask)
    assert ferr < 1e-5 and werr < 1e-4, (ferr, werr)


@pytest.mark.parametrize("name", ["dia-C", "a-C", "bcc-Fe", "fcc-Fe", "sc-Fe", "B1-Fe-C"])
def test_fd_forces_virial_brenner_fec_masked(name):
    # tests/test_forces_and_virial.py:103-114 (Henriksson_PRB_79_114107_FeC,
    # mask=True, rattled)
    rng = np.random.default_rng(25)
    s = {"dia-C": lambda: S.diamond("C", 3.566, (2, 2, 2)),
         "a-C": lambda: random_carbon(64, seed=26),
         "bcc-Fe": lambda: S.bcc("Fe", 2.87, (3, 3, 3)),
         "fcc-Fe": lambda: S.fcc("Fe", 3.6, (2, 2, 2)),
         "sc-Fe": lambda: S.sc("Fe", 2.4, (3, 3, 3)),
         "B1-Fe-C": lambda: S.b1(("Fe", "C"), 3.9, (2, 2, 2))}[name]()
    s.positions += rng.uniform(-0.1, 0.1, s.positions.shape)
    mask = rng.integers(0, 2, len(s)).astype(bool)
    ferr, werr = fd_check("brenner", s, P.Henriksson_PRB_79_114107_FeC, natoms=8, mask=mask)
    assert ferr < 1e-5 and werr < 1e-4, (ferr, werr)


def test_fd_forces_virial_brenner_aln_fractional_n():
    # Kioseoglou Al-N: n = 0.72 and 6.0865 (the zeta^n branch of bo)
    s = S.b3(("Al", "N"), 4.38, (2, 2, 2))
    s.positions += np.random.default_rng(27).uniform(-0.3, 0.3, s.positions.shape)
    ferr, werr = fd_check("brenner", s, P.Kioseoglou_PSSb_245_1118_AlN, natoms=12)
    assert ferr < 1e-5 and werr < 1e-4, (ferr, werr)


def test_fd_forces_virial_eam(tmp_path):
    fn = gio.cu_analytic_setfl(str(tmp_path / "cu.setfl"), nr=3000, nrho=3000)
    e = oracle.EAM(fn)
    rng = np.random.default_rng(6)
    # a = 3.7 keeps the 4th shell (5.23 A) clear of the untapered 5.0 A cutoff,
    # where the zero-padded spline's large third derivative spoils central FD.
    s = S.fcc("Cu", 3.7, (2, 2, 2))
    s.positions += rng.normal(0, 0.05, s.positions.shape)
    mask = rng.integers(0, 2, len(s)).astype(bool)
    ferr, werr = fd_check("eam", s, e, natoms=8)
    assert ferr < 1e-6 and werr < 1e-5, (ferr, werr)
    ferr, werr = fd_check("eam", s, e, natoms=8, mask=mask)
    assert ferr < 1e-6 and werr < 1e-5, (ferr, werr)


def test_eam_special_cases(reference_tests_dir):
    e = oracle.EAM(os.path.join(reference_tests_dir, "Cu_mishin1.eam.alloy"))
    a = gio.read_poscar(os.path.join(reference_tests_dir, "eam_crash1.poscar"))
    energy("eam", a, e)
    orig = gio.read_poscar(os.path.join(reference_tests_dir, "eam_crash2.poscar"))
    for fac in (0.2, 0.3, 0.4, 0.5):
        s = orig.copy()
        s.set_cell(fac * s.cell, scale_atoms=True)
        o = energy("eam", s, e)
        err = 0.0
        for q in range(0, len(s), 8):
            for c in range(3):
                sp, sm = s.copy(), s.copy()
                sp.positions[q, c] += 1e-6
                sm.positions[q, c] -= 1e-6
                ffd = -(energy("eam", sp, e)["epot"] - energy("eam", sm, e)["epot"]) / 2e-6
                err = max(err, (ffd - o["f"][q, c]) ** 2)
        assert err < 1e-6, (fac, err)


@pytest.mark.parametrize("kind", ["tersoff", "tersoff_scr", "brenner", "brenner_scr", "juslin",
                                  "juslin_scr"])
def test_mask_additivity(kind):
    # tests/test_mask.py:68 (Tersoff, TersoffScr; Brenner, BrennerScr; the
    # same property for Juslin, JuslinScr on a W-C-H packing)
    s = random_wch(96, seed=8) if kind.startswith("juslin") else random_carbon(96, seed=8)
    mask = np.random.default_rng(9).integers(0, 2, len(s)).astype(bool)
    o = energy(kind, s, PARAMS[kind])
    o1 = energy(kind, s, PARAMS[kind], mask=mask)
    o2 = energy(kind, s, PARAMS[kind], mask=~mask)
    assert abs(o["epot"] - o1["epot"] - o2["epot"]) < 1e-6
    assert np.max(np.abs(o["f"] - o1["f"] - o2["f"])) < 1e-6
    assert np.max(np.abs(o["wpot"] - o1["wpot"] - o2["wpot"])) < 1e-6


def test_neighbor_list_pbc_counts():
    base = S.Structure(np.array([[0.1, 0.5, 0.5], [0.9, 0.5, 0.5]]), np.eye(3),
                       np.array([True] * 3), np.array([6, 6], dtype=np.int32))
    for pbc, n in (((True, True, True), 2), ((False, False, False), 0),
                   ((False, False, True), 0), ((True, False, False), 2)):
        s = base.copy()
        s.pbc = np.array(pbc)
        assert len(oracle.neighbors(s, 0.3).nbr) == n


def _brute_pairs(s, cutoff):
    """All (i, j, shift) with |r_i - r_j + shift.cell| < cutoff by brute force."""
    inv = np.linalg.inv(s.cell)
    heights = 1.0 / np.linalg.norm(inv, axis=0)
    rng = [np.arange(-int(np.ceil(cutoff / h)) - 1, int(np.ceil(cutoff / h)) + 2) if p
           else np.array([0]) for h, p in zip(heights, s.pbc)]
    shifts = np.stack(np.meshgrid(*rng, indexing="ij"), -1).reshape(-1, 3)
    out = []
    r = s.positions
    for i in range(len(s)):
        d = r[i][None, None, :] - r[None, :, :] + (shifts @ s.cell)[:, None, :]
        d2 = np.einsum("abk,abk->ab", d, d)
        for q, j in zip(*np.nonzero(d2 < cutoff * cutoff)):
            if i == j and not shifts[q].any():
                continue
            out.append((i, j, *shifts[q]))
    t = np.array(sorted(out), dtype=np.int64)
    return t


@pytest.mark.parametrize("case", ["carbon", "triclinic", "small", "nopbc"])
def test_neighbor_list_against_brute_force(case):
    from helpers import triclinic_si
    if case == "carbon":
        s, cut = random_carbon(64, seed=10), 5.0
    elif case == "triclinic":
        s, cut = triclinic_si(16, seed=11), 3.0
    elif case == "small":
        s, cut = rattled_diamond("Si", 5.431, (1, 1, 1), 0.3, 12), 4.5
    else:
        s, cut = rattled_diamond("Si", 5.431, (2, 2, 2), 0.3, 13), 3.0
        s.pbc = np.array([True, False, True])
        s.positions[3] += np.array([0, 20.0, 0])
    nl = oracle.neighbors(s, cut)
    assert np.array_equal(nl.triples(), _brute_pairs(s, cut))
    d = s.positions[nl.i] - s.positions[nl.nbr] + nl.dc @ s.cell
    assert np.all(np.sqrt((d * d).sum(1)) < cut)


def test_shift_invariance_and_small_cells():
    s = random_carbon(96, seed=14)
    e1 = energy("tersoff", s, TERSOFF)["epot"]
    t = s.copy()
    t.positions[10] += 3 * t.cell[0]
    t.positions[20] += t.cell.T.dot([1, 3, -4])
    assert abs(energy("tersoff", t, TERSOFF)["epot"] - e1) < 1e-8
    # no pbc, cell shrunk without moving atoms (test_no_pbc_small_cell)
    u = s.copy()
    u.pbc = np.array([False] * 3)
    e1 = energy("tersoff", u, TERSOFF)["epot"]
    u.cell = u.cell * 0.9
    assert abs(energy("tersoff", u, TERSOFF)["epot"] - e1) < 1e-8


def test_floating_point_issue_coordination():
    pos = np.array([[-4.41173839e-52, 0.0, 0.0], [-4.41173839e-52, 2.26371743, 2.26371743],
                    [2.26371743, 0.0, 2.26371743], [2.26371743, 2.26371743, 0.0],
                    [1.13185872, 1.13185872, 1.13185872], [1.13185872, 3.39557615, 3.39557615],
                    [3.39557615, 1.13185872, 3.39557615], [3.39557615, 3.39557615, 1.13185872]])
    cell = np.eye(3) * 4.527434867899659
    s = S.Structure(pos, cell, np.array([True] * 3),
                    np.array([14] * 4 + [6] * 4, dtype=np.int32))
    for t in (s, S.Structure(s.get_scaled_positions() @ cell, cell, s.pbc, s.numbers)):
        nl = oracle.neighbors(t, 3.0)
        d = t.positions[nl.i] - t.positions[nl.nbr] + nl.dc @ t.cell
        r = np.sqrt((d * d).sum(1))
        assert np.all(np.bincount(nl.i[r < 3.0], minlength=8) == 4)


@pytest.mark.parametrize("kind", ["kumagai", "kumagai_scr"])
def test_dimer_continuity_kumagai(kind):
    # tests/test_dimers.py:109-136 (Kumagai, KumagaiScr)
    vac = 4.0
    e, f = [], []
    for d in np.linspace(1.8, 6.2, 1000):
        s = S.Structure(np.array([[vac, vac, vac], [vac + d, vac, vac]]),
                        np.diag([2 * vac + d + 6.2, 2 * vac, 2 * vac]), np.array([False] * 3),
                        np.array([14, 14], dtype=np.int32))
        o = energy(kind, s, PARAMS[kind])
        e.append(o["epot"])
        f.append(o["f"][0, 0])
    assert np.max(np.abs(np.diff(e))) < 0.08
    assert np.max(np.abs(np.diff(f))) < 0.4
