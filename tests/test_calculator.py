"""The ASE-style calculators (aseinterface.py:143-450 mirror) on the GPU
against the oracle: energy, forces, Voigt stress wpot/V, per-atom energies
and stresses, and recomputation after the positions change."""

import numpy as np
import pytest

import oracle
from atomistica_gb300 import io as gio

from helpers import (KUMAGAI, KUMAGAI_SCR, TERSOFF, TERSOFF_SCR, random_carbon,
                     rattled_diamond)

pytestmark = pytest.mark.gpu


def _voigt(w):
    return np.array([w[0, 0], w[1, 1], w[2, 2], (w[1, 2] + w[2, 1]) / 2,
                     (w[0, 2] + w[2, 0]) / 2, (w[0, 1] + w[1, 0]) / 2])


@pytest.mark.parametrize("name", ["Tersoff", "Kumagai", "TersoffScr", "KumagaiScr"])
def test_bop_calculators(gpu, name):
    import atomistica_gb300 as ag
    kind, params = {"Tersoff": ("tersoff", TERSOFF), "Kumagai": ("kumagai", KUMAGAI),
                    "TersoffScr": ("tersoff_scr", TERSOFF_SCR),
                    "KumagaiScr": ("kumagai_scr", KUMAGAI_SCR)}[name]
    s = random_carbon(64, seed=31) if name == "Tersoff" else \
        rattled_diamond("Si", 5.431, (2, 2, 2), 0.3, 32)
    calc = getattr(ag, name)()
    ref = oracle.bop(kind, params, s)
    V = abs(np.linalg.det(s.cell))
    assert abs(calc.get_potential_energy(s) - ref["epot"]) < 1e-10 * len(s)
    assert np.max(np.abs(calc.get_forces(s) - ref["f"])) < 1e-9
    assert np.max(np.abs(calc.get_stress(s) - _voigt(ref["wpot"]) / V)) < 1e-9
    assert np.max(np.abs(calc.get_potential_energies(s) - ref["epot_per_at"])) < 1e-9
    st = calc.get_stresses(s)
    w = ref["wpot_per_at"]
    ref_st = np.transpose([w[:, 0, 0], w[:, 1, 1], w[:, 2, 2], (w[:, 1, 2] + w[:, 2, 1]) / 2,
                           (w[:, 0, 2] + w[:, 2, 0]) / 2, (w[:, 0, 1] + w[:, 1, 0]) / 2])
    assert np.max(np.abs(st - ref_st)) < 1e-9
    # moved atoms are recomputed
    t = s.copy()
    t.positions[0] += 0.05
    ref2 = oracle.bop(kind, params, t)
    assert abs(calc.get_potential_energy(t) - ref2["epot"]) < 1e-10 * len(t)
    assert np.max(np.abs(calc.get_forces(t) - ref2["f"])) < 1e-9


def test_eam_calculator(gpu, tmp_path):
    import atomistica_gb300 as ag
    from atomistica_gb300 import structures as S
    fn = gio.cu_analytic_setfl(str(tmp_path / "cu.setfl"), nr=2000, nrho=2000)
    s = S.fcc("Cu", 3.615, (3, 3, 3))
    s.positions += np.random.default_rng(33).normal(0, 0.05, s.positions.shape)
    calc = ag.TabulatedAlloyEAM(fn=fn)
    ref = oracle.EAM(fn).compute(s)
    assert abs(calc.get_potential_energy(s) - ref["epot"]) < 1e-10 * len(s)
    assert np.max(np.abs(calc.get_forces(s) - ref["f"])) < 1e-9
    assert np.max(np.abs(calc.get_stress(s) - _voigt(ref["wpot"]) / s.get_volume())) < 1e-9
