"""Screened Tersoff / Kumagai (TersoffScr, KumagaiScr) on the GPU against the
FP64 oracle: energies, forces, virials, per-atom and per-bond outputs and
masks on crystals, rattled crystals (partially screened bonds) and random
carbon, plus the API rules of the screened variants."""

import numpy as np
import pytest

import oracle
from atomistica_gb300 import structures as S

from helpers import (KUMAGAI_SCR, TERSOFF_SCR, compare, gpu_bop, random_carbon,
                     rattled_diamond)

pytestmark = pytest.mark.gpu


def _cases():
    sic = S.b3(("Si", "C"), 4.3596, (2, 2, 2))
    sic.positions += np.random.default_rng(13).uniform(-0.3, 0.3, sic.positions.shape)
    slab = rattled_diamond("Si", 5.431, (2, 2, 3), 0.2, 14)
    slab.pbc = np.array([True, True, False])
    return [
        ("dia-Si", "tersoff_scr", TERSOFF_SCR, S.diamond("Si", 5.432, (2, 2, 2))),
        ("rattled Si", "tersoff_scr", TERSOFF_SCR, rattled_diamond("Si", 5.431, (2, 2, 2), 0.5, 11)),
        ("rattled C", "tersoff_scr", TERSOFF_SCR, rattled_diamond("C", 3.566, (2, 2, 2), 0.3, 12)),
        ("a-C", "tersoff_scr", TERSOFF_SCR, random_carbon(128, seed=15)),
        ("B3-SiC", "tersoff_scr", TERSOFF_SCR, sic),
        ("Si slab", "tersoff_scr", TERSOFF_SCR, slab),
        ("kumagai Si", "kumagai_scr", KUMAGAI_SCR, rattled_diamond("Si", 5.429, (2, 2, 2), 0.4, 16)),
    ]


@pytest.mark.parametrize("case", _cases(), ids=lambda c: c[0])
def test_screened_matches_oracle(gpu, case):
    name, kind, params, s = case
    ref = oracle.bop(kind, params, s)
    got = gpu_bop(kind, s)
    compare(ref, got, len(s))
    # same neighbour list entries (the screened range)
    seed, j, dc = got["nl"]
    assert len(j) == len(ref["nl"].nbr)


def test_screened_per_bond_and_mask(gpu):
    s = random_carbon(96, seed=17)
    mask = np.random.default_rng(18).integers(0, 2, len(s)).astype(bool)
    ref = oracle.bop("tersoff_scr", TERSOFF_SCR, s, mask=mask, per_bond=True)
    got = gpu_bop("tersoff_scr", s, mask=mask, per_bond=True)
    compare(ref, got, len(s))
    # per-bond outputs in list order; the GPU list equals the oracle's
    seed, j, dc = got["nl"]
    assert np.array_equal(np.asarray(j), ref["nl"].nbr)
    assert np.max(np.abs(got["epot_per_bond"] - ref["epot_per_bond"])) < 1e-10
    assert np.max(np.abs(got["f_per_bond"] - ref["f_per_bond"])) < 1e-9
    assert np.max(np.abs(got["wpot_per_bond"] - ref["wpot_per_bond"])) < 1e-9


def test_screened_deterministic(gpu):
    s = random_carbon(128, seed=19)
    a = gpu_bop("tersoff_scr", s, repeat=2)
    b = gpu_bop("tersoff_scr", s)
    assert np.array_equal(a["f"], b["f"]) and a["epot"] == b["epot"]


def test_screened_api_rules(gpu):
    from atomistica_gb300 import native
    from atomistica_gb300._lib import AtomisticaError
    pot = native.TersoffScr()
    assert abs(pot.get_cutoff() - np.sqrt(9 / 8) * 6.0) < 1e-12
    with pytest.raises(AtomisticaError):
        pot.set_precision("mixed")
    b = native.Batch(S.si_batch(4, seed=3))
    with pytest.raises(AtomisticaError):
        b.energy_and_forces(native.KumagaiScr())
