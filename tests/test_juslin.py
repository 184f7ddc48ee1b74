"""Juslin-form bond-order potential and its screened variant on the GPU
against the FP64 oracle: the W-C-H set on rattled W and W-C crystals and on
random W-C-H packings (every ordered pair and triplet type, so the per-triplet
h = omega exp(alpha dr) with alpha = 4 and omega != 1 is exercised); the
Kuopanportti Fe-C-H set; masks and per-bond outputs; the mixed form;
JuslinScr with the front-end's and the compiled-in screened sets; the
compiled-in default set; batches and the ghost-atom contract."""

import numpy as np
import pytest

import oracle
from atomistica_gb300 import parameters as P
from atomistica_gb300 import structures as S

from helpers import MIXED_F_TOL, compare, fold, ghost_system, gpu_bop, random_carbon, \
    random_wch

pytestmark = pytest.mark.gpu

WCH = P.Juslin_JAP_98_123520_WCH
WCH_SCR = P.Juslin_JAP_98_123520_WCH__Scr
FECH = P.Kuopanportti_CMS_111_525_FeCH
FECH_SCR = P.Kuopanportti_CMS_111_525_FeCH__Scr

# The compiled-in non-screened set differs from the front-end's dictionary in
# the W-H cutoff (juslin_params.f90:105-106).
WCH_COMPILED = dict(WCH, r1=[3.20, 2.60, 1.95, 0.0, 1.70, 1.30, 0.0, 1.30, 1.10],
                    r2=[3.80, 3.00, 2.35, 0.0, 2.00, 1.80, 0.0, 1.80, 1.70])


def _rattled(s, seed, amp):
    s.positions += np.random.default_rng(seed).uniform(-amp, amp, s.positions.shape)
    return s


def _hydrocarbon(seed):
    s = random_carbon(96, density=2.0, seed=seed, dmin=1.0)
    s.numbers[np.random.default_rng(seed + 1).random(len(s)) < 0.4] = 1
    return s


def _fech(seed):
    s = random_wch(96, seed=seed)
    s.numbers[s.numbers == 74] = 26
    return s


def _cases():
    slab = _rattled(S.bcc("W", 3.165, (3, 3, 4)), 101, 0.1)
    slab.pbc = np.array([True, True, False])
    return [
        ("bcc-W", WCH, _rattled(S.bcc("W", 3.165, (3, 3, 3)), 102, 0.15)),
        ("B1-WC", WCH, _rattled(S.b1(("W", "C"), 4.38, (2, 2, 2)), 103, 0.15)),
        ("B2-WC", WCH, _rattled(S.b2(("W", "C"), 2.704, (3, 3, 3)), 104, 0.1)),
        ("B3-WC", WCH, _rattled(S.b3(("W", "C"), 4.679, (2, 2, 2)), 105, 0.2)),
        ("W-C-H a", WCH, random_wch(128, seed=106)),
        ("W-C-H b", WCH, random_wch(96, seed=107, frac=(0.2, 0.4, 0.4))),
        ("C-H", WCH, _hydrocarbon(108)),
        ("W slab", WCH, slab),
        ("Fe-C-H", FECH, _fech(109)),
    ]


@pytest.mark.parametrize("case", _cases(), ids=lambda c: c[0])
def test_juslin_matches_oracle(gpu, case):
    name, params, s = case
    ref = oracle.bop("juslin", params, s)
    got = gpu_bop("juslin", s, params=params)
    compare(ref, got, len(s))


def test_juslin_mask_and_per_bond(gpu):
    s = random_wch(96, seed=110)
    mask = np.random.default_rng(111).integers(0, 2, len(s)).astype(bool)
    ref = oracle.bop("juslin", WCH, s, mask=mask, per_bond=True)
    got = gpu_bop("juslin", s, params=WCH, mask=mask, per_bond=True)
    compare(ref, got, len(s))
    seed, j, dc = got["nl"]
    assert np.array_equal(np.asarray(j), ref["nl"].nbr)
    assert np.max(np.abs(got["epot_per_bond"] - ref["epot_per_bond"])) < 1e-10
    assert np.max(np.abs(got["f_per_bond"] - ref["f_per_bond"])) < 1e-9
    assert np.max(np.abs(got["wpot_per_bond"] - ref["wpot_per_bond"])) < 1e-9


@pytest.mark.parametrize("name", ["bcc-W", "W-C-H", "C-H", "Fe-C-H"])
def test_juslin_mixed(gpu, name):
    params = FECH if name == "Fe-C-H" else WCH
    s = {"bcc-W": lambda: _rattled(S.bcc("W", 3.165, (4, 4, 4)), 112, 0.2),
         "W-C-H": lambda: random_wch(256, seed=113),
         "C-H": lambda: _hydrocarbon(114),
         "Fe-C-H": lambda: _fech(115)}[name]()
    ref = oracle.bop("juslin", params, s)
    got = gpu_bop("juslin", s, precision="mixed", params=params)
    assert np.max(np.abs(got["f"] - ref["f"])) < MIXED_F_TOL
    assert abs(got["epot"] - ref["epot"]) / len(s) < 1e-6
    assert np.max(np.abs(got["wpot"] - ref["wpot"])) < 1e-5 * len(s)


@pytest.mark.parametrize("name", ["bcc-W", "W-C-H", "C-H", "Fe-C-H"])
def test_juslin_scr_matches_oracle(gpu, name):
    params = FECH_SCR if name == "Fe-C-H" else WCH_SCR
    s = {"bcc-W": lambda: _rattled(S.bcc("W", 3.165, (3, 3, 3)), 116, 0.15),
         "W-C-H": lambda: random_wch(96, seed=117),
         "C-H": lambda: _hydrocarbon(118),
         "Fe-C-H": lambda: _fech(119)}[name]()
    ref = oracle.bop("juslin_scr", params, s)
    got = gpu_bop("juslin_scr", s, params=params)
    compare(ref, got, len(s))
    assert len(got["nl"][1]) == len(ref["nl"].nbr)


def test_juslin_defaults(gpu):
    # no parameters: the compiled-in W-C-H sets (non-screened and screened)
    # of the reference's Fortran database
    from atomistica_gb300 import native
    s = random_wch(96, seed=120)
    ref = oracle.bop("juslin", WCH_COMPILED, s)
    compare(ref, gpu_bop("juslin", s), len(s))
    ref = oracle.bop("juslin_scr", native._JUSLIN_SCR_DEFAULT, s)
    compare(ref, gpu_bop("juslin_scr", s), len(s))


def test_juslin_batch_and_ghost(gpu):
    from atomistica_gb300 import native
    structs = [random_wch(64, seed=121), _rattled(S.b1(("W", "C"), 4.38, (1, 1, 1)), 122, 0.1),
               _hydrocarbon(123)]
    for precision, ftol in (("fp64", 1e-9), ("mixed", MIXED_F_TOL)):
        b = native.Batch(structs)
        e, f, w = b.energy_and_forces(native.Juslin(precision=precision, **WCH))
        for q, s in enumerate(structs):
            ref = oracle.bop("juslin", WCH, s, per_at=False)
            fq = f[b.offsets[q]:b.offsets[q + 1]]
            assert abs(e[q] - ref["epot"]) / len(s) < (1e-10 if precision == "fp64" else 1e-6)
            assert np.max(np.abs(fq - ref["f"])) < ftol
    s = random_wch(128, seed=124)
    pot = native.Juslin(**WCH)
    r_all, Z, owner, seed, nbr = ghost_system(s, pot.get_cutoff())
    n = len(s)
    epot, fg, wpot = pot.energy_and_forces_ghost(r_all, Z, seed, nbr, n)
    ref = oracle.bop("juslin", WCH, s)
    assert abs(epot - ref["epot"]) / n < 1e-10
    assert np.max(np.abs(fold(owner, fg, n) - ref["f"])) < 1e-9


def test_juslin_deterministic(gpu):
    s = random_wch(128, seed=125)
    for precision in ("fp64", "mixed"):
        a = gpu_bop("juslin", s, precision=precision, params=WCH, repeat=2)
        b = gpu_bop("juslin", s, precision=precision, params=WCH)
        assert np.array_equal(a["f"], b["f"]) and a["epot"] == b["epot"]
