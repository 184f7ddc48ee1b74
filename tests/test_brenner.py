"""Brenner-form (Albe-Erhart) bond-order potential and its screened variant
on the GPU against the FP64 oracle: the Erhart Si-C set on crystals, rattled
crystals and random carbon; Henriksson Fe-C with masks; Kioseoglou Al-N
(n != 1); per-bond outputs; the mixed form; BrennerScr; the compiled-in
default sets; batches and the ghost-atom contract."""

import numpy as np
import pytest

import oracle
from atomistica_gb300 import parameters as P
from atomistica_gb300 import structures as S

from helpers import MIXED_F_TOL, compare, fold, ghost_system, gpu_bop, random_carbon, \
    rattled_diamond

pytestmark = pytest.mark.gpu

ERHART = P.Erhart_PRB_71_035211_SiC
ERHART_SCR = P.Erhart_PRB_71_035211_SiC__Scr
FEC = P.Henriksson_PRB_79_114107_FeC
ALN = P.Kioseoglou_PSSb_245_1118_AlN


def _sic(seed, amp=0.3):
    s = S.b3(("Si", "C"), 4.3596, (2, 2, 2))
    s.positions += np.random.default_rng(seed).uniform(-amp, amp, s.positions.shape)
    return s


def _cases():
    fe = S.b1(("Fe", "C"), 3.9, (2, 2, 2))
    fe.positions += np.random.default_rng(61).uniform(-0.1, 0.1, fe.positions.shape)
    aln = S.b3(("Al", "N"), 4.38, (2, 2, 2))
    aln.positions += np.random.default_rng(62).uniform(-0.2, 0.2, aln.positions.shape)
    slab = rattled_diamond("Si", 5.429, (2, 2, 3), 0.2, 63)
    slab.pbc = np.array([True, True, False])
    return [
        ("dia-C", ERHART, S.diamond("C", 3.566, (2, 2, 2))),
        ("rattled C", ERHART, rattled_diamond("C", 3.566, (2, 2, 2), 0.3, 64)),
        ("rattled Si", ERHART, rattled_diamond("Si", 5.429, (2, 2, 2), 0.4, 65)),
        ("B3-SiC", ERHART, _sic(66)),
        ("a-C", ERHART, random_carbon(128, seed=67)),
        ("Si slab", ERHART, slab),
        ("B1-FeC", FEC, fe),
        ("AlN n!=1", ALN, aln),
        ("brenner II a-C", P.Brenner_PRB_42_9458_C_II, random_carbon(96, seed=68)),
    ]


@pytest.mark.parametrize("case", _cases(), ids=lambda c: c[0])
def test_brenner_matches_oracle(gpu, case):
    name, params, s = case
    ref = oracle.bop("brenner", params, s)
    got = gpu_bop("brenner", s, params=params)
    compare(ref, got, len(s))


def test_brenner_mask_and_per_bond(gpu):
    s = S.bcc("Fe", 2.87, (3, 3, 3))
    s.positions += np.random.default_rng(69).uniform(-0.1, 0.1, s.positions.shape)
    s.numbers[::5] = 6
    mask = np.random.default_rng(70).integers(0, 2, len(s)).astype(bool)
    ref = oracle.bop("brenner", FEC, s, mask=mask, per_bond=True)
    got = gpu_bop("brenner", s, params=FEC, mask=mask, per_bond=True)
    compare(ref, got, len(s))
    seed, j, dc = got["nl"]
    assert np.array_equal(np.asarray(j), ref["nl"].nbr)
    assert np.max(np.abs(got["epot_per_bond"] - ref["epot_per_bond"])) < 1e-10
    assert np.max(np.abs(got["f_per_bond"] - ref["f_per_bond"])) < 1e-9
    assert np.max(np.abs(got["wpot_per_bond"] - ref["wpot_per_bond"])) < 1e-9


@pytest.mark.parametrize("name", ["B3-SiC", "a-C", "AlN"])
def test_brenner_mixed(gpu, name):
    if name == "B3-SiC":
        params, s = ERHART, _sic(71, 0.4)
    elif name == "a-C":
        params, s = ERHART, random_carbon(256, seed=72)
    else:
        params = ALN
        s = S.b3(("Al", "N"), 4.38, (3, 3, 3))
        s.positions += np.random.default_rng(73).uniform(-0.2, 0.2, s.positions.shape)
    ref = oracle.bop("brenner", params, s)
    got = gpu_bop("brenner", s, precision="mixed", params=params)
    assert np.max(np.abs(got["f"] - ref["f"])) < MIXED_F_TOL
    assert abs(got["epot"] - ref["epot"]) / len(s) < 1e-6
    assert np.max(np.abs(got["wpot"] - ref["wpot"])) < 1e-5 * len(s)


@pytest.mark.parametrize("name", ["dia-Si", "rattled C", "a-C", "B3-SiC"])
def test_brenner_scr_matches_oracle(gpu, name):
    s = {"dia-Si": lambda: S.diamond("Si", 5.429, (2, 2, 2)),
         "rattled C": lambda: rattled_diamond("C", 3.566, (2, 2, 2), 0.3, 74),
         "a-C": lambda: random_carbon(128, seed=75),
         "B3-SiC": lambda: _sic(76)}[name]()
    ref = oracle.bop("brenner_scr", ERHART_SCR, s)
    got = gpu_bop("brenner_scr", s, params=ERHART_SCR)
    compare(ref, got, len(s))
    assert len(got["nl"][1]) == len(ref["nl"].nbr)


def test_brenner_defaults(gpu):
    # no parameters: the compiled-in Erhart-Albe sets (non-screened and
    # screened) of the reference's Fortran database
    from atomistica_gb300 import native
    s = _sic(77)
    ref = oracle.bop("brenner", ERHART, s)
    compare(ref, gpu_bop("brenner", s), len(s))
    ref = oracle.bop("brenner_scr", native._BRENNER_SCR_DEFAULT, s)
    compare(ref, gpu_bop("brenner_scr", s), len(s))


def test_brenner_batch_and_ghost(gpu):
    from atomistica_gb300 import native
    structs = [_sic(78), rattled_diamond("C", 3.566, (1, 1, 1), 0.2, 79),
               random_carbon(64, seed=80)]
    b = native.Batch(structs)
    e, f, w = b.energy_and_forces(native.Brenner(**ERHART))
    for q, s in enumerate(structs):
        ref = oracle.bop("brenner", ERHART, s, per_at=False)
        fq = f[b.offsets[q]:b.offsets[q + 1]]
        assert abs(e[q] - ref["epot"]) / len(s) < 1e-10
        assert np.max(np.abs(fq - ref["f"])) < 1e-9
        assert np.max(np.abs(w[q] - ref["wpot"])) < 1e-9 * len(s)
    s = rattled_diamond("C", 3.566, (3, 3, 3), 0.2, 81)
    pot = native.Brenner(**ERHART)
    r_all, Z, owner, seed, nbr = ghost_system(s, pot.get_cutoff())
    n = len(s)
    epot, fg, wpot = pot.energy_and_forces_ghost(r_all, Z, seed, nbr, n)
    ref = oracle.bop("brenner", ERHART, s)
    assert abs(epot - ref["epot"]) / n < 1e-10
    assert np.max(np.abs(fold(owner, fg, n) - ref["f"])) < 1e-9


def test_brenner_deterministic(gpu):
    s = random_carbon(128, seed=82)
    a = gpu_bop("brenner", s, params=ERHART, repeat=2)
    b = gpu_bop("brenner", s, params=ERHART)
    assert np.array_equal(a["f"], b["f"]) and a["epot"] == b["epot"]


def test_brenner_md_matches_host_verlet(gpu):
    # the velocity-Verlet graph (gb_batch_md_*) with Brenner forces against the
    # same integrator on the host with the oracle's forces
    from atomistica_gb300 import native
    structs = [_sic(83, 0.1), rattled_diamond("C", 3.566, (2, 2, 2), 0.05, 84)]
    n = sum(len(s) for s in structs)
    rng = np.random.default_rng(85)
    v = rng.normal(0.0, 0.02, (n, 3))
    m = np.array([28.0855 if z == 14 else 12.011 for s in structs for z in s.numbers])
    b = native.Batch(structs)
    b.md_set_state(v, m)
    b.md_run(native.Brenner(**ERHART), 0.05, 10)
    r, vg, f = b.md_get_state()
    for q, s in enumerate(structs):
        sl = slice(b.offsets[q], b.offsets[q + 1])
        t, vv, mq = s.copy(), v[sl].copy(), m[sl]
        fh = oracle.bop("brenner", ERHART, t, per_at=False)["f"]
        for _ in range(10):
            vv = vv + 0.5 * fh / mq[:, None] * 0.05
            t.positions = t.positions + vv * 0.05
            fh = oracle.bop("brenner", ERHART, t, per_at=False)["f"]
            vv = vv + 0.5 * fh / mq[:, None] * 0.05
        assert np.max(np.abs(r[sl] - t.positions)) < 1e-9
        assert np.max(np.abs(vg[sl] - vv)) < 1e-9
        assert np.max(np.abs(f[sl] - fh)) < 1e-8
