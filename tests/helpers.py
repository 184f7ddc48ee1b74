"""Shared helpers of the test-suite: run the GPU path and the oracle on the
same structure and compare."""

import numpy as np

from atomistica_gb300 import parameters as P
from atomistica_gb300 import structures as S

TERSOFF = P.Tersoff_PRB_39_5566_Si_C
KUMAGAI = P.Kumagai_CompMaterSci_39_457_Si
TERSOFF_SCR = P.Tersoff_PRB_39_5566_Si_C__Scr
KUMAGAI_SCR = P.Kumagai_CompMaterSci_39_457_Si__Scr

# Tolerances of the FP64 drop-in against the FP64 oracle (per atom energy,
# force and virial components), and of the mixed form's forces.
E_TOL = 1e-10      # eV/atom
F_TOL = 1e-9       # eV/A
W_TOL = 1e-9       # eV per atom of virial magnitude (scaled by nat below)
MIXED_F_TOL = 1e-5  # eV/A


def gpu_bop(kind, s, precision="fp64", params=None, mask=None, per_at=True, per_bond=False,
            repeat=1):
    from atomistica_gb300 import native
    p = native.from_atoms(s)
    nl = native.Neighbors(100)
    cls = {"tersoff": native.Tersoff, "kumagai": native.Kumagai,
           "tersoff_scr": native.TersoffScr, "kumagai_scr": native.KumagaiScr,
           "brenner": native.Brenner, "brenner_scr": native.BrennerScr,
           "juslin": native.Juslin, "juslin_scr": native.JuslinScr}[kind]
    pot = cls(precision=precision, **(params or {}))
    pot.bind_to(p, nl)
    out = None
    for _ in range(repeat):
        kw = dict(mask=mask)
        if per_at:
            kw.update(epot_per_at=True, wpot_per_at=True)
        if per_bond:
            kw.update(epot_per_bond=True, f_per_bond=True, wpot_per_bond=True)
        res = pot.energy_and_forces(p, nl, **kw)
        out = {"epot": res[0], "f": res[1], "wpot": res[2]}
        k = 3
        if per_at:
            out["epot_per_at"] = res[k]
            out["wpot_per_at"] = res[k + 1] if not per_bond else res[k + 3]
            if per_bond:
                out["epot_per_bond"] = res[k + 1]
                out["f_per_bond"] = res[k + 2]
                out["wpot_per_bond"] = res[k + 4]
        elif per_bond:
            out["epot_per_bond"], out["f_per_bond"], out["wpot_per_bond"] = res[k:k + 3]
    out["nl"] = nl.get_list(p)
    out["timing"] = pot.last_timing()
    return out


def gpu_eam(fn, s, mask=None, per_at=True):
    from atomistica_gb300 import native
    p = native.from_atoms(s)
    nl = native.Neighbors(100)
    pot = native.TabulatedAlloyEAM(fn)
    pot.bind_to(p, nl)
    kw = dict(mask=mask)
    if per_at:
        kw.update(epot_per_at=True, wpot_per_at=True)
    res = pot.energy_and_forces(p, nl, **kw)
    out = {"epot": res[0], "f": res[1], "wpot": res[2]}
    if per_at:
        out["epot_per_at"], out["wpot_per_at"] = res[3], res[4]
    out["nl"] = nl.get_list(p)
    return out


def compare(ref, got, nat, etol=E_TOL, ftol=F_TOL, wtol=W_TOL, per_at=True):
    """Max deviations; asserts they are within tolerance."""
    de = abs(ref["epot"] - got["epot"]) / max(nat, 1)
    df = float(np.max(np.abs(ref["f"] - got["f"]))) if nat else 0.0
    dw = float(np.max(np.abs(ref["wpot"] - got["wpot"])))
    wscale = max(1.0, nat)
    assert de < etol, "energy per atom differs by %g" % de
    assert df < ftol, "forces differ by %g" % df
    assert dw < wtol * wscale, "virial differs by %g" % dw
    if per_at and "epot_per_at" in got and nat:
        assert np.max(np.abs(ref["epot_per_at"] - got["epot_per_at"])) < etol * 10
        assert np.max(np.abs(ref["wpot_per_at"] - got["wpot_per_at"])) < wtol * 10
    return de, df, dw


def rattled_diamond(symbol="Si", a=5.431, size=(2, 2, 2), amp=0.3, seed=0):
    rng = np.random.default_rng(seed)
    s = S.diamond(symbol, a, size)
    s.positions += rng.uniform(-amp, amp, s.positions.shape)
    return s


def random_carbon(nat=128, density=3.0, seed=0, dmin=1.2):
    """Amorphous-carbon-like random packing (a stand-in for aC.cfg)."""
    rng = np.random.default_rng(seed)
    mass = 12.011
    L = (nat * mass / (density * 6.02214076e23) * 1e24) ** (1.0 / 3.0)
    cell = np.eye(3) * L
    pos = S._random_packing(rng, nat, cell, dmin)
    return S.Structure(pos, cell, np.array([True, True, True]),
                       np.full(nat, 6, dtype=np.int32))


def random_wch(nat=96, seed=0, frac=(0.4, 0.35, 0.25), density=3.0, dmin=1.1):
    return S.random_wch(nat, seed=seed, frac=frac, density=density, dmin=dmin)


def triclinic_si(nat=24, seed=0, strain=0.08, dmin=2.0):
    rng = np.random.default_rng(seed)
    n = S.si_number_density()
    L = (nat / n) ** (1.0 / 3.0)
    eps = rng.uniform(-strain, strain, size=(3, 3))
    cell = (np.eye(3) * L) @ (np.eye(3) + eps).T
    pos = S._random_packing(rng, nat, cell, dmin)
    return S.Structure(pos, cell, np.array([True, True, True]),
                       np.full(nat, 14, dtype=np.int32))


def sorted_triples(seed, j, dc):
    i = np.repeat(np.arange(len(seed) - 1), np.diff(seed))
    t = np.column_stack([i, j, dc]).astype(np.int64)
    return t[np.lexsort(t.T[::-1])]


def ghost_system(s, cutoff):
    """(r_all, Z_all, owner, seed, nbr): local atoms first, then the images
    within 2 cutoff of the (orthorhombic) box; CSR list within cutoff over
    all atoms, brute force in chunks."""
    L = np.diag(s.cell)
    assert np.allclose(s.cell, np.diag(L))
    w = 2.0 * cutoff
    r = s.positions % L
    rs, own = [r], [np.arange(len(r))]
    m = int(np.ceil(w / L.min()))
    for n in np.ndindex(2 * m + 1, 2 * m + 1, 2 * m + 1):
        n = np.array(n) - m
        if not n.any():
            continue
        img = r + n * L
        keep = np.all((img > -w) & (img < L + w), axis=1)
        rs.append(img[keep])
        own.append(np.nonzero(keep)[0])
    r_all = np.concatenate(rs)
    owner = np.concatenate(own)
    nat = len(r_all)
    seed = np.zeros(nat + 1, dtype=np.int32)
    nbrs = []
    for a in range(0, nat, 512):
        d = r_all[a:a + 512, None, :] - r_all[None, :, :]
        d2 = np.einsum("ijk,ijk->ij", d, d)
        for q in range(d2.shape[0]):
            js = np.nonzero((d2[q] < cutoff * cutoff) & (np.arange(nat) != a + q))[0]
            nbrs.append(js.astype(np.int32))
            seed[a + q + 1] = seed[a + q] + len(js)
    Z = np.asarray(s.numbers, dtype=np.int32)[owner]
    return r_all, Z, owner, seed, np.concatenate(nbrs) if nbrs else np.zeros(0, np.int32)


def fold(owner, x, n):
    out = np.zeros((n,) + x.shape[1:])
    np.add.at(out, owner, x)
    return out
