"""
Parameter sets for the bond-order potentials, in the dictionary format of
Atomistica's Python front-end (src/python/atomistica/parameters.py).

Per-element arrays (beta, n, c, d, h, eta, delta, c1..c5) are indexed by the
element of the centre atom i; pair arrays (A, B, xi, lambda, mu, omega, mubo,
m, lambda1, lambda2, alpha, r1, r2) use the symmetric pair index of
src/macros.inc:123 (``pair_index`` below, 0-based).

The numerical values are those of the original publications as tabulated in
src/potentials/bop/tersoff/tersoff_params.f90:99-142,
src/potentials/bop/kumagai/kumagai_params.f90:97-132 and
src/potentials/bop/brenner/brenner_params.f90:67-200 (Brenner-form sets,
whose arrays are all per element pair) and
src/potentials/bop/juslin/juslin_params.f90:75-145 (Juslin-form sets, arrays
per ordered element pair and per element triplet).
"""

from math import log, sqrt


def pair_index(i, j, maxval):
    """Symmetric 0-based pair index (src/macros.inc:123,
    src/python/atomistica/parameters.py:33-34)."""
    return min(i + j * maxval, j + i * maxval) - min(i * (i + 1) // 2, j * (j + 1) // 2)


# Tersoff, Phys. Rev. B 39, 5566 (1989); Si-C with geometric/arithmetic mixing.
Tersoff_PRB_39_5566_Si_C = {
    "__ref__": "Tersoff J., Phys. Rev. B 39, 5566 (1989)",
    "el": ["C", "Si"],
    "A": [1.3936e3, sqrt(1.3936e3 * 1.8308e3), 1.8308e3],
    "B": [3.4674e2, sqrt(3.4674e2 * 4.7118e2), 4.7118e2],
    "xi": [1.0, 0.9776e0, 1.0],
    "lambda": [3.4879e0, (3.4879e0 + 2.4799e0) / 2, 2.4799e0],
    "mu": [2.2119e0, (2.2119e0 + 1.7322e0) / 2, 1.7322e0],
    "omega": [1.0, 1.0, 1.0],
    "mubo": [0.0, 0.0, 0.0],
    "m": [1, 1, 1],
    "beta": [1.5724e-7, 1.1000e-6],
    "n": [7.2751e-1, 7.8734e-1],
    "c": [3.8049e4, 1.0039e5],
    "d": [4.3484e0, 1.6217e1],
    "h": [-5.7058e-1, -5.9825e-1],
    "r1": [1.80, sqrt(1.80 * 2.70), 2.70],
    "r2": [2.10, sqrt(2.10 * 3.00), 3.00],
}

# Kumagai, Izumi, Hara, Sakai, Comp. Mater. Sci. 39, 457 (2007); Si.
Kumagai_CompMaterSci_39_457_Si = {
    "__ref__": "Kumagai T., Izumi S., Hara S., Sakai S., Comp. Mater. Sci. 39, 457 (2007)",
    "el": ["Si"],
    "A": [3281.5905],
    "B": [121.00047],
    "lambda1": [3.2300135],
    "lambda2": [1.3457970],
    "eta": [1.0000000],
    "delta": [0.53298909],
    "alpha": [2.3890327],
    "beta": [1],
    "c1": [0.20173476],
    "c2": [730418.72],
    "c3": [1000000.0],
    "c4": [1.0000000],
    "c5": [26.000000],
    "h": [-0.36500000],
    "r1": [2.70],
    "r2": [3.30],
}

# Screened variants (TersoffScr / KumagaiScr; Pastewka et al., PRB 87, 205410
# (2013)): inner cutoff r1 < r2 without screening, outer (VA, VR) cutoff
# or1 < or2 and bond-order cutoff bor1 < bor2 with the screening window
# Cmin < C < Cmax (tersoff_params.f90:114-135, kumagai_params.f90:119-128
# under SCREENING; src/python/atomistica/parameters.py:79-107, 409-420).
# mubo is the inverse dimer length (lambda - mu) / ln(lambda A / (mu B)).
Tersoff_PRB_39_5566_Si_C__Scr = dict(
    Tersoff_PRB_39_5566_Si_C,
    m=[3, 3, 3],
    r1=[2.00, sqrt(2.00 * 2.50), 2.50],
    r2=[2.00 * 1.2, sqrt(2.00 * 2.50) * 1.2, 2.50 * 1.2],
    or1=[2.00, sqrt(2.00 * 3.00), 3.00],
    or2=[2.00 * 2.0, sqrt(2.00 * 3.00) * 2.0, 3.00 * 2.0],
    bor1=[2.00, sqrt(2.00 * 3.00), 3.00],
    bor2=[2.00 * 2.0, sqrt(2.00 * 3.00) * 2.0, 3.00 * 2.0],
    Cmin=[1.00, 1.00, 1.00],
    Cmax=[3.00, 3.00, 3.00],
)
Tersoff_PRB_39_5566_Si_C__Scr["mubo"] = [
    (Tersoff_PRB_39_5566_Si_C__Scr["lambda"][q] - Tersoff_PRB_39_5566_Si_C__Scr["mu"][q]) /
    log(Tersoff_PRB_39_5566_Si_C__Scr["lambda"][q] * Tersoff_PRB_39_5566_Si_C__Scr["A"][q] /
        (Tersoff_PRB_39_5566_Si_C__Scr["mu"][q] * Tersoff_PRB_39_5566_Si_C__Scr["B"][q]))
    for q in range(3)]

Kumagai_CompMaterSci_39_457_Si__Scr = dict(
    Kumagai_CompMaterSci_39_457_Si,
    r1=[2.50], r2=[2.50 * 1.2],
    or1=[3.00], or2=[3.00 * 2.0],
    bor1=[3.00], bor2=[3.00 * 2.0],
    Cmin=[1.00], Cmax=[3.00],
)

SCREENING_KEYS = ("or1", "or2", "bor1", "bor2", "Cmin", "Cmax")

# Brenner-form (Albe-Erhart) bond-order sets for the *Brenner* potential
# (src/potentials/bop/brenner/brenner_params.f90:67-200,
# src/python/atomistica/parameters.py:174-276, 346-380).  Every array is per
# symmetric element pair: VR = D0/(S-1) exp(-beta sqrt(2S) (r-r0)),
# VA = -S D0/(S-1) exp(-beta sqrt(2/S) (r-r0)),
# g = gamma (1 + c^2/d^2 - c^2/(d^2 + (h + cos)^2)) of the (i,k) pair,
# b = (1 + zeta^n)^(-1/(2n)), h(dr) = exp((2 mu dr)^m).
BRENNER_KEYS = ("D0", "r0", "S", "beta", "gamma", "c", "d", "h", "mu", "n", "m", "r1", "r2")

Erhart_PRB_71_035211_SiC = {
    "__ref__": "Erhart P., Albe K., Phys. Rev. B 71, 035211 (2005)",
    "el": ["C", "Si"],
    "D0": [6.00, 4.36, 3.24],
    "r0": [1.4276, 1.79, 2.232],
    "S": [2.167, 1.847, 1.842],
    "beta": [2.0099, 1.6991, 1.4761],
    "gamma": [0.11233, 0.011877, 0.114354],
    "c": [181.910, 273987.0, 2.00494],
    "d": [6.28433, 180.314, 0.81472],
    "h": [0.5556, 0.68, 0.259],
    "mu": [0.0, 0.0, 0.0],
    "n": [1.0, 1.0, 1.0],
    "m": [1, 1, 1],
    "r1": [1.85, 2.20, 2.68],
    "r2": [2.15, 2.60, 2.96],
}

# Screened form of the same set (BrennerScr), as the reference's Python
# front-end tabulates it (parameters.py:196-218).
Erhart_PRB_71_035211_SiC__Scr = dict(
    Erhart_PRB_71_035211_SiC,
    mu=[1.0 / 1.4276, 1.0 / 1.79, 1.0 / 1.842],
    m=[3, 3, 3],
    r1=[2.00, 2.40, 2.50],
    r2=[2.00 * 1.2, 2.40 * 1.2, 2.50 * 1.2],
    or1=[2.00, 2.40, 3.00],
    or2=[2.00 * 2.0, 2.40 * 2.0, 3.00 * 2.0],
    bor1=[2.00, 2.40, 3.00],
    bor2=[2.00 * 2.0, 2.40 * 2.0, 3.00 * 2.0],
    Cmin=[1.00, 1.00, 1.00],
    Cmax=[3.00, 3.00, 3.00],
)

Albe_PRB_65_195124_PtC = {
    "__ref__": "Albe K., Nordlund K., Averback R. S., Phys. Rev. B 65, 195124 (2002)",
    "el": ["Pt", "C"],
    "D0": [3.683, 5.3, 6.0],
    "r0": [2.384, 1.84, 1.39],
    "S": [2.24297, 1.1965, 1.22],
    "beta": [1.64249, 1.836, 2.1],
    "gamma": [8.542e-4, 9.7e-3, 2.0813e-4],
    "c": [34.0, 1.23, 330.0],
    "d": [1.1, 0.36, 3.5],
    "h": [1.0, 1.0, 1.0],
    "mu": [1.335, 0.0, 0.0],
    "n": [1.0, 1.0, 1.0],
    "m": [1, 1, 1],
    "r1": [2.9, 2.5, 1.7],
    "r2": [3.3, 2.8, 2.0],
}

Henriksson_PRB_79_114107_FeC = {
    "__ref__": "Henriksson K.O.E., Nordlund K., Phys. Rev. B 79, 144107 (2009)",
    "el": ["Fe", "C"],
    "D0": [1.5, 4.82645134, 6.0],
    "r0": [2.29, 1.47736510, 1.39],
    "S": [2.0693109, 1.43134755, 1.22],
    "beta": [1.4, 1.63208170, 2.1],
    "gamma": [0.0115751, 0.00205862, 0.00020813],
    "c": [1.2898716, 8.95583221, 330.0],
    "d": [0.3413219, 0.72062047, 3.5],
    "h": [-0.26, 0.87099874, 1.0],
    "mu": [0.0, 0.0, 0.0],
    "n": [1.0, 1.0, 1.0],
    "m": [1, 1, 1],
    "r1": [2.95, 2.3, 1.70],
    "r2": [3.35, 2.7, 2.00],
}

Kioseoglou_PSSb_245_1118_AlN = {
    "__ref__": "Kioseoglou J., Komninou Ph., Karakostas Th., Phys. Stat. Sol. (b) 245, 1118 "
               "(2008)",
    "el": ["N", "Al"],
    "D0": [9.9100, 3.3407, 1.5000],
    "r0": [1.1100, 1.8616, 2.4660],
    "S": [1.4922, 1.7269, 2.7876],
    "beta": [2.05945, 1.7219, 1.0949],
    "gamma": [0.76612, 1.1e-6, 0.3168],
    "c": [0.178493, 100390, 0.0748],
    "d": [0.20172, 16.2170, 19.5691],
    "h": [0.045238, 0.5980, 0.6593],
    "mu": [0.0, 0.0, 0.0],
    "n": [1.0, 0.7200, 6.0865],
    "m": [1, 1, 1],
    "r1": [2.00, 2.19, 3.40],
    "r2": [2.40, 2.49, 3.60],
}

# Brenner's carbon potentials I and II without the correction tables
# (Brenner, Phys. Rev. B 42, 9458 (1990); parameters.py:346-380).
Brenner_PRB_42_9458_C_I = {
    "__ref__": "Brenner D., Phys. Rev. B 42, 9458 (1990) [potential I]",
    "el": ["C"],
    "D0": [6.325], "r0": [1.315], "S": [1.29], "beta": [1.5], "gamma": [0.011304],
    "c": [19.0], "d": [2.5], "h": [1.0], "mu": [0.0], "n": [1.0 / (2 * 0.80469)], "m": [1],
    "r1": [1.70], "r2": [2.00],
}

Brenner_PRB_42_9458_C_II = {
    "__ref__": "Brenner D., Phys. Rev. B 42, 9458 (1990) [potential II]",
    "el": ["C"],
    "D0": [6.0], "r0": [1.39], "S": [1.22], "beta": [2.1], "gamma": [0.00020813],
    "c": [330.0], "d": [3.5], "h": [1.0], "mu": [0.0], "n": [1.0 / (2 * 0.5)], "m": [1],
    "r1": [1.70], "r2": [2.00],
}

# Juslin-form sets (src/potentials/bop/juslin/): the Brenner functions with
# every pair array per ORDERED element pair, entry j + i*nel (src/macros.inc:139;
# an entry with r0 < 0 takes the constants of its mirror pair), and h(dr) =
# omega exp((alpha dr)^m) with alpha, omega, m per element triplet, entry
# k + nel*(j + nel*i) (src/macros.inc:146).  m defaults to 1.
JUSLIN_KEYS = ("D0", "r0", "S", "beta", "gamma", "c", "d", "h", "n", "r1", "r2")
JUSLIN_TRIPLET_KEYS = ("alpha", "omega", "m")

_JUSLIN_ALPHA_H = [0.0] * 14 + [4.0, 0.0, 4.0, 4.0, 0.0, 0.0, 0.0, 0.0, 4.0, 4.0, 0.0, 4.0, 4.0]
_JUSLIN_OMEGA = [1.0] * 16 + [2.94586, 4.54415, 1.0, 1.0, 1.0, 1.0, 0.33946, 0.22006,
                              1.0, 1.0, 1.0]

# Juslin et al., J. Appl. Phys. 98, 123520 (2005); W-C-H
# (juslin_params.f90:75-108, parameters.py:278-295).
Juslin_JAP_98_123520_WCH = {
    "__ref__": "Juslin N., Erhart P., Traskelin P., Nord J., Henriksson K.O.E, Nordlund K., "
               "Salonen E., Albe K., J. Appl. Phys. 98, 123520 (2005)",
    "el": ["W", "C", "H"],
    "D0": [5.41861, 6.64, 2.748, 0.0, 6.0, 3.6422, 0.0, 3.642, 4.7509],
    "r0": [2.34095, 1.90547, 1.727, -1.0, 1.39, 1.1199, -1.0, 1.1199, 0.74144],
    "S": [1.92708, 2.96149, 1.2489, 0.0, 1.22, 1.69077, 0.0, 1.69077, 2.3432],
    "beta": [1.38528, 1.80370, 1.52328, 0.0, 2.1, 1.9583, 0.0, 1.9583, 1.9436],
    "gamma": [0.00188227, 0.072855, 0.0054, 0.0, 0.00020813, 0.00020813, 0.0, 12.33, 12.33],
    "c": [2.14969, 1.10304, 1.788, 0.0, 330.0, 330.0, 0.0, 0.0, 0.0],
    "d": [0.17126, 0.33018, 0.8255, 0.0, 3.5, 3.5, 0.0, 1.0, 1.0],
    "h": [-0.27780, 0.75107, 0.38912, 0.0, 1.0, 1.0, 0.0, 1.0, 1.0],
    "n": [1.0, 1.0, 1.0, 0.0, 1.0, 1.0, 0.0, 1.0, 1.0],
    "alpha": [0.45876, 0.0, 0.0, 0.45876, 0.0, 0.0, 0.45876] + _JUSLIN_ALPHA_H[7:],
    "omega": list(_JUSLIN_OMEGA),
    "r1": [3.20, 2.60, 2.68, 0.0, 1.70, 1.30, 0.0, 1.30, 1.10],
    "r2": [3.80, 3.00, 2.96, 0.0, 2.00, 1.80, 0.0, 1.80, 1.70],
}

# The screened set of the Python front-end (parameters.py:297-309): the outer
# and bond-order cutoffs equal the inner ones, and Cmin / Cmax are set to the
# r1 / r2 values as the reference tabulates them.
Juslin_JAP_98_123520_WCH__Scr = dict(
    Juslin_JAP_98_123520_WCH,
    or1=list(Juslin_JAP_98_123520_WCH["r1"]), or2=list(Juslin_JAP_98_123520_WCH["r2"]),
    bor1=list(Juslin_JAP_98_123520_WCH["r1"]), bor2=list(Juslin_JAP_98_123520_WCH["r2"]),
    Cmin=list(Juslin_JAP_98_123520_WCH["r1"]), Cmax=list(Juslin_JAP_98_123520_WCH["r2"]),
    m=[1] * 27,
)

# Kuopanportti et al., Comp. Mat. Sci. 111, 525 (2016); Fe-C-H
# (parameters.py:313-327).
Kuopanportti_CMS_111_525_FeCH = {
    "__ref__": "Kuopanportti P., Hayward, N., Fu C., Kuronen A., Nordlund K., "
               "Comp. Mat. Sci. 111, 525 (2016)",
    "el": ["Fe", "C", "H"],
    "D0": [1.5, 4.82645134, 1.630, 0.0, 6.0, 3.6422, 0.0, 3.642, 4.7509],
    "r0": [2.29, 1.47736510, 1.589, -1.0, 1.39, 1.1199, -1.0, 1.1199, 0.74144],
    "S": [2.0693, 1.43134755, 4.000, 0.0, 1.22, 1.69077, 0.0, 1.69077, 2.3432],
    "beta": [1.4, 1.63208170, 1.875, 0.0, 2.1, 1.9583, 0.0, 1.9583, 1.9436],
    "gamma": [0.01158, 0.00205862, 0.01332, 0.0, 0.00020813, 0.00020813, 0.0, 12.33, 12.33],
    "c": [1.2899, 8.95583221, 424.5, 0.0, 330.0, 330.0, 0.0, 0.0, 0.0],
    "d": [0.3413, 0.72062047, 7.282, 0.0, 3.5, 3.5, 0.0, 1.0, 1.0],
    "h": [-0.26, 0.87099874, -0.1091, 0.0, 1.0, 1.0, 0.0, 1.0, 1.0],
    "n": [1.0, 1.0, 1.0, 0.0, 1.0, 1.0, 0.0, 1.0, 1.0],
    "alpha": list(_JUSLIN_ALPHA_H),
    "omega": list(_JUSLIN_OMEGA),
    "r1": [2.95, 2.30, 2.2974, 0.0, 1.70, 1.30, 0.0, 1.30, 1.10],
    "r2": [3.35, 2.70, 2.6966, 0.0, 2.00, 1.80, 0.0, 1.80, 1.70],
}

# parameters.py:330-342
Kuopanportti_CMS_111_525_FeCH__Scr = dict(
    Kuopanportti_CMS_111_525_FeCH,
    or1=list(Kuopanportti_CMS_111_525_FeCH["r1"]), or2=list(Kuopanportti_CMS_111_525_FeCH["r2"]),
    bor1=list(Kuopanportti_CMS_111_525_FeCH["r1"]),
    bor2=list(Kuopanportti_CMS_111_525_FeCH["r2"]),
    Cmin=[1.0, 1.0, 1.0, 0.0, 1.0, 1.0, 0.0, 1.0, 1.0],
    Cmax=[3.0, 3.0, 3.0, 0.0, 3.0, 3.0, 0.0, 3.0, 3.0],
    m=[1] * 27,
)

# The 14 continuous Tersoff parameters of a single-element set, in the order
# used by the parameter-gradient interface.
TERSOFF_FIT_KEYS = ("A", "B", "lambda", "mu", "beta", "n", "c", "d", "h",
                    "r1", "r2", "xi", "omega", "mubo")

_SYMBOLS = [
    "X", "H", "He", "Li", "Be", "B", "C", "N", "O", "F", "Ne", "Na", "Mg", "Al",
    "Si", "P", "S", "Cl", "Ar", "K", "Ca", "Sc", "Ti", "V", "Cr", "Mn", "Fe", "Co",
    "Ni", "Cu", "Zn", "Ga", "Ge", "As", "Se", "Br", "Kr", "Rb", "Sr", "Y", "Zr",
    "Nb", "Mo", "Tc", "Ru", "Rh", "Pd", "Ag", "Cd", "In", "Sn", "Sb", "Te", "I",
    "Xe", "Cs", "Ba", "La", "Ce", "Pr", "Nd", "Pm", "Sm", "Eu", "Gd", "Tb", "Dy",
    "Ho", "Er", "Tm", "Yb", "Lu", "Hf", "Ta", "W", "Re", "Os", "Ir", "Pt", "Au",
    "Hg", "Tl", "Pb", "Bi", "Po", "At", "Rn",
]

atomic_numbers = {s: z for z, s in enumerate(_SYMBOLS) if z > 0}
chemical_symbols = list(_SYMBOLS)


def tersoff_single_element(p, symbol):
    """Reduce a multi-element Tersoff set to the single-element set of
    ``symbol`` (its own element and pair entries)."""
    els = p["el"]
    e = els.index(symbol)
    nel = len(els)
    ij = pair_index(e, e, nel)
    q = {"el": [symbol]}
    for k in ("A", "B", "xi", "lambda", "mu", "omega", "mubo", "m", "r1", "r2") + \
            tuple(k for k in SCREENING_KEYS if k in p):
        q[k] = [p[k][ij]]
    for k in ("beta", "n", "c", "d", "h"):
        q[k] = [p[k][e]]
    return q
