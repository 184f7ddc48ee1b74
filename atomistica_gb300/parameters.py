"""
Parameter sets for the bond-order potentials, in the dictionary format of
Atomistica's Python front-end (src/python/atomistica/parameters.py).

Per-element arrays (beta, n, c, d, h, eta, delta, c1..c5) are indexed by the
element of the centre atom i; pair arrays (A, B, xi, lambda, mu, omega, mubo,
m, lambda1, lambda2, alpha, r1, r2) use the symmetric pair index of
src/macros.inc:123 (``pair_index`` below, 0-based).

The numerical values are those of the original publications as tabulated in
src/potentials/bop/tersoff/tersoff_params.f90:99-142 and
src/potentials/bop/kumagai/kumagai_params.f90:97-132.
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
