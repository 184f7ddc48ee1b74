"""
Small file readers/writers needed by the force path without ASE:

* ``read_cfg``   — AtomEye extended .cfg (the reference's aC.cfg fixtures).
* ``write_setfl`` / ``cu_analytic_setfl`` — DYNAMO setfl tables in the layout
  read by src/potentials/eam/tabulated_alloy_eam.f90:178-253.
* ``write_funcfl`` / ``cu_analytic_funcfl`` — single-element DYNAMO funcfl
  tables as read by src/potentials/eam/tabulated_eam.f90:147-200.
"""

import numpy as np

from .parameters import atomic_numbers
from .structures import Structure


def read_cfg(fn):
    """Read an AtomEye extended CFG file (scaled coordinates, H0 rows)."""
    with open(fn) as f:
        lines = f.read().splitlines()
    nat = None
    A = 1.0
    H = np.zeros((3, 3))
    entry_count = None
    k = 0
    while k < len(lines):
        ln = lines[k].strip()
        if not ln or ln.startswith("#"):
            k += 1
            continue
        if ln.startswith("Number of particles"):
            nat = int(ln.split("=")[1])
        elif ln.startswith("A ="):
            A = float(ln.split("=")[1].split()[0])
        elif ln.startswith("H0("):
            ij = ln[3:ln.index(")")].split(",")
            H[int(ij[0]) - 1, int(ij[1]) - 1] = float(ln.split("=")[1].split()[0])
        elif ln.startswith("entry_count"):
            entry_count = int(ln.split("=")[1])
        elif ln.startswith(".NO_VELOCITY."):
            pass
        elif ln.startswith("auxiliary") or ln.startswith("R =") or ln.startswith("Transform") \
                or ln.startswith("eta"):
            pass
        else:
            break
        k += 1
    cell = H * A
    frac = []
    numbers = []
    sym = None
    while k < len(lines) and len(frac) < nat:
        toks = lines[k].split()
        k += 1
        if not toks:
            continue
        if len(toks) == 1:
            try:
                float(toks[0])
                continue  # mass line
            except ValueError:
                sym = toks[0]
                continue
        frac.append([float(t) for t in toks[:3]])
        numbers.append(atomic_numbers[sym])
    frac = np.array(frac)
    return Structure(frac @ cell, cell, np.array([True, True, True]),
                     np.array(numbers, dtype=np.int32), {"file": str(fn)})


def write_setfl(fn, elements, nrho, drho, nr, dr, cutoff, F, rho, rphi, comments=None,
                Z=None, mass=None, a0=None, lattice=None):
    """Write a setfl file.  F[e] has nrho values, rho[e] nr values and
    rphi[(i, j)] (i >= j) nr values of r*phi(r)."""
    nel = len(elements)
    comments = list(comments or ["", "", ""])[:3]
    while len(comments) < 3:
        comments.append("")
    with open(fn, "w") as f:
        for c in comments:
            f.write(c + "\n")
        f.write("%d %s\n" % (nel, " ".join(elements)))
        f.write("%d %.17g %d %.17g %.17g\n" % (nrho, drho, nr, dr, cutoff))

        def block(v):
            v = np.asarray(v, dtype=float)
            for q in range(0, len(v), 5):
                f.write(" ".join("%.17g" % x for x in v[q:q + 5]) + "\n")

        for e, el in enumerate(elements):
            z = Z[e] if Z else atomic_numbers[el]
            m = mass[e] if mass else 0.0
            a = a0[e] if a0 else 0.0
            lat = lattice[e] if lattice else "fcc"
            f.write("%d %.17g %.17g %s\n" % (z, m, a, lat))
            block(F[e])
            block(rho[e])
        for i in range(nel):
            for j in range(i + 1):
                block(rphi[(i, j)])


def cu_analytic_setfl(fn, nr=10000, cutoff=5.0, nrho=10000, rho_max=40.0):
    """Analytic Cu EAM tables sampled on ``nr`` points out to ``cutoff``:
    density f(r) = exp(-3(r/2.556 - 1)), Morse pair term D=0.35 eV,
    alpha=1.4 1/A, r0=2.556 A (stored as r*phi per setfl), embedding
    F(rho) = -1.2 sqrt(rho) on ``nrho`` points over [0, rho_max]."""
    dr = cutoff / (nr - 1)
    r = np.arange(nr) * dr
    frho = np.exp(-3.0 * (r / 2.556 - 1.0))
    D, alpha, r0 = 0.35, 1.4, 2.556
    phi = D * (np.exp(-2 * alpha * (r - r0)) - 2 * np.exp(-alpha * (r - r0)))
    rphi = r * phi
    drho = rho_max / (nrho - 1)
    rho = np.arange(nrho) * drho
    F = -1.2 * np.sqrt(rho)
    write_setfl(fn, ["Cu"], nrho, drho, nr, dr, cutoff, [F], [frho], {(0, 0): rphi},
                comments=["Analytic Cu EAM: f=exp(-3(r/2.556-1)), Morse D=0.35 "
                          "alpha=1.4 r0=2.556, F=-1.2 sqrt(rho)",
                          "nr=%d cutoff=%g nrho=%d rho_max=%g" % (nr, cutoff, nrho, rho_max),
                          "generated by atomistica_gb300.io.cu_analytic_setfl"],
                Z=[29], mass=[63.546], a0=[3.615], lattice=["fcc"])
    return fn


def analytic_alloy_setfl(fn, elements, nr=2000, cutoff=5.0, nrho=2000, rho_max=60.0, seed=0):
    """Analytic alloy EAM tables for any number of elements, with seeded
    per-element parameters: density f_e(r) = a_e exp(-b_e (r/r_e - 1)),
    embedding F_e(rho) = -c_e sqrt(rho) + g_e rho, and Morse pair terms
    phi_ij(r) = D (exp(-2 alpha (r - r0)) - 2 exp(-alpha (r - r0))) with
    D = sqrt(D_i D_j) and the means of alpha and r0 (stored as r*phi per
    setfl).  Test tables of a plausible shape, not a fitted alloy."""
    rng = np.random.default_rng(seed)
    nel = len(elements)
    dr = cutoff / (nr - 1)
    r = np.arange(nr) * dr
    drho = rho_max / (nrho - 1)
    rhov = np.arange(nrho) * drho
    a = rng.uniform(0.7, 1.3, nel)
    b = rng.uniform(2.5, 3.5, nel)
    re = rng.uniform(2.45, 2.75, nel)
    c = rng.uniform(0.9, 1.5, nel)
    g = rng.uniform(0.0, 0.02, nel)
    D = rng.uniform(0.25, 0.45, nel)
    al = rng.uniform(1.2, 1.6, nel)
    r0 = rng.uniform(2.45, 2.75, nel)
    F = [-c[e] * np.sqrt(rhov) + g[e] * rhov for e in range(nel)]
    frho = [a[e] * np.exp(-b[e] * (r / re[e] - 1.0)) for e in range(nel)]
    rphi = {}
    for i in range(nel):
        for j in range(i + 1):
            Dij, aij, rij = np.sqrt(D[i] * D[j]), 0.5 * (al[i] + al[j]), 0.5 * (r0[i] + r0[j])
            rphi[(i, j)] = r * Dij * (np.exp(-2 * aij * (r - rij)) - 2 * np.exp(-aij * (r - rij)))
    write_setfl(fn, list(elements), nrho, drho, nr, dr, cutoff, F, frho, rphi,
                comments=["Analytic %d-element alloy EAM test tables (seed %d)" % (nel, seed),
                          "nr=%d cutoff=%g nrho=%d rho_max=%g" % (nr, cutoff, nrho, rho_max),
                          "generated by atomistica_gb300.io.analytic_alloy_setfl"],
                Z=[atomic_numbers[x] for x in elements])
    return fn


def write_funcfl(fn, comment, Z, mass, a0, lattice, nrho, drho, nr, dr, cutoff, F, Zr, rho):
    """DYNAMO funcfl file (single element; tabulated_eam.f90:147-200 format):
    comment; Z mass a0 lattice; nrho drho nr dr cutoff; F(rho), Z(r), rho(r)."""
    def block(a):
        a = np.asarray(a, dtype=np.float64)
        return "\n".join(" ".join("% .16e" % x for x in a[q:q + 5]) for q in range(0, len(a), 5))
    with open(fn, "w") as f:
        f.write(comment.strip() + "\n")
        f.write("%d %.6f %.6f %s\n" % (Z, mass, a0, lattice))
        f.write("%d %.16e %d %.16e %.16e\n" % (nrho, drho, nr, dr, cutoff))
        f.write(block(F) + "\n" + block(Zr) + "\n" + block(rho) + "\n")
    return fn


def cu_analytic_funcfl(fn, nr=2000, cutoff=5.5, nrho=2000, rho_max=40.0):
    """Analytic funcfl Cu: density exp(-3(r/2.556 - 1)), effective charge
    Z(r) = 10 exp(-1.5 r) (screened Coulomb pair term Z^2/r in the reference's
    units), embedding F(rho) = -1.2 sqrt(rho)."""
    dr = cutoff / (nr - 1)
    r = np.arange(nr) * dr
    rho = np.exp(-3.0 * (r / 2.556 - 1.0))
    Zr = 10.0 * np.exp(-1.5 * r)
    drho = rho_max / (nrho - 1)
    F = -1.2 * np.sqrt(np.arange(nrho) * drho)
    return write_funcfl(fn, "Analytic Cu funcfl (atomistica_gb300.io.cu_analytic_funcfl)", 29,
                        63.546, 3.615, "FCC", nrho, drho, nr, dr, cutoff, F, Zr, rho)


def read_poscar(fn):
    """Read a VASP POSCAR (VASP 5 format with element line)."""
    with open(fn) as f:
        lines = [ln.strip() for ln in f.read().splitlines()]
    scale = float(lines[1].split()[0])
    cell = np.array([[float(x) for x in lines[2 + k].split()[:3]] for k in range(3)]) * scale
    toks = lines[5].split()
    if all(t.isdigit() for t in toks):
        symbols = lines[0].split()
        counts = [int(t) for t in toks]
        k = 6
    else:
        symbols = toks
        counts = [int(t) for t in lines[6].split()]
        k = 7
    if lines[k][:1].lower() == "s":
        k += 1
    cart = lines[k][:1].lower() in ("c", "k")
    k += 1
    nat = sum(counts)
    xyz = np.array([[float(x) for x in lines[k + q].split()[:3]] for q in range(nat)])
    pos = xyz * scale if cart else xyz @ cell
    numbers = np.concatenate([[atomic_numbers[s]] * c for s, c in zip(symbols, counts)])
    return Structure(pos, cell, np.array([True, True, True]), numbers.astype(np.int32),
                     {"file": str(fn)})
