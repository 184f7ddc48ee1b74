"""
TEST INFRASTRUCTURE ONLY — a second, independent restatement of the Tersoff,
Kumagai and tabulated alloy EAM energies that pins the C++ oracle
(oracle/oracle.cpp).

Atomistica is Fortran, and no Fortran compiler exists on either machine this
project builds or runs on, so the reference itself cannot be executed to pin
the oracle.  This module checks the oracle against a restatement that shares
none of its code and none of its structure:

* pairs are enumerated by brute force over all periodic images (no cell
  binning), numpy;
* the energy is written once, vectorised over bonds and triplets, in torch
  FP64 from the reference's functional forms:
  E = sum over directed bonds ij of 1/2 fc(r_ij) (VR(r_ij) + b_ij VA(r_ij))
  (bop_kernel.f90:1356-1368, 1613), zeta_ij = sum_{ik != ij} fc(r_ik)
  g(cos theta_ijk) h(r_ij - r_ik) (bop_kernel.f90:1171-1280), with the
  Tersoff functions of tersoff_func.f90:32-211, the Kumagai functions of
  kumagai_func.f90:32-221 and the trigonometric cutoff of
  cutoff.f90:171-196;
* forces and the virial are not written at all: they are the automatic
  derivatives of that energy with respect to the positions and to a
  homogeneous strain (torch.autograd), so they check the oracle's
  hand-written derivative chain (bop_kernel.f90:1171-1529) independently.

For the alloy EAM the setfl file is parsed here again and each table becomes
a natural cubic spline built by scipy (the interpolant that
simple_spline.f90:127-195 builds by its own tridiagonal sweep, evaluated from
scipy's piecewise-polynomial coefficients instead of the reference's); the
energy is E = sum_i F_i(max(rho_i, 0)) + sum_i sum_j (r phi)_ij(r_ij) / (2 r_ij)
(tabulated_alloy_eam.f90:147-259, 423-627), with the mask on the centre
atom only and the element filter skipping atoms as centre and neighbour.

Parameters use the dictionary format of atomistica_gb300.parameters (per
element arrays by the centre atom's element, pair arrays by the symmetric
pair index of macros.inc:123).  Small systems only (all pairs of all images
are tested): a few hundred atoms.
"""

import itertools

import numpy as np

_SYMBOLS = {"H": 1, "C": 6, "N": 7, "Si": 14, "Ge": 32, "Fe": 26, "W": 74, "Al": 13, "Pt": 78}


def _pair_index(i, j, n):
    return min(i + j * n, j + i * n) - min(i * (i + 1) // 2, j * (j + 1) // 2)


def image_pairs(positions, cell, pbc, cutoff):
    """All (i, j, shift) with |r_j + shift . cell - r_i| < cutoff, i == j
    allowed for shift != 0 (self-images), by testing every image of every
    pair.  cell rows are the lattice vectors."""
    pos = np.asarray(positions, dtype=np.float64)
    cell = np.asarray(cell, dtype=np.float64)
    frac = np.linalg.solve(cell.T, pos.T).T
    vol = abs(np.linalg.det(cell))
    rng = []
    for k in range(3):
        if not pbc[k]:
            rng.append([0])
            continue
        other = np.cross(cell[(k + 1) % 3], cell[(k + 2) % 3])
        height = vol / np.linalg.norm(other)
        span = frac[:, k].max() - frac[:, k].min() + cutoff / height
        n = int(np.ceil(span)) + 1
        rng.append(range(-n, n + 1))
    out_i, out_j, out_s = [], [], []
    c2 = cutoff * cutoff
    for s in itertools.product(*rng):
        off = np.asarray(s, dtype=np.float64) @ cell
        d = pos[None, :, :] + off[None, None, :] - pos[:, None, :]
        r2 = np.einsum("ijk,ijk->ij", d, d)
        ok = r2 < c2
        if s == (0, 0, 0):
            np.fill_diagonal(ok, False)
        ii, jj = np.nonzero(ok)
        out_i.append(ii)
        out_j.append(jj)
        out_s.append(np.tile(np.asarray(s, dtype=np.int64), (len(ii), 1)))
    i = np.concatenate(out_i)
    j = np.concatenate(out_j)
    sh = np.concatenate(out_s)
    order = np.lexsort((sh[:, 2], sh[:, 1], sh[:, 0], j, i))
    return i[order], j[order], sh[order]


def _trig_cutoff(torch, r, r1, r2):
    x = np.pi * (r - r1) / (r2 - r1)
    mid = 0.5 * (1.0 + torch.cos(torch.clamp(x, 0.0, np.pi)))
    return torch.where(r <= r1, torch.ones_like(r), torch.where(r >= r2, torch.zeros_like(r), mid))


def _elements(params, numbers):
    syms = list(params["el"])
    zs = [_SYMBOLS[x] for x in syms]
    return np.array([zs.index(z) if z in zs else -1 for z in numbers], dtype=np.int64)


def bop_energy(kind, params, positions, cell, pbc, numbers, mask=None, strain=None):
    """Energy (torch scalar) and per-atom energies of a Tersoff ("tersoff")
    or Kumagai ("kumagai") system as a differentiable function of positions
    (torch (nat,3) FP64) and cell (torch (3,3)); strain (torch (3,3) or
    None) deforms both by (I + strain)."""
    import torch
    nel = len(params["el"])
    el = _elements(params, numbers)
    npairs = nel * (nel + 1) // 2
    r2max = max(params["r2"][:npairs])
    pos_np = positions.detach().cpu().numpy()
    cell_np = cell.detach().cpu().numpy()
    i, j, sh = image_pairs(pos_np, cell_np, pbc, r2max)
    keep = (el[i] >= 0) & (el[j] >= 0)
    i, j, sh = i[keep], j[keep], sh[keep]
    pidx = np.array([_pair_index(a, b, nel) for a, b in zip(el[i], el[j])], dtype=np.int64)
    if strain is not None:
        F = torch.eye(3, dtype=torch.float64) + strain
        positions = positions @ F.T
        cell = cell @ F.T
    ti, tj = torch.as_tensor(i), torch.as_tensor(j)
    d = positions[tj] + torch.as_tensor(sh, dtype=torch.float64) @ cell - positions[ti]
    r = torch.sqrt((d * d).sum(1))
    P = {k: torch.as_tensor(np.asarray(v, dtype=np.float64)) for k, v in params.items()
         if k not in ("el", "__ref__")}
    tp = torch.as_tensor(pidx)
    inside = (r < P["r2"][tp]).detach().numpy()
    # bonds: pairs within their own pair cutoff
    b_i, b_j, b_p = i[inside], j[inside], pidx[inside]
    tb = torch.as_tensor(np.nonzero(inside)[0])
    rb, db, tpb = r[tb], d[tb], torch.as_tensor(b_p)
    fc = _trig_cutoff(torch, rb, P["r1"][tpb], P["r2"][tpb])
    # triplets (ij, ik) of the same centre i, ik != ij (k may equal j as
    # another image)
    nb = len(b_i)
    starts = np.searchsorted(b_i, np.arange(len(numbers) + 1))
    t_ij, t_ik = [], []
    for a in range(len(numbers)):
        rng = np.arange(starts[a], starts[a + 1])
        if len(rng) < 2:
            continue
        x, y = np.meshgrid(rng, rng, indexing="ij")
        off = x != y
        t_ij.append(x[off])
        t_ik.append(y[off])
    t_ij = torch.as_tensor(np.concatenate(t_ij) if t_ij else np.zeros(0, np.int64))
    t_ik = torch.as_tensor(np.concatenate(t_ik) if t_ik else np.zeros(0, np.int64))
    ei = torch.as_tensor(el[b_i])
    cos = (db[t_ij] * db[t_ik]).sum(1) / (rb[t_ij] * rb[t_ik])
    dr = rb[t_ij] - rb[t_ik]
    eit, pik = ei[t_ij], tpb[t_ik]
    if kind == "tersoff":
        hc = P["h"][eit] - cos
        c2, d2 = P["c"][eit] ** 2, P["d"][eit] ** 2
        g = P["omega"][pik] * (1.0 + c2 / d2 - c2 / (d2 + hc * hc))
        mu, m = P["mubo"][pik], P["m"][pik]
        arg = 2.0 * mu * dr
        hval = torch.where(mu == 0.0, torch.ones_like(dr),
                           torch.exp(torch.where(m == 1, arg, arg ** m)))
    elif kind == "kumagai":
        hc = P["h"][eit] - cos
        hc2 = hc * hc
        g = P["c1"][eit] + P["c2"][eit] * hc2 / (P["c3"][eit] + hc2) * \
            (1.0 + P["c4"][eit] * torch.exp(-P["c5"][eit] * hc2))
        alpha, beta = P["alpha"][pik], P["beta"][pik]
        hval = torch.where(alpha == 0.0, torch.ones_like(dr),
                           torch.where(beta == 1, torch.exp(alpha * dr),
                                       torch.where(beta == 3, torch.exp(dr ** 3),
                                                   torch.exp(alpha * dr ** beta))))
    else:
        raise ValueError(kind)
    zeta = torch.zeros(nb, dtype=torch.float64).index_add(0, t_ij, fc[t_ik] * g * hval)
    pos_z = zeta > 0.0
    zs = torch.where(pos_z, zeta, torch.ones_like(zeta))
    if kind == "tersoff":
        n = P["n"][ei]
        bval = P["xi"][tpb] * (1.0 + P["beta"][ei] ** n * zs ** n) ** (-0.5 / n)
        VA = -P["B"][tpb] * torch.exp(-P["mu"][tpb] * rb)
        VR = P["A"][tpb] * torch.exp(-P["lambda"][tpb] * rb)
    else:
        bval = (1.0 + zs ** P["eta"][ei]) ** (-P["delta"][ei])
        VA = -P["B"][tpb] * torch.exp(-P["lambda2"][tpb] * rb)
        VR = P["A"][tpb] * torch.exp(-P["lambda1"][tpb] * rb)
    bval = torch.where(pos_z, bval, torch.ones_like(bval))
    if mask is not None:
        mk = np.asarray(mask) != 0
        mf = torch.as_tensor((mk[b_i].astype(np.float64) + mk[b_j].astype(np.float64)) / 2.0)
    else:
        mf = torch.ones(nb, dtype=torch.float64)
    e_bond = 0.5 * fc * mf * (VR + bval * VA)
    nat = len(numbers)
    pe = torch.zeros(nat, dtype=torch.float64)
    pe = pe.index_add(0, torch.as_tensor(b_i), e_bond).index_add(0, torch.as_tensor(b_j), e_bond)
    return e_bond.sum(), 0.5 * pe


def bop(kind, params, s, mask=None):
    """Energy, forces (nat,3), virial (3,3) in the layout of oracle.bop
    (wpot[a, c] = sum over bonds of r_ij[a] f_i[c]) and per-atom energies."""
    import torch
    pos = torch.tensor(s.positions, dtype=torch.float64, requires_grad=True)
    cell = torch.tensor(s.cell, dtype=torch.float64)
    eps = torch.zeros((3, 3), dtype=torch.float64, requires_grad=True)
    E, pe = bop_energy(kind, params, pos, cell, s.pbc, s.numbers, mask=mask, strain=eps)
    gpos, geps = torch.autograd.grad(E, (pos, eps))
    # dE/d eps[a, b] = sum_i dE/dr_i[a] r_i[b]; the reference's virial is
    # W[a, c] = sum r_ij[a] df_i[c] = (dE/d eps)^T.
    return {"epot": float(E.detach()), "f": -gpos.numpy(), "wpot": geps.numpy().T.copy(),
            "epot_per_at": pe.detach().numpy()}


def read_setfl(fn):
    """(elements, Z, F tables, rho tables, r*phi tables {(i, j)}, grids) of a
    DYNAMO setfl file, values read across line breaks."""
    with open(fn) as f:
        lines = f.read().split("\n")
    head = lines[3].split()
    nel = int(head[0])
    names = head[1:1 + nel]
    g = lines[4].split()
    nF, dF, nr, dr, cutoff = int(g[0]), float(g[1]), int(g[2]), float(g[3]), float(g[4])
    pos = 5
    Z, F, rho, rphi = [], [], [], {}
    toks = []

    def take(n):
        nonlocal pos, toks
        while len(toks) < n:
            toks += lines[pos].split()
            pos += 1
        out, toks = np.array(toks[:n], dtype=np.float64), toks[n:]
        return out

    for e in range(nel):
        Z.append(int(lines[pos].split()[0]))
        pos += 1
        toks = []
        F.append(take(nF))
        rho.append(take(nr))
        toks = []
    for i in range(nel):
        for j in range(i + 1):
            rphi[(i, j)] = take(nr)
    return dict(names=names, Z=Z, F=F, rho=rho, rphi=rphi, nF=nF, dF=dF, nr=nr, dr=dr,
                cutoff=cutoff)


class _Spline:
    """Natural cubic spline through (x0 + k dx, y_k), extrapolated by its end
    polynomials, evaluated differentiably in torch on fixed intervals."""

    def __init__(self, y, dx):
        from scipy.interpolate import CubicSpline
        self.dx = dx
        self.n = len(y)
        self.c = CubicSpline(np.arange(self.n) * dx, y, bc_type="natural").c  # (4, n-1)

    def __call__(self, torch, x):
        k = np.clip(np.floor(x.detach().numpy() / self.dx).astype(np.int64), 0, self.n - 2)
        t = x - torch.as_tensor(k * self.dx, dtype=torch.float64)
        c = torch.as_tensor(self.c[:, k])
        return ((c[0] * t + c[1]) * t + c[2]) * t + c[3]


def eam_energy(fn, positions, cell, pbc, numbers, mask=None, elements=None, strain=None):
    """Energy and per-atom energies of a tabulated alloy EAM (setfl file fn)
    as a differentiable function of positions and cell (torch FP64).
    elements: None or a list of atomic numbers (the element filter)."""
    import torch
    t = read_setfl(fn)
    nel = len(t["Z"])
    db = np.array([t["Z"].index(z) if z in t["Z"] else -1 for z in numbers], dtype=np.int64)
    if elements is not None:
        db[~np.isin(numbers, list(elements))] = -1
    Fs = [_Spline(t["F"][e], t["dF"]) for e in range(nel)]
    pad = np.zeros(2)
    rhos = [_Spline(np.concatenate([t["rho"][e], pad]), t["dr"]) for e in range(nel)]
    phis = {k: _Spline(0.5 * np.concatenate([v, pad]), t["dr"]) for k, v in t["rphi"].items()}
    i, j, sh = image_pairs(positions.detach().numpy(), cell.detach().numpy(), pbc, t["cutoff"])
    on_i = db[i] >= 0
    if mask is not None:
        on_i &= np.asarray(mask)[i] != 0
    keep = on_i & (db[j] >= 0)
    i, j, sh = i[keep], j[keep], sh[keep]
    if strain is not None:
        Fm = torch.eye(3, dtype=torch.float64) + strain
        positions = positions @ Fm.T
        cell = cell @ Fm.T
    d = positions[torch.as_tensor(j)] + torch.as_tensor(sh, dtype=torch.float64) @ cell - \
        positions[torch.as_tensor(i)]
    r = torch.sqrt((d * d).sum(1))
    nat = len(numbers)
    rho = torch.zeros(nat, dtype=torch.float64)
    pe = torch.zeros(nat, dtype=torch.float64)
    for e in range(nel):
        sel = np.nonzero(db[j] == e)[0]
        if len(sel):
            ts = torch.as_tensor(sel)
            rho = rho.index_add(0, torch.as_tensor(i[sel]), rhos[e](torch, r[ts]))
    for a in range(nel):
        for b in range(nel):
            sel = np.nonzero((db[i] == a) & (db[j] == b))[0]
            if len(sel):
                ts = torch.as_tensor(sel)
                ph = phis[(max(a, b), min(a, b))](torch, r[ts]) / r[ts]
                pe = pe.index_add(0, torch.as_tensor(i[sel]), ph)
    centre = db >= 0
    if mask is not None:
        centre &= np.asarray(mask) != 0
    for e in range(nel):
        sel = np.nonzero(centre & (db == e))[0]
        if len(sel):
            ts = torch.as_tensor(sel)
            pe = pe.index_add(0, ts, Fs[e](torch, torch.clamp(rho[ts], min=0.0)))
    return pe.sum(), pe


def eam(fn, s, mask=None, elements=None):
    """Energy, forces, virial (layout of oracle.EAM.compute) and per-atom
    energies of the alloy EAM of setfl file fn."""
    import torch
    pos = torch.tensor(s.positions, dtype=torch.float64, requires_grad=True)
    cell = torch.tensor(s.cell, dtype=torch.float64)
    eps = torch.zeros((3, 3), dtype=torch.float64, requires_grad=True)
    E, pe = eam_energy(fn, pos, cell, s.pbc, s.numbers, mask=mask, elements=elements,
                       strain=eps)
    gpos, geps = torch.autograd.grad(E, (pos, eps))
    return {"epot": float(E.detach()), "f": -gpos.numpy(), "wpot": geps.numpy().T.copy(),
            "epot_per_at": pe.detach().numpy()}
