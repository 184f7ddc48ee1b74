"""
Native objects with the interface of Atomistica's Python extension
``_atomistica`` (src/python/c/particles.c, neighbors.c, potential.c):

    p = Particles(); p.allocate(nat); p.set_cell(cell, pbc)
    p.coordinates[:] = r; p.I_changed_positions()
    p.Z[:] = numbers; p.update_elements()
    nl = Neighbors(avgn)
    pot = Tersoff(**params); pot.bind_to(p, nl)
    epot, f, wpot, ... = pot.energy_and_forces(p, nl, forces=..., mask=...,
                          epot_per_at=True, epot_per_bond=..., f_per_bond=...,
                          wpot_per_at=..., wpot_per_bond=...)

Return layouts follow potential.c:622-657: f (nat,3); wpot (3,3) with
wpot[a,c] = W(a,c); wpot_per_at (nat,3,3) and wpot_per_bond (n,3,3) with
[i,x,y] = W_i(y,x) (the Fortran (3,3,n) buffer viewed C-ordered); per-bond
arrays follow the neighbour-list order of Neighbors.get_neighbors.

Arrays may be numpy (host) or torch CUDA tensors (used in place).  All
computation runs in libatomistica_gb300 on the GPU; there is no CPU path.
"""

import ctypes

import numpy as np

from . import _lib
from ._lib import GB_PRECISION_FP64, GB_PRECISION_MIXED, check, load
from .parameters import (BRENNER_KEYS, JUSLIN_KEYS, SCREENING_KEYS, Erhart_PRB_71_035211_SiC,
                         Juslin_JAP_98_123520_WCH,
                         Kumagai_CompMaterSci_39_457_Si,
                         Kumagai_CompMaterSci_39_457_Si__Scr, Tersoff_PRB_39_5566_Si_C,
                         Tersoff_PRB_39_5566_Si_C__Scr, atomic_numbers)

try:  # PyTorch is optional: only for device-resident inputs/outputs.
    import torch
except Exception:  # pragma: no cover
    torch = None


def _is_torch(x):
    return torch is not None and isinstance(x, torch.Tensor)


def _ptr(x, dtype):
    """(pointer, keepalive) for a numpy array or torch tensor."""
    if x is None:
        return None, None
    if _is_torch(x):
        want = torch.float64 if dtype == np.float64 else torch.int32
        if x.dtype != want or not x.is_contiguous():
            raise TypeError("tensor must be contiguous %s" % want)
        return x.data_ptr(), x
    a = np.ascontiguousarray(x, dtype=dtype)
    return a.ctypes.data, a


def _to_numpy(x):
    if _is_torch(x):
        return x.detach().cpu().numpy()
    return np.asarray(x)


class Particles:
    """particles_t: positions (nat,3), cell (rows = lattice vectors), pbc,
    atomic numbers (python_particles.f90:85-140)."""

    def __init__(self):
        self._L = load()
        self._h = ctypes.c_void_p()
        check(self._L.gb_particles_new(ctypes.byref(self._h)), "particles_new")
        self.nat = 0
        self.coordinates = np.zeros((0, 3))
        self.Z = np.zeros(0, dtype=np.int32)
        self.cell = np.eye(3)
        self.pbc = np.array([True, True, True])

    def __del__(self):
        if getattr(self, "_h", None) and self._h.value:
            self._L.gb_particles_free(self._h)
            self._h = ctypes.c_void_p()

    def __len__(self):
        return self.nat

    def allocate(self, nat):
        check(self._L.gb_particles_allocate(self._h, int(nat)), "particles_allocate")
        self.nat = int(nat)
        self.coordinates = np.zeros((self.nat, 3))
        self.Z = np.zeros(self.nat, dtype=np.int32)

    def set_cell(self, cell, pbc=True):
        cell = np.asarray(cell, dtype=np.float64)
        if cell.shape == (3,):
            cell = np.diag(cell)
        pbc = np.broadcast_to(np.asarray(pbc, dtype=bool), (3,)).copy()
        c = np.ascontiguousarray(cell)
        pb = np.ascontiguousarray(pbc.astype(np.int32))
        check(self._L.gb_particles_set_cell(self._h, c.ctypes.data, pb.ctypes.data),
              "particles_set_cell")
        self.cell = cell.copy()
        self.pbc = pbc

    def I_changed_positions(self):
        """Upload ``coordinates`` (particles_I_changed_positions)."""
        self.set_positions(self.coordinates)

    def set_positions(self, r):
        """Positions (nat,3): numpy array or torch CUDA tensor (float64).  A
        C-contiguous float64 numpy array becomes ``coordinates`` itself (no
        copy), as the reference's coordinates array is the particles'
        storage; later writes to it take effect on I_changed_positions()."""
        ptr, keep = _ptr(r, np.float64)
        if not _is_torch(r):
            self.coordinates = keep
        check(self._L.gb_particles_set_positions(self._h, ptr), "particles_set_positions")

    def update_elements(self):
        z = np.ascontiguousarray(self.Z, dtype=np.int32)
        check(self._L.gb_particles_set_Z(self._h, z.ctypes.data), "particles_set_Z")

    def set_Z(self, Z):
        self.Z = np.ascontiguousarray(_to_numpy(Z), dtype=np.int32)
        self.update_elements()

    def set_stream(self, stream):
        check(self._L.gb_particles_set_stream(self._h, stream), "particles_set_stream")


def from_atoms(atoms):
    """Particles from an ASE-like object (positions, cell, pbc, numbers)."""
    p = Particles()
    pos = atoms.get_positions() if hasattr(atoms, "get_positions") else atoms.positions
    cell = atoms.get_cell() if hasattr(atoms, "get_cell") else atoms.cell
    pbc = atoms.get_pbc() if hasattr(atoms, "get_pbc") else atoms.pbc
    numbers = atoms.get_atomic_numbers() if hasattr(atoms, "get_atomic_numbers") else \
        atoms.numbers
    p.allocate(len(pos))
    p.set_cell(np.asarray(cell), pbc)
    p.Z[:] = numbers
    p.update_elements()
    p.coordinates[:] = pos
    p.I_changed_positions()
    return p


class Neighbors:
    """neighbors_t: full directed cell-list neighbour list."""

    def __init__(self, avgn=100):
        self._L = load()
        self._h = ctypes.c_void_p()
        check(self._L.gb_neighbors_new(ctypes.byref(self._h), int(avgn)), "neighbors_new")

    def __del__(self):
        if getattr(self, "_h", None) and self._h.value:
            self._L.gb_neighbors_free(self._h)
            self._h = ctypes.c_void_p()

    def request_interaction_range(self, cutoff):
        check(self._L.gb_neighbors_request_interaction_range(self._h, float(cutoff)),
              "request_interaction_range")

    @property
    def interaction_range(self):
        return self._L.gb_neighbors_get_interaction_range(self._h)

    def update(self, p):
        check(self._L.gb_neighbors_update(self._h, p._h), "neighbors_update")

    def get_list(self, p):
        """(seed (nat+1), j (n), dc (n,3)): CSR list in reference order."""
        self.update(p)
        n = self._L.gb_neighbors_get_size(self._h)
        seed = np.zeros(len(p) + 1, dtype=np.int64)
        j = np.zeros(max(n, 1), dtype=np.int32)
        dc = np.zeros((max(n, 1), 3), dtype=np.int32)
        check(self._L.gb_neighbors_get(self._h, p._h, seed.ctypes.data, j.ctypes.data,
                                       dc.ctypes.data), "neighbors_get")
        return seed, j[:n], dc[:n]

    def get_neighbors(self, p, vec=False):
        """(i, j, [dr], abs_dr) with dr = r_i - r_j + cell^T dc
        (f_get_all_neighbors[_vec], neighbors_wrap.f90:425-492)."""
        seed, j, dc = self.get_list(p)
        i = np.repeat(np.arange(len(p), dtype=np.int32), np.diff(seed))
        r = p.coordinates
        dr = r[i] - r[j] + dc @ p.cell
        abs_dr = np.sqrt(np.sum(dr * dr, axis=1))
        if vec:
            return i, j, dr, abs_dr
        return i, j, abs_dr

    def get_coordination_numbers(self, p, cutoff):
        i, j, r = self.get_neighbors(p)
        return np.bincount(i[r < cutoff], minlength=len(p))


def _fill(arr, vals, n):
    for q in range(n):
        arr[q] = vals[q]


def tersoff_params(params, base=Tersoff_PRB_39_5566_Si_C):
    """gb_tersoff_params_t from a parameter dict (parameters.py format);
    keys not given keep the values of ``base`` (the default Si-C set)."""
    d = dict(base)
    d.update({k: v for k, v in params.items() if not k.startswith("__")})
    p = _lib.TersoffParams()
    els = d["el"]
    p.nel = len(els)
    if not 1 <= p.nel <= 3:
        raise ValueError("Tersoff supports 1..3 elements")
    for q, s in enumerate(els):
        p.Z[q] = atomic_numbers[s]
    npair = p.nel * (p.nel + 1) // 2
    for k in ("A", "B", "xi", "lambda", "mu", "omega", "mubo", "r1", "r2"):
        vals = d.get(k)
        if vals is None or len(vals) < npair:
            vals = list(vals or []) + [{"xi": 1.0, "omega": 1.0, "mubo": 0.0}.get(k, 1.0)] * npair
        _fill(getattr(p, "lambda_" if k == "lambda" else k), [float(v) for v in vals], npair)
    ms = list(d.get("m", [1] * npair)) + [1] * npair
    _fill(p.m, [int(v) for v in ms], npair)
    for k in ("beta", "n", "c", "d", "h"):
        _fill(getattr(p, k), [float(v) for v in d[k]], p.nel)
    return p


def screening_params(params, base):
    """gb_screening_params_t (or1, or2, bor1, bor2, Cmin, Cmax per pair)."""
    d = dict(base)
    d.update({k: v for k, v in params.items() if k in SCREENING_KEYS})
    p = _lib.ScreeningParams()
    for k in SCREENING_KEYS:
        _fill(getattr(p, k), [float(v) for v in d[k]], len(d[k]))
    return p


# The compiled-in default of BrennerScr (brenner_params.f90:92-104 under
# SCREENING), the base that keyword arguments override; it differs from the
# front-end's Erhart_PRB_71_035211_SiC__Scr dictionary in the C-Si cutoffs.
_BRENNER_SCR_DEFAULT = dict(
    Erhart_PRB_71_035211_SiC,
    mu=[1.0 / 1.4276, 1.0 / 1.79, 1.0 / 1.842], m=[3, 3, 3],
    r1=[2.00, (2.00 * 2.50) ** 0.5, 2.50],
    r2=[2.00 * 1.2, (2.00 * 2.50) ** 0.5 * 1.2, 2.50 * 1.2],
    or1=[2.00, (2.00 * 3.00) ** 0.5, 3.00], or2=[2.00 * 2.0, (2.00 * 3.00) ** 0.5 * 2.0, 6.0],
    bor1=[2.00, (2.00 * 3.00) ** 0.5, 3.00], bor2=[2.00 * 2.0, (2.00 * 3.00) ** 0.5 * 2.0, 6.0],
    Cmin=[1.0, 1.0, 1.0], Cmax=[3.0, 3.0, 3.0])


def brenner_params(params, base=Erhart_PRB_71_035211_SiC):
    """gb_brenner_params_t from a parameter dict (every array per element
    pair); keys not given keep the values of ``base``."""
    d = dict(base)
    d.update({k: v for k, v in params.items() if not k.startswith("__")})
    p = _lib.BrennerParams()
    els = d["el"]
    p.nel = len(els)
    if not 1 <= p.nel <= 3:
        raise ValueError("Brenner supports 1..3 elements")
    for q, s in enumerate(els):
        p.Z[q] = atomic_numbers[s]
    npair = p.nel * (p.nel + 1) // 2
    for k in BRENNER_KEYS:
        if len(d[k]) < npair:
            raise ValueError("Brenner: %s needs %d entries (one per element pair)" % (k, npair))
        if k == "m":
            _fill(p.m, [int(v) for v in d[k]], npair)
        else:
            _fill(getattr(p, k), [float(v) for v in d[k]], npair)
    return p


def juslin_params(params, base=Juslin_JAP_98_123520_WCH):
    """gb_juslin_params_t from a parameter dict (pair arrays per ordered
    element pair, alpha / omega / m per element triplet); keys not given keep
    the values of ``base``.  m defaults to 1 for every triplet."""
    d = dict(base)
    d.update({k: v for k, v in params.items() if not k.startswith("__")})
    p = _lib.JuslinParams()
    els = d["el"]
    p.nel = len(els)
    if not 1 <= p.nel <= 3:
        raise ValueError("Juslin supports 1..3 elements")
    for q, s in enumerate(els):
        p.Z[q] = atomic_numbers[s]
    npair, ntrip = p.nel * p.nel, p.nel ** 3
    for k in JUSLIN_KEYS:
        if len(d[k]) < npair:
            raise ValueError("Juslin: %s needs %d entries (one per ordered element pair)"
                             % (k, npair))
        _fill(getattr(p, k), [float(v) for v in d[k]], npair)
    ms = d.get("m", [1] * ntrip)
    for k, vals in (("alpha", d["alpha"]), ("omega", d["omega"]), ("m", ms)):
        if len(vals) < ntrip:
            raise ValueError("Juslin: %s needs %d entries (one per element triplet)"
                             % (k, ntrip))
        _fill(getattr(p, k), [int(v) if k == "m" else float(v) for v in vals], ntrip)
    return p


def kumagai_params(params, base=Kumagai_CompMaterSci_39_457_Si):
    d = dict(base)
    d.update({k: v for k, v in params.items() if not k.startswith("__")})
    p = _lib.KumagaiParams()
    if len(d["el"]) != 1:
        raise ValueError("Kumagai supports exactly one element")
    p.nel = 1
    p.Z[0] = atomic_numbers[d["el"][0]]
    for k in ("A", "B", "lambda1", "lambda2", "eta", "delta", "alpha", "c1", "c2", "c3",
              "c4", "c5", "h", "r1", "r2"):
        getattr(p, k)[0] = float(d[k][0])
    p.beta[0] = int(d["beta"][0])
    return p


class _Potential:
    """Common energy_and_forces front-end (src/python/c/potential.c:347-666)."""

    features = ("mask", "per_at", "per_bond")

    def __init__(self):
        self._L = load()
        self._h = ctypes.c_void_p()

    def __del__(self):
        if getattr(self, "_h", None) and self._h.value:
            self._L.gb_potential_free(self._h)
            self._h = ctypes.c_void_p()

    @property
    def precision(self):
        return self._precision

    def set_precision(self, precision):
        code = {"fp64": GB_PRECISION_FP64, "mixed": GB_PRECISION_MIXED,
                GB_PRECISION_FP64: GB_PRECISION_FP64,
                GB_PRECISION_MIXED: GB_PRECISION_MIXED}[precision]
        check(self._L.gb_potential_set_precision(self._h, code), "set_precision")
        self._precision = "fp64" if code == GB_PRECISION_FP64 else "mixed"

    def set_stream(self, stream):
        check(self._L.gb_potential_set_stream(self._h, stream), "set_stream")

    def get_cutoff(self):
        return self._L.gb_potential_get_cutoff(self._h)

    def bind_to(self, p, nl):
        err = ctypes.c_int(0)
        check(self._L.gb_potential_bind_to(self._h, p._h, nl._h, ctypes.byref(err)), "bind_to")

    def last_timing(self):
        """(neighbour-list ms, force ms, total ms, dominant kernel ms) of the
        last call (CUDA events on the potential's stream)."""
        t = (ctypes.c_double * 4)()
        self._L.gb_potential_last_timing(self._h, t)
        return tuple(t)

    def energy_and_forces_ghost(self, r, Z, seed, nbr, natloc, **kw):
        """The LAMMPS contract: see gb_potential_energy_and_forces_ghost."""
        return _ghost_call(self, r, Z, seed, nbr, natloc, **kw)

    def set_tile_atoms(self, atoms):
        """Atoms per bond-order tile (power of two <= 64; 0: automatic)."""
        check(self._L.gb_potential_set_tile_atoms(self._h, int(atoms)), "set_tile_atoms")

    def set_graph(self, on=True):
        """CUDA-graph replay of whole evaluations (gb_potential_set_graph):
        after an eager call, calls with only energy, forces and virial on
        the same particles, list, cell and force array replay one graph."""
        check(self._L.gb_potential_set_graph(self._h, 1 if on else 0), "set_graph")

    def last_stats(self):
        """(directed bonds, bonds recomputed on the accurate path of the mixed
        form, atoms per tile) of the last call."""
        v = (ctypes.c_int64 * 4)()
        self._L.gb_potential_last_stats(self._h, v)
        return tuple(v[:3])

    def last_replayed(self):
        """True when the last call was a CUDA-graph replay."""
        v = (ctypes.c_int64 * 4)()
        self._L.gb_potential_last_stats(self._h, v)
        return bool(v[3])

    def energy_and_forces(self, particles, neighbors, forces=None, mask=None, charges=None,
                          epot_per_at=None, epot_per_bond=None, f_per_bond=None,
                          wpot_per_at=None, wpot_per_bond=None, accumulate=True):
        nat = len(particles)
        dev = _is_torch(forces) and forces.is_cuda
        accumulate = accumulate and forces is not None  # a fresh array is just written

        def zeros(shape):
            if dev:
                return torch.zeros(shape, dtype=torch.float64, device=forces.device)
            return np.zeros(shape)

        if forces is None:
            forces = zeros((nat, 3))
        elif tuple(forces.shape) != (nat, 3):
            raise RuntimeError("Length of force array (= %d) does not equal  number of atoms "
                               "(= %d)." % (forces.shape[0], nat))
        if mask is not None:
            if len(mask) != nat:
                raise RuntimeError("Length of mask array (= %d) does not equal number of "
                                   "atoms (= %d)." % (len(mask), nat))
            if _is_torch(mask):
                mask = mask.to(torch.int32).contiguous()
            else:
                mask = np.ascontiguousarray(np.asarray(mask).astype(np.int32))
        if "per_bond" not in self.features and (epot_per_bond or f_per_bond or wpot_per_bond):
            raise RuntimeError("Per-bond properties are not supported by %s."
                               % type(self).__name__)
        nb = 0
        if epot_per_bond or f_per_bond or wpot_per_bond:
            neighbors.update(particles)
            nb = self._L.gb_neighbors_get_size(neighbors._h)
        wpot = np.zeros((3, 3), order="F")
        out = {}
        if epot_per_at:
            out["epot_per_at"] = zeros((nat,))
        if epot_per_bond:
            out["epot_per_bond"] = zeros((nb,))
        if f_per_bond:
            out["f_per_bond"] = zeros((nb, 3))
        if wpot_per_at:
            out["wpot_per_at"] = zeros((nat, 3, 3))
        if wpot_per_bond:
            out["wpot_per_bond"] = zeros((nb, 3, 3))
        fp, fkeep = _ptr(forces, np.float64)
        mp, mkeep = _ptr(mask, np.int32)
        ptrs = {k: _ptr(v, np.float64) for k, v in out.items()}
        epot = ctypes.c_double(0.0)
        err = ctypes.c_int(0)
        g = lambda k: ptrs[k][0] if k in ptrs else None  # noqa: E731
        # accumulate=False: the forces array is overwritten (no upload of it)
        rc = self._L.gb_potential_energy_and_forces_flags(
            self._h, particles._h, neighbors._h, None, ctypes.byref(epot), fp,
            wpot.ctypes.data, mp, g("epot_per_at"), g("epot_per_bond"), g("f_per_bond"),
            g("wpot_per_at"), g("wpot_per_bond"), 0 if accumulate else _lib.GB_FORCES_SET,
            ctypes.byref(err))
        check(rc, "%s.energy_and_forces" % type(self).__name__)
        if fkeep is not forces and not _is_torch(forces):
            forces[...] = fkeep
        for k, (ptr, keep) in ptrs.items():
            out[k] = keep
        res = [epot.value, forces, np.ascontiguousarray(wpot)]
        for k, flag in (("epot_per_at", epot_per_at), ("epot_per_bond", epot_per_bond),
                        ("f_per_bond", f_per_bond), ("wpot_per_at", wpot_per_at),
                        ("wpot_per_bond", wpot_per_bond)):
            if flag is not None:
                res.append(out.get(k) if flag else None)
        return tuple(res)


def _ghost_call(pot, r, Z, seed, nbr, natloc, forces=None, mask=None, epot_per_at=False,
                wpot_per_at=False, vatom=None):
    """energy_and_forces on a caller's list over local + ghost atoms (the
    LAMMPS contract): returns (epot, forces (nat,3), wpot, [epot_per_at],
    [wpot_per_at]); bonds of the first natloc atoms, forces on all.  With
    ``vatom`` (a (nat,6) float64 array) the per-atom virial is accumulated
    into it in LAMMPS's layout and sign instead
    (gb_potential_energy_and_forces_lammps)."""
    r = np.ascontiguousarray(r, dtype=np.float64)
    nat = len(r)
    Z = np.ascontiguousarray(Z, dtype=np.int32)
    seed = np.ascontiguousarray(seed, dtype=np.int32)
    nbr = np.ascontiguousarray(nbr, dtype=np.int32)
    f = np.zeros((nat, 3)) if forces is None else forces
    epot = ctypes.c_double(0.0)
    wpot = np.zeros((3, 3), order="F")  # (layouts as energy_and_forces)
    epa = np.zeros(nat) if epot_per_at else None
    wpa = np.zeros((nat, 3, 3)) if wpot_per_at else None
    m = None if mask is None else np.ascontiguousarray(np.asarray(mask).astype(np.int32))
    err = ctypes.c_int(0)
    ptr = lambda a: None if a is None else a.ctypes.data  # noqa: E731
    if vatom is not None:
        if vatom.shape != (nat, 6) or vatom.dtype != np.float64 or \
                not vatom.flags["C_CONTIGUOUS"]:
            raise ValueError("vatom must be a C-contiguous (nat, 6) float64 array")
        if wpot_per_at:
            raise ValueError("vatom and wpot_per_at exclude each other")
        fn, wpa, name = (pot._L.gb_potential_energy_and_forces_lammps, vatom,
                         "energy_and_forces_lammps")
    else:
        fn, name = pot._L.gb_potential_energy_and_forces_ghost, "energy_and_forces_ghost"
    check(fn(pot._h, nat, int(natloc), r.ctypes.data, Z.ctypes.data, seed.ctypes.data,
             nbr.ctypes.data if len(nbr) else None, ctypes.byref(epot), f.ctypes.data,
             wpot.ctypes.data, ptr(m), ptr(epa), ptr(wpa), ctypes.byref(err)), name)
    out = [epot.value, f, np.ascontiguousarray(wpot)]
    if epot_per_at:
        out.append(epa)
    if wpot_per_at:
        out.append(wpa)
    return tuple(out)


class Tersoff(_Potential):
    """Tersoff bond-order potential (src/potentials/bop/tersoff/)."""

    def __init__(self, precision="fp64", **params):
        super().__init__()
        if params:
            p = tersoff_params(params)
            check(self._L.gb_tersoff_new(ctypes.byref(self._h), ctypes.byref(p)), "Tersoff")
        else:
            check(self._L.gb_tersoff_new(ctypes.byref(self._h), None), "Tersoff")
        self.set_precision(precision)


class Kumagai(_Potential):
    """Kumagai bond-order potential (src/potentials/bop/kumagai/)."""

    def __init__(self, precision="fp64", **params):
        super().__init__()
        if params:
            p = kumagai_params(params)
            check(self._L.gb_kumagai_new(ctypes.byref(self._h), ctypes.byref(p)), "Kumagai")
        else:
            check(self._L.gb_kumagai_new(ctypes.byref(self._h), None), "Kumagai")
        self.set_precision(precision)


class TersoffScr(_Potential):
    """Screened Tersoff potential (src/potentials/bop/tersoff/tersoff_scr.f90):
    FP64 only; default parameters Tersoff_PRB_39_5566_Si_C__Scr."""

    def __init__(self, precision="fp64", **params):
        super().__init__()
        base = Tersoff_PRB_39_5566_Si_C__Scr
        p = tersoff_params(params, base)
        sp = screening_params(params, base)
        check(self._L.gb_tersoff_scr_new(ctypes.byref(self._h), ctypes.byref(p),
                                         ctypes.byref(sp)), "TersoffScr")
        self.set_precision(precision)


class KumagaiScr(_Potential):
    """Screened Kumagai potential (src/potentials/bop/kumagai/kumagai_scr.f90):
    FP64 only; default parameters Kumagai_CompMaterSci_39_457_Si__Scr."""

    def __init__(self, precision="fp64", **params):
        super().__init__()
        base = Kumagai_CompMaterSci_39_457_Si__Scr
        p = kumagai_params(params, base)
        sp = screening_params(params, base)
        check(self._L.gb_kumagai_scr_new(ctypes.byref(self._h), ctypes.byref(p),
                                         ctypes.byref(sp)), "KumagaiScr")
        self.set_precision(precision)


class Brenner(_Potential):
    """Brenner-form (Albe-Erhart) bond-order potential
    (src/potentials/bop/brenner/); default Erhart_PRB_71_035211_SiC."""

    def __init__(self, precision="fp64", **params):
        super().__init__()
        if params:
            p = brenner_params(params)
            check(self._L.gb_brenner_new(ctypes.byref(self._h), ctypes.byref(p)), "Brenner")
        else:
            check(self._L.gb_brenner_new(ctypes.byref(self._h), None), "Brenner")
        self.set_precision(precision)


class BrennerScr(_Potential):
    """Screened Brenner potential (src/potentials/bop/brenner/brenner_scr.f90):
    FP64 only; default parameters the compiled-in screened Erhart-Albe Si-C
    set (pass **Erhart_PRB_71_035211_SiC__Scr for the front-end's table)."""

    def __init__(self, precision="fp64", **params):
        super().__init__()
        if params:
            p = brenner_params(params, _BRENNER_SCR_DEFAULT)
            sp = screening_params(params, _BRENNER_SCR_DEFAULT)
            check(self._L.gb_brenner_scr_new(ctypes.byref(self._h), ctypes.byref(p),
                                             ctypes.byref(sp)), "BrennerScr")
        else:
            check(self._L.gb_brenner_scr_new(ctypes.byref(self._h), None, None), "BrennerScr")
        self.set_precision(precision)


class Juslin(_Potential):
    """Juslin-form bond-order potential (src/potentials/bop/juslin/): Brenner's
    functions on ordered element pairs with a three-body h per element
    triplet.  Default: the compiled-in W-C-H set (juslin_params.f90:75-108,
    W-H cutoff 1.95-2.35 A); the front-end's Juslin_JAP_98_123520_WCH
    dictionary has 2.68-2.96 A there."""

    def __init__(self, precision="fp64", **params):
        super().__init__()
        if params:
            p = juslin_params(params)
            check(self._L.gb_juslin_new(ctypes.byref(self._h), ctypes.byref(p)), "Juslin")
        else:
            check(self._L.gb_juslin_new(ctypes.byref(self._h), None), "Juslin")
        self.set_precision(precision)


# The compiled-in default of JuslinScr (juslin_params.f90:95-103 under
# SCREENING): the screened r1, r2 for the outer and bond-order cutoffs too,
# Cmin = 1, Cmax = 3.  The front-end's Juslin_JAP_98_123520_WCH__Scr table
# differs in Cmin and Cmax.
_JUSLIN_SCR_DEFAULT = dict(
    Juslin_JAP_98_123520_WCH,
    or1=list(Juslin_JAP_98_123520_WCH["r1"]), or2=list(Juslin_JAP_98_123520_WCH["r2"]),
    bor1=list(Juslin_JAP_98_123520_WCH["r1"]), bor2=list(Juslin_JAP_98_123520_WCH["r2"]),
    Cmin=[1.0, 1.0, 1.0, 0.0, 1.0, 1.0, 0.0, 1.0, 1.0],
    Cmax=[3.0, 3.0, 3.0, 0.0, 3.0, 3.0, 0.0, 3.0, 3.0])


class JuslinScr(_Potential):
    """Screened Juslin potential (src/potentials/bop/juslin/juslin_scr.f90):
    FP64 only; default parameters the compiled-in screened W-C-H set (pass
    **Juslin_JAP_98_123520_WCH__Scr for the front-end's table)."""

    def __init__(self, precision="fp64", **params):
        super().__init__()
        if params:
            p = juslin_params(params, _JUSLIN_SCR_DEFAULT)
            sp = screening_params(params, _JUSLIN_SCR_DEFAULT)
            check(self._L.gb_juslin_scr_new(ctypes.byref(self._h), ctypes.byref(p),
                                            ctypes.byref(sp)), "JuslinScr")
        else:
            check(self._L.gb_juslin_scr_new(ctypes.byref(self._h), None, None), "JuslinScr")
        self.set_precision(precision)


class TabulatedEAM(_Potential):
    """Single-element tabulated EAM from a DYNAMO funcfl file
    (src/potentials/eam/tabulated_eam.f90)."""

    features = ("per_at",)

    def __init__(self, fn, elements="*"):
        super().__init__()
        check(self._L.gb_tabulated_eam_new(ctypes.byref(self._h), str(fn).encode()),
              "TabulatedEAM")
        self._precision = "fp64"
        self.set_elements(elements)

    def set_elements(self, elements="*"):
        """Element filter (filter_from_string): "*" or comma-separated
        symbols; atoms of other elements are skipped."""
        check(self._L.gb_potential_set_elements(self._h, str(elements or "*").encode()),
              "elements")


class TabulatedAlloyEAM(_Potential):
    """Tabulated alloy EAM from a DYNAMO setfl file
    (src/potentials/eam/tabulated_alloy_eam.f90)."""

    features = ("mask", "per_at")

    def __init__(self, fn, elements="*"):
        super().__init__()
        check(self._L.gb_tabulated_alloy_eam_new(ctypes.byref(self._h),
                                                 str(fn).encode()), "TabulatedAlloyEAM")
        self._precision = "fp64"
        self.set_elements(elements)

    def set_elements(self, elements="*"):
        """Element filter (tabulated_alloy_eam.f90:72, filter_from_string):
        "*" or comma-separated symbols; atoms of other elements are skipped
        as centre and as neighbour."""
        check(self._L.gb_potential_set_elements(self._h, str(elements or "*").encode()),
              "elements")

    def table(self, which, idx):
        """((x0, dx, cut), coefficients (8, n)) of a spline table:
        which = 0 F(rho), 1 rho(r), 2 phi(r) (index i*nel+j)."""
        x = np.zeros(3)
        n = self._L.gb_tabulated_alloy_eam_table(self._h, which, idx, x.ctypes.data, None)
        if n < 0:
            check(n, "table")
        c = np.zeros((8, n))
        self._L.gb_tabulated_alloy_eam_table(self._h, which, idx, x.ctypes.data, c.ctypes.data)
        return x, c


class Batch:
    """Many independent periodic structures evaluated together: one neighbour
    build and one bond-order tile launch for all of them (no counterpart in
    the reference, which evaluates one particles object per call).

    ``structures``: objects with ``positions`` (n,3), ``cell`` (3,3, rows =
    lattice vectors), ``pbc`` (3,) and ``numbers`` (n,) (ASE-like).
    """

    def __init__(self, structures=None):
        self._L = load()
        self._h = ctypes.c_void_p()
        check(self._L.gb_batch_new(ctypes.byref(self._h)), "batch_new")
        self.nat = []
        if structures is not None:
            self.set_structures(structures)

    def __del__(self):
        if getattr(self, "_h", None) and self._h.value:
            self._L.gb_batch_free(self._h)
            self._h = ctypes.c_void_p()

    def __len__(self):
        return len(self.nat)

    def set_stream(self, stream):
        check(self._L.gb_batch_set_stream(self._h, stream), "batch_set_stream")

    def set_options(self, graph=False, autotune=False):
        """CUDA-graph replay of the whole evaluation; tile-size autotuning."""
        check(self._L.gb_batch_set_options(self._h, int(bool(graph)), int(bool(autotune))),
              "batch_set_options")

    def last_info(self):
        """{'replayed', 'tile_bonds' (the bond budget of the tiles),
        'graph_kernels', 'tuned_candidates'} of the last evaluation."""
        v = (ctypes.c_int64 * 4)()
        check(self._L.gb_batch_last_info(self._h, v), "batch_last_info")
        return {"replayed": bool(v[0]), "tile_bonds": int(v[1]),
                "graph_kernels": int(v[2]), "tuned_candidates": int(v[3])}

    def set_structures(self, structures):
        """Cells, pbc flags, atomic numbers and positions of all structures."""
        nat = np.array([len(s.positions) for s in structures], dtype=np.int32)
        cells = np.ascontiguousarray(np.array([np.asarray(s.cell, dtype=np.float64)
                                               for s in structures]).reshape(-1, 3, 3))
        pbc = np.ascontiguousarray(np.array([np.broadcast_to(np.asarray(s.pbc, dtype=bool), (3,))
                                             for s in structures], dtype=np.int32))
        Z = np.ascontiguousarray(np.concatenate([np.asarray(s.numbers, dtype=np.int32)
                                                 for s in structures])
                                 if len(structures) else np.zeros(0, np.int32))
        check(self._L.gb_batch_set_structures(self._h, len(structures), nat.ctypes.data,
                                              cells.ctypes.data, pbc.ctypes.data,
                                              Z.ctypes.data), "batch_set_structures")
        self.nat = [int(n) for n in nat]
        self.offsets = np.concatenate([[0], np.cumsum(nat)]).astype(np.int64)
        r = (np.concatenate([np.asarray(s.positions, dtype=np.float64) for s in structures])
             if len(structures) else np.zeros((0, 3)))
        self.set_positions(r)

    def set_positions(self, r):
        """Positions of all atoms, (total, 3): numpy array or CUDA tensor."""
        ptr, keep = _ptr(r, np.float64)
        self._r = keep
        check(self._L.gb_batch_set_positions(self._h, ptr), "batch_set_positions")

    def md_set_state(self, velocities, masses):
        """Velocities (total, 3) and masses (total,) for md_run (m <= 0
        freezes an atom)."""
        v = np.ascontiguousarray(velocities, dtype=np.float64)
        m = np.ascontiguousarray(masses, dtype=np.float64)
        check(self._L.gb_batch_md_set_state(self._h, v.ctypes.data, m.ctypes.data),
              "batch_md_set_state")

    def md_run(self, pot, dt, nsteps):
        """nsteps velocity-Verlet steps (verlet.f90); (epot (nstruct,),
        wpot (nstruct, 3, 3)) of the last step."""
        e = np.zeros(len(self.nat))
        w = np.zeros((len(self.nat), 3, 3))
        check(self._L.gb_batch_md_run(self._h, pot._h, float(dt), int(nsteps), e.ctypes.data,
                                      w.ctypes.data), "batch_md_run")
        return e, w

    def md_get_state(self):
        """(positions, velocities, forces at the positions), each (total, 3)."""
        n = int(self.offsets[-1]) if len(self.nat) else 0
        r, v, f = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 3))
        check(self._L.gb_batch_md_get_state(self._h, r.ctypes.data, v.ctypes.data,
                                            f.ctypes.data), "batch_md_get_state")
        return r, v, f

    def energy_and_forces(self, pot, forces=None):
        """(epot (nstruct,), forces (total, 3), wpot (nstruct, 3, 3)); forces
        (numpy or CUDA tensor) is accumulated into when given."""
        total = int(self.offsets[-1]) if len(self.nat) else 0
        if forces is None:
            forces = np.zeros((total, 3))
        dev = _is_torch(forces) and forces.is_cuda
        if dev:
            epot = torch.zeros(len(self.nat), dtype=torch.float64, device=forces.device)
            wpot = torch.zeros((len(self.nat), 3, 3), dtype=torch.float64, device=forces.device)
        else:
            epot = np.zeros(len(self.nat))
            wpot = np.zeros((len(self.nat), 3, 3))
        fp, fkeep = _ptr(forces, np.float64)
        ep, ekeep = _ptr(epot, np.float64)
        wp, wkeep = _ptr(wpot, np.float64)
        check(self._L.gb_batch_energy_and_forces(self._h, pot._h, ep, fp, wp),
              "batch_energy_and_forces")
        if fkeep is not forces and not dev:
            forces[...] = fkeep
        return epot, forces, wpot
