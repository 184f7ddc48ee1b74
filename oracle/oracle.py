"""
TEST INFRASTRUCTURE ONLY — ctypes wrapper around the C++ FP64 oracle
(oracle/oracle.cpp).  Imported by tests/ and by bench.py's CPU-baseline leg;
never by the atomistica_gb300 package.

The oracle restates Atomistica's neighbour build (python_neighbors.f90),
the Tersoff/Kumagai/Brenner BOP kernel (bop_kernel.f90 + *_func.f90) and the tabulated
alloy EAM (tabulated_alloy_eam.f90 + simple_spline.f90); see oracle.cpp for
line citations.  Output layouts follow src/python/c/potential.c:446-611:
f (nat,3), wpot (3,3) with wpot[a,c] = W(a,c), wpot_per_at (nat,3,3) with
wpot_per_at[i,x,y] = W_i(y,x).
"""

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "liboracle.so")
_SRC = os.path.join(_HERE, "oracle.cpp")

_lib = None


def build(force=False):
    """Compile oracle.cpp into liboracle.so (g++, OpenMP, no FP contraction)."""
    if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < os.path.getmtime(_SRC):
        cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC",
               "-shared", _SRC, "-o", _LIB]
        subprocess.check_call(cmd)
    return _LIB


class TersoffParams(ctypes.Structure):
    _fields_ = [("nel", ctypes.c_int), ("Z", ctypes.c_int * 3)] + \
        [(k, ctypes.c_double * 6) for k in ("A", "B", "xi", "lambda_", "mu", "omega", "mubo")] + \
        [("m", ctypes.c_int * 6)] + \
        [(k, ctypes.c_double * 3) for k in ("beta", "n", "c", "d", "h")] + \
        [("r1", ctypes.c_double * 6), ("r2", ctypes.c_double * 6)]


class KumagaiParams(ctypes.Structure):
    _fields_ = [("nel", ctypes.c_int), ("Z", ctypes.c_int * 1)] + \
        [(k, ctypes.c_double * 1) for k in ("A", "B", "lambda1", "lambda2", "eta", "delta",
                                            "alpha")] + \
        [("beta", ctypes.c_int * 1)] + \
        [(k, ctypes.c_double * 1) for k in ("c1", "c2", "c3", "c4", "c5", "h", "r1", "r2")]


class BrennerParams(ctypes.Structure):
    _fields_ = [("nel", ctypes.c_int), ("Z", ctypes.c_int * 3)] + \
        [(k, ctypes.c_double * 6) for k in ("D0", "r0", "S", "beta", "gamma", "c", "d", "h",
                                            "mu", "n")] + \
        [("m", ctypes.c_int * 6), ("r1", ctypes.c_double * 6), ("r2", ctypes.c_double * 6)]


class JuslinParams(ctypes.Structure):
    _fields_ = [("nel", ctypes.c_int), ("Z", ctypes.c_int * 3)] + \
        [(k, ctypes.c_double * 9) for k in ("D0", "r0", "S", "beta", "gamma", "c", "d", "h",
                                            "n")] + \
        [("alpha", ctypes.c_double * 27), ("omega", ctypes.c_double * 27),
         ("m", ctypes.c_int * 27), ("r1", ctypes.c_double * 9), ("r2", ctypes.c_double * 9)]


class ScrParams(ctypes.Structure):
    """Screened variants: outer / bond-order cutoffs and the screening window
    (tersoff_params.f90:81-90, kumagai_params.f90 under SCREENING), one entry
    per element pair (nine for Juslin's ordered pairs)."""
    _fields_ = [(k, ctypes.c_double * 9) for k in ("or1", "or2", "bor1", "bor2", "Cmin",
                                                   "Cmax")]


def scr_params(d):
    p = ScrParams()
    n = len(d["or1"])
    for k in ("or1", "or2", "bor1", "bor2", "Cmin", "Cmax"):
        arr = getattr(p, k)
        for q in range(n):
            arr[q] = float(d[k][q])
    return p


def _kind(kind):
    """(base kind, screened?) of 'tersoff', 'kumagai', 'brenner', 'juslin'
    and their '_scr' forms."""
    base = kind[:-4] if kind.endswith("_scr") else kind
    if base not in ("tersoff", "kumagai", "brenner", "juslin"):
        raise ValueError("unknown bond-order potential %r" % kind)
    return base, kind.endswith("_scr")


_KIND_ID = {"tersoff": 0, "kumagai": 1, "brenner": 2, "juslin": 3}


def _params(base, d):
    return {"tersoff": tersoff_params, "kumagai": kumagai_params,
            "brenner": brenner_params, "juslin": juslin_params}[base](d)


def _Z(sym):
    from atomistica_gb300.parameters import atomic_numbers
    return atomic_numbers[sym]


def tersoff_params(d):
    p = TersoffParams()
    els = d["el"]
    p.nel = len(els)
    for q, s in enumerate(els):
        p.Z[q] = _Z(s)
    npair = p.nel * (p.nel + 1) // 2
    defaults = {"xi": 1.0, "omega": 1.0, "mubo": 0.0}
    for k in ("A", "B", "xi", "lambda", "mu", "omega", "mubo", "r1", "r2"):
        arr = getattr(p, "lambda_" if k == "lambda" else k)
        vals = d.get(k, [defaults.get(k, 1.0)] * npair)
        for q in range(npair):
            arr[q] = float(vals[q])
    ms = d.get("m", [1] * npair)
    for q in range(npair):
        p.m[q] = int(ms[q])
    for k in ("beta", "n", "c", "d", "h"):
        arr = getattr(p, k)
        for q in range(p.nel):
            arr[q] = float(d[k][q])
    return p


def kumagai_params(d):
    p = KumagaiParams()
    p.nel = 1
    p.Z[0] = _Z(d["el"][0])
    for k in ("A", "B", "lambda1", "lambda2", "eta", "delta", "alpha", "c1", "c2", "c3",
              "c4", "c5", "h", "r1", "r2"):
        getattr(p, k)[0] = float(d[k][0])
    p.beta[0] = int(d["beta"][0])
    return p


def brenner_params(d):
    p = BrennerParams()
    els = d["el"]
    p.nel = len(els)
    for q, s in enumerate(els):
        p.Z[q] = _Z(s)
    npair = p.nel * (p.nel + 1) // 2
    for k in ("D0", "r0", "S", "beta", "gamma", "c", "d", "h", "mu", "n", "r1", "r2"):
        arr = getattr(p, k)
        for q in range(npair):
            arr[q] = float(d[k][q])
    for q in range(npair):
        p.m[q] = int(d["m"][q])
    return p


def juslin_params(d):
    """Juslin set: pair arrays of nel^2 ordered pairs, alpha / omega / m of
    nel^3 triplets (m defaults to 1, as the reference's Python sets leave it
    to the compiled-in table)."""
    p = JuslinParams()
    els = d["el"]
    p.nel = len(els)
    for q, s in enumerate(els):
        p.Z[q] = _Z(s)
    npair = p.nel * p.nel
    for k in ("D0", "r0", "S", "beta", "gamma", "c", "d", "h", "n", "r1", "r2"):
        arr = getattr(p, k)
        for q in range(npair):
            arr[q] = float(d[k][q])
    ms = d.get("m", [1] * npair * p.nel)
    for q in range(npair * p.nel):
        p.alpha[q] = float(d["alpha"][q])
        p.omega[q] = float(d["omega"][q])
        p.m[q] = int(ms[q])
    return p


_P = ctypes.c_void_p


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB)
        L.orc_neighbors_build.restype = _P
        L.orc_neighbors_build.argtypes = [ctypes.c_int, _P, _P, _P, ctypes.c_double]
        L.orc_neighbors_size.restype = ctypes.c_int64
        L.orc_neighbors_size.argtypes = [_P]
        L.orc_neighbors_copy.argtypes = [_P, _P, _P, _P]
        L.orc_neighbors_free.argtypes = [_P]
        L.orc_cell_inverse.argtypes = [_P, _P]
        for name in ("orc_tersoff_cutoff", "orc_kumagai_cutoff", "orc_brenner_cutoff",
                     "orc_juslin_cutoff"):
            getattr(L, name).restype = ctypes.c_double
            getattr(L, name).argtypes = [_P, ctypes.c_int, _P]
        kargs = [_P, ctypes.c_int, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P,
                 _P, _P, ctypes.c_int]
        for name in ("orc_tersoff_kernel", "orc_kumagai_kernel", "orc_brenner_kernel",
                     "orc_juslin_kernel"):
            getattr(L, name).restype = ctypes.c_int
            getattr(L, name).argtypes = kargs
        cargs = [_P, ctypes.c_int, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, ctypes.c_int]
        for name in ("orc_tersoff_compute", "orc_kumagai_compute", "orc_brenner_compute",
                     "orc_juslin_compute"):
            getattr(L, name).restype = ctypes.c_int
            getattr(L, name).argtypes = cargs
        for name in ("orc_tersoff_scr_cutoff", "orc_kumagai_scr_cutoff",
                     "orc_brenner_scr_cutoff", "orc_juslin_scr_cutoff"):
            getattr(L, name).restype = ctypes.c_double
            getattr(L, name).argtypes = [_P, _P, ctypes.c_int, _P]
        for name in ("orc_tersoff_scr_kernel", "orc_kumagai_scr_kernel",
                     "orc_brenner_scr_kernel", "orc_juslin_scr_kernel"):
            getattr(L, name).restype = ctypes.c_int
            getattr(L, name).argtypes = [_P] + kargs
        for name in ("orc_tersoff_scr_compute", "orc_kumagai_scr_compute",
                     "orc_brenner_scr_compute", "orc_juslin_scr_compute"):
            getattr(L, name).restype = ctypes.c_int
            getattr(L, name).argtypes = [_P] + cargs
        L.orc_bop_ghost.restype = ctypes.c_int
        L.orc_bop_ghost.argtypes = [ctypes.c_int, _P, _P, ctypes.c_int, ctypes.c_int, _P, _P, _P,
                                    _P, _P, _P, _P, _P, _P, _P, ctypes.c_int]
        L.orc_funcfl_load.restype = _P
        L.orc_funcfl_load.argtypes = [ctypes.c_char_p, _P]
        L.orc_funcfl_free.argtypes = [_P]
        L.orc_funcfl_cutoff.restype = ctypes.c_double
        L.orc_funcfl_cutoff.argtypes = [_P]
        L.orc_funcfl_compute.restype = ctypes.c_int
        L.orc_funcfl_compute.argtypes = [_P, ctypes.c_int, _P, _P, _P, _P, _P, _P, _P,
                                         ctypes.c_int]
        L.orc_eam_load.restype = _P
        L.orc_eam_load.argtypes = [ctypes.c_char_p, _P]
        L.orc_eam_free.argtypes = [_P]
        L.orc_eam_cutoff.restype = ctypes.c_double
        L.orc_eam_cutoff.argtypes = [_P]
        L.orc_eam_nel.restype = ctypes.c_int
        L.orc_eam_nel.argtypes = [_P]
        L.orc_eam_table.restype = ctypes.c_int
        L.orc_eam_table.argtypes = [_P, ctypes.c_int, ctypes.c_int, _P, _P]
        L.orc_eam_kernel.restype = ctypes.c_int
        L.orc_eam_kernel.argtypes = [_P, ctypes.c_int, _P, _P, _P, _P, _P, _P, _P, _P, _P,
                                     _P, _P, _P, _P, ctypes.c_int]
        L.orc_eam_compute.restype = ctypes.c_int
        L.orc_eam_compute.argtypes = [_P, ctypes.c_int, _P, _P, _P, _P, _P, _P, _P, _P, _P,
                                      _P, ctypes.c_int]
        L.orc_max_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data


def _geom(s):
    r = np.ascontiguousarray(s.positions, dtype=np.float64)
    cell = np.ascontiguousarray(s.cell, dtype=np.float64)
    pbc = np.ascontiguousarray(np.asarray(s.pbc).astype(np.int32))
    Z = np.ascontiguousarray(s.numbers, dtype=np.int32)
    return r, cell, pbc, Z


class NeighborList:
    """Full directed neighbour list: CSR ``seed`` (nat+1), ``nbr`` and
    integer image shifts ``dc`` (n, 3), in the reference's per-atom order."""

    def __init__(self, seed, nbr, dc):
        self.seed, self.nbr, self.dc = seed, nbr, dc

    @property
    def i(self):
        return np.repeat(np.arange(len(self.seed) - 1, dtype=np.int32), np.diff(self.seed))

    def triples(self):
        """Sorted (i, j, s0, s1, s2) rows for set comparison."""
        t = np.column_stack([self.i, self.nbr, self.dc]).astype(np.int64)
        order = np.lexsort(t.T[::-1])
        return t[order]


def neighbors(s, cutoff):
    L = lib()
    r, cell, pbc, _ = _geom(s)
    h = L.orc_neighbors_build(len(r), _ptr(r), _ptr(cell), _ptr(pbc), float(cutoff))
    if not h:
        raise RuntimeError("oracle: singular cell")
    try:
        n = L.orc_neighbors_size(h)
        seed = np.zeros(len(r) + 1, dtype=np.int64)
        nbr = np.zeros(max(n, 1), dtype=np.int32)
        dc = np.zeros((max(n, 1), 3), dtype=np.int32)
        L.orc_neighbors_copy(h, _ptr(seed), _ptr(nbr), _ptr(dc))
    finally:
        L.orc_neighbors_free(h)
    return NeighborList(seed, nbr[:n], dc[:n])


def cell_inverse(cell):
    out = np.zeros((3, 3))
    c = np.ascontiguousarray(cell, dtype=np.float64)
    lib().orc_cell_inverse(_ptr(c), _ptr(out))
    return out


def _alloc_outputs(nat, nb, per_at, per_bond):
    f = np.zeros((nat, 3))
    wpot = np.zeros((3, 3), order="F")
    out = dict(f=f, wpot=wpot)
    if per_at:
        out["epot_per_at"] = np.zeros(nat)
        out["wpot_per_at"] = np.zeros((nat, 3, 3))
    if per_bond:
        out["epot_per_bond"] = np.zeros(nb)
        out["f_per_bond"] = np.zeros((nb, 3))
        out["wpot_per_bond"] = np.zeros((nb, 3, 3))
    return out


def bop_cutoff(kind, params, s):
    """Interaction range requested by bind_to for the elements of s."""
    L = lib()
    _, _, _, Z = _geom(s)
    base, scr = _kind(kind)
    p = _params(base, params)
    pre = (ctypes.byref(p), ctypes.byref(scr_params(params))) if scr else (ctypes.byref(p),)
    return getattr(L, "orc_%s_cutoff" % kind)(*pre, len(Z), _ptr(Z))


def bop(kind, params, s, nl=None, mask=None, per_at=True, per_bond=False, nthreads=0):
    """Tersoff or Kumagai energy_and_forces.  Returns a dict with epot, f,
    wpot, [epot_per_at, wpot_per_at], [epot_per_bond, f_per_bond,
    wpot_per_bond] and the neighbour list used."""
    L = lib()
    r, cell, pbc, Z = _geom(s)
    nat = len(r)
    base, scr = _kind(kind)
    p = _params(base, params)
    pre = (ctypes.byref(p), ctypes.byref(scr_params(params))) if scr else (ctypes.byref(p),)
    if nl is None:
        cut = getattr(L, "orc_%s_cutoff" % kind)(*pre, nat, _ptr(Z))
        nl = neighbors(s, cut) if cut > 0 else NeighborList(
            np.zeros(nat + 1, np.int64), np.zeros(0, np.int32), np.zeros((0, 3), np.int32))
    out = _alloc_outputs(nat, len(nl.nbr), per_at, per_bond)
    epot = ctypes.c_double(0.0)
    m = None if mask is None else np.ascontiguousarray(np.asarray(mask).astype(np.int32))
    nbr = nl.nbr if len(nl.nbr) else np.zeros(1, np.int32)
    dc = np.ascontiguousarray(nl.dc) if len(nl.nbr) else np.zeros((1, 3), np.int32)
    rc = getattr(L, "orc_%s_kernel" % kind)(
        *pre, nat, _ptr(r), _ptr(cell), _ptr(pbc), _ptr(Z), _ptr(nl.seed),
        _ptr(nbr), _ptr(dc), _ptr(m), ctypes.byref(epot), _ptr(out["f"]),
        _ptr(out["wpot"]), _ptr(out.get("epot_per_at")), _ptr(out.get("epot_per_bond")),
        _ptr(out.get("f_per_bond")), _ptr(out.get("wpot_per_at")),
        _ptr(out.get("wpot_per_bond")), int(nthreads))
    if rc != 0:
        raise RuntimeError("oracle bop kernel failed: %d" % rc)
    out["epot"] = epot.value
    out["wpot"] = np.ascontiguousarray(out["wpot"])
    out["nl"] = nl
    return out


def bop_ghost(kind, params, r, Z, seed, nbr, natloc, mask=None, nthreads=0):
    """The LAMMPS contract: explicit local + ghost positions, a shift-free
    CSR list over all atoms, bonds of the first natloc atoms; returns epot,
    f, wpot, epot_per_at, wpot_per_at for all atoms."""
    L = lib()
    base, scr = _kind(kind)
    p = _params(base, params)
    sp = scr_params(params) if scr else None
    r = np.ascontiguousarray(r, dtype=np.float64)
    nat = len(r)
    Z = np.ascontiguousarray(Z, dtype=np.int32)
    seed = np.ascontiguousarray(seed, dtype=np.int64)
    nbr = np.ascontiguousarray(nbr, dtype=np.int32) if len(nbr) else np.zeros(1, np.int32)
    out = _alloc_outputs(nat, 0, True, False)
    epot = ctypes.c_double(0.0)
    m = None if mask is None else np.ascontiguousarray(np.asarray(mask).astype(np.int32))
    rc = L.orc_bop_ghost(_KIND_ID[base], ctypes.byref(p),
                         ctypes.byref(sp) if sp is not None else None, nat, int(natloc),
                         _ptr(r), _ptr(Z), _ptr(seed), _ptr(nbr), _ptr(m), ctypes.byref(epot),
                         _ptr(out["f"]), _ptr(out["wpot"]), _ptr(out["epot_per_at"]),
                         _ptr(out["wpot_per_at"]), int(nthreads))
    if rc != 0:
        raise RuntimeError("oracle ghost kernel failed: %d" % rc)
    out["epot"] = epot.value
    out["wpot"] = np.ascontiguousarray(out["wpot"])
    return out


def bop_compute(kind, params, s, mask=None, per_at=False, nthreads=0):
    """Neighbour build + kernel in one call (the CPU baseline's timed unit)."""
    L = lib()
    r, cell, pbc, Z = _geom(s)
    nat = len(r)
    base, scr = _kind(kind)
    p = _params(base, params)
    pre = (ctypes.byref(p), ctypes.byref(scr_params(params))) if scr else (ctypes.byref(p),)
    out = _alloc_outputs(nat, 0, per_at, False)
    epot = ctypes.c_double(0.0)
    m = None if mask is None else np.ascontiguousarray(np.asarray(mask).astype(np.int32))
    rc = getattr(L, "orc_%s_compute" % kind)(
        *pre, nat, _ptr(r), _ptr(cell), _ptr(pbc), _ptr(Z), _ptr(m),
        ctypes.byref(epot), _ptr(out["f"]), _ptr(out["wpot"]), _ptr(out.get("epot_per_at")),
        _ptr(out.get("wpot_per_at")), int(nthreads))
    if rc != 0:
        raise RuntimeError("oracle bop compute failed: %d" % rc)
    out["epot"] = epot.value
    out["wpot"] = np.ascontiguousarray(out["wpot"])
    return out


class FuncflEAM:
    """Single-element funcfl EAM oracle (TabulatedEAM, tabulated_eam.f90)."""

    def __init__(self, fn):
        L = lib()
        err = ctypes.c_int(0)
        self._h = L.orc_funcfl_load(os.fsencode(fn), ctypes.byref(err))
        if not self._h:
            raise RuntimeError("oracle: cannot read funcfl %s (%d)" % (fn, err.value))
        self.cutoff = L.orc_funcfl_cutoff(self._h)

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.orc_funcfl_free(self._h)
            self._h = None

    def compute(self, s, per_at=True, nthreads=0):
        L = lib()
        r, cell, pbc, Z = _geom(s)
        nat = len(r)
        out = _alloc_outputs(nat, 0, per_at, False)
        epot = ctypes.c_double(0.0)
        rc = L.orc_funcfl_compute(self._h, nat, _ptr(r), _ptr(cell), _ptr(pbc),
                                  ctypes.byref(epot), _ptr(out["f"]), _ptr(out["wpot"]),
                                  _ptr(out.get("epot_per_at")), int(nthreads))
        if rc != 0:
            raise RuntimeError("oracle funcfl kernel failed: %d" % rc)
        out["epot"] = epot.value
        out["wpot"] = np.ascontiguousarray(out["wpot"])
        return out


class EAM:
    """Tabulated alloy EAM oracle (setfl file)."""

    def __init__(self, fn):
        L = lib()
        err = ctypes.c_int(0)
        self._h = L.orc_eam_load(os.fsencode(fn), ctypes.byref(err))
        if not self._h:
            raise RuntimeError("oracle: cannot read setfl %s (%d)" % (fn, err.value))
        self.cutoff = L.orc_eam_cutoff(self._h)
        self.nel = L.orc_eam_nel(self._h)

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.orc_eam_free(self._h)
            self._h = None

    def table(self, which, idx):
        """(x0, dx, cut), coefficient array (8, n): y, d2y, c1..c3, d1..d3."""
        L = lib()
        x = np.zeros(3)
        n = L.orc_eam_table(self._h, which, idx, _ptr(x), None)
        c = np.zeros((8, n))
        L.orc_eam_table(self._h, which, idx, _ptr(x), _ptr(c))
        return x, c

    def compute(self, s, nl=None, mask=None, per_at=True, nthreads=0, elements=None):
        """elements: None / "*" or a list of atomic numbers (the element
        filter, tabulated_alloy_eam.f90:316-335: atoms of other elements are
        skipped as i and as j, exactly as atoms of elements the file has no
        parameters for, so they are given Z = 0 here)."""
        L = lib()
        r, cell, pbc, Z = _geom(s)
        if elements not in (None, "*"):
            Z = np.ascontiguousarray(np.where(np.isin(Z, list(elements)), Z, 0).astype(np.int32))
        nat = len(r)
        if nl is None:
            nl = neighbors(s, self.cutoff)
        out = _alloc_outputs(nat, 0, per_at, False)
        epot = ctypes.c_double(0.0)
        m = None if mask is None else np.ascontiguousarray(np.asarray(mask).astype(np.int32))
        nbr = nl.nbr if len(nl.nbr) else np.zeros(1, np.int32)
        dc = np.ascontiguousarray(nl.dc) if len(nl.nbr) else np.zeros((1, 3), np.int32)
        rc = L.orc_eam_kernel(self._h, nat, _ptr(r), _ptr(cell), _ptr(pbc), _ptr(Z),
                              _ptr(nl.seed), _ptr(nbr), _ptr(dc), _ptr(m),
                              ctypes.byref(epot), _ptr(out["f"]), _ptr(out["wpot"]),
                              _ptr(out.get("epot_per_at")), _ptr(out.get("wpot_per_at")),
                              int(nthreads))
        if rc != 0:
            raise RuntimeError("oracle eam kernel failed: %d" % rc)
        out["epot"] = epot.value
        out["wpot"] = np.ascontiguousarray(out["wpot"])
        out["nl"] = nl
        return out

    def compute_full(self, s, mask=None, per_at=False, nthreads=0):
        L = lib()
        r, cell, pbc, Z = _geom(s)
        nat = len(r)
        out = _alloc_outputs(nat, 0, per_at, False)
        epot = ctypes.c_double(0.0)
        m = None if mask is None else np.ascontiguousarray(np.asarray(mask).astype(np.int32))
        rc = L.orc_eam_compute(self._h, nat, _ptr(r), _ptr(cell), _ptr(pbc), _ptr(Z), _ptr(m),
                               ctypes.byref(epot), _ptr(out["f"]), _ptr(out["wpot"]),
                               _ptr(out.get("epot_per_at")), _ptr(out.get("wpot_per_at")),
                               int(nthreads))
        if rc != 0:
            raise RuntimeError("oracle eam compute failed: %d" % rc)
        out["epot"] = epot.value
        out["wpot"] = np.ascontiguousarray(out["wpot"])
        return out


def max_threads():
    return lib().orc_max_threads()
