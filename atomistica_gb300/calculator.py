"""
ASE-style calculator over the native potentials, mirroring
src/python/atomistica/aseinterface.py (class Atomistica, :143-450).

Works with ASE ``Atoms`` when ASE is installed and with any object exposing
positions / cell / pbc / numbers (e.g. atomistica_gb300.structures.Structure).
Stress is the Voigt form of wpot / V (aseinterface.py:428-433).
"""

import numpy as np

from . import native


def _get(atoms, name):
    g = getattr(atoms, "get_" + name, None)
    if g is not None:
        return np.asarray(g())
    alias = {"atomic_numbers": "numbers"}.get(name, name)
    return np.asarray(getattr(atoms, alias))


def _volume(atoms):
    return abs(np.linalg.det(np.asarray(_get(atoms, "cell"), dtype=float)))


class Atomistica:
    """Calculator: initialize / update / calculate like aseinterface.py."""

    potential_class = None
    avgn = 100
    name = "Atomistica"

    def __init__(self, potentials=None, avgn=None, precision="fp64", **kwargs):
        if potentials is not None:
            self.pots = list(potentials)
        else:
            if self.potential_class in (native.TabulatedAlloyEAM, native.TabulatedEAM):
                self.pots = [self.potential_class(**kwargs)]
            else:
                self.pots = [self.potential_class(precision=precision, **kwargs)]
        if avgn:
            self.avgn = avgn
        self.particles = None
        self.nl = None
        self.mask = None
        self.kwargs = kwargs
        self.compute_epot_per_bond = False
        self.compute_f_per_bond = False
        self.compute_wpot_per_bond = False
        self.epot_per_bond = None
        self.f_per_bond = None
        self.wpot_per_bond = None
        self.results = {}
        self._key = None

    # -- state handling (aseinterface.py:227-329) --
    def initialize(self, atoms):
        if self.mask is not None and len(self.mask) != len(atoms):
            raise RuntimeError("Length of mask array (= %d) does not equal number of atoms "
                               "(= %d)." % (len(self.mask), len(atoms)))
        self.particles = native.Particles()
        self.particles.allocate(len(atoms))
        self.particles.set_cell(_get(atoms, "cell"), _get(atoms, "pbc"))
        self.particles.Z[:] = _get(atoms, "atomic_numbers")
        self.particles.update_elements()
        self.particles.coordinates[:, :] = _get(atoms, "positions")
        self.particles.I_changed_positions()
        self.nl = native.Neighbors(self.avgn)
        for pot in self.pots:
            pot.bind_to(self.particles, self.nl)
        self._key = None

    def update(self, atoms):
        numbers = _get(atoms, "atomic_numbers")
        if self.particles is None or len(self.particles) != len(atoms) or \
                np.any(self.particles.Z != numbers):
            self.initialize(atoms)
        cell = _get(atoms, "cell")
        pbc = _get(atoms, "pbc")
        if np.any(self.particles.cell != cell) or np.any(self.particles.pbc != pbc):
            self.particles.set_cell(cell, pbc)
        pos = _get(atoms, "positions")
        if np.any(self.particles.coordinates != pos):
            self.particles.coordinates[:, :] = pos
            self.particles.I_changed_positions()

    def set_mask(self, mask):
        self.mask = None if mask is None else np.asarray(mask)
        self._key = None

    def set_per_bond(self, epot=None, f=None, wpot=None):
        if epot is not None:
            self.compute_epot_per_bond = epot
        if f is not None:
            self.compute_f_per_bond = f
        if wpot is not None:
            self.compute_wpot_per_bond = wpot
        self._key = None

    def _state_key(self, atoms):
        return (_get(atoms, "positions").tobytes(), _get(atoms, "cell").tobytes(),
                _get(atoms, "pbc").tobytes(), _get(atoms, "atomic_numbers").tobytes(),
                None if self.mask is None else self.mask.tobytes())

    # -- aseinterface.py:355-449 --
    def calculate(self, atoms, properties=("energy",)):
        self.update(atoms)
        epot = 0.0
        forces = np.zeros((len(self.particles), 3))
        wpot = np.zeros((3, 3))
        compute_epot_per_at = "energies" in properties
        compute_wpot_per_at = "stresses" in properties
        kwargs = dict(epot_per_at=compute_epot_per_at, epot_per_bond=self.compute_epot_per_bond,
                      f_per_bond=self.compute_f_per_bond, wpot_per_at=compute_wpot_per_at,
                      wpot_per_bond=self.compute_wpot_per_bond)
        if self.mask is not None:
            kwargs["mask"] = self.mask
        epot_per_at = wpot_per_at = None
        for pot in self.pots:
            if "per_bond" not in pot.features:
                kw = dict(kwargs)
                for k in ("epot_per_bond", "f_per_bond", "wpot_per_bond"):
                    kw[k] = False
            else:
                kw = kwargs
            _epot, _f, _wpot, epa, self.epot_per_bond, self.f_per_bond, wpa, \
                self.wpot_per_bond = pot.energy_and_forces(self.particles, self.nl,
                                                           forces=forces, **kw)
            epot += _epot
            wpot += _wpot
            if epa is not None:
                epot_per_at = epa if epot_per_at is None else epot_per_at + epa
            if wpa is not None:
                wpot_per_at = wpa if wpot_per_at is None else wpot_per_at + wpa
        volume = _volume(atoms)
        self.results = {
            "energy": epot, "free_energy": epot, "forces": forces,
            "stress": np.array([wpot[0, 0], wpot[1, 1], wpot[2, 2],
                                (wpot[1, 2] + wpot[2, 1]) / 2, (wpot[0, 2] + wpot[2, 0]) / 2,
                                (wpot[0, 1] + wpot[1, 0]) / 2]) / volume,
            "virial": wpot,
        }
        if compute_epot_per_at:
            self.results["energies"] = epot_per_at
        if compute_wpot_per_at:
            w = wpot_per_at
            self.results["stresses"] = np.transpose([
                w[:, 0, 0], w[:, 1, 1], w[:, 2, 2], (w[:, 1, 2] + w[:, 2, 1]) / 2,
                (w[:, 0, 2] + w[:, 2, 0]) / 2, (w[:, 0, 1] + w[:, 1, 0]) / 2])
        self._key = (self._state_key(atoms), tuple(sorted(properties)))

    def _ensure(self, atoms, prop):
        props = ("energy", prop) if prop not in ("energy",) else ("energy",)
        key = (self._state_key(atoms), tuple(sorted(props)))
        if self._key != key or prop not in self.results:
            self.calculate(atoms, props)
        return self.results[prop]

    def get_potential_energy(self, atoms):
        return self._ensure(atoms, "energy")

    def get_forces(self, atoms):
        return self._ensure(atoms, "forces").copy()

    def get_stress(self, atoms):
        return self._ensure(atoms, "stress").copy()

    def get_potential_energies(self, atoms):
        return self._ensure(atoms, "energies").copy()

    def get_stresses(self, atoms):
        return self._ensure(atoms, "stresses").copy()

    def get_neighbors(self):
        return self.nl.get_neighbors(self.particles)


class Tersoff(Atomistica):
    name = "Tersoff"
    potential_class = native.Tersoff


class Kumagai(Atomistica):
    name = "Kumagai"
    potential_class = native.Kumagai


class TersoffScr(Atomistica):
    name = "TersoffScr"
    potential_class = native.TersoffScr


class KumagaiScr(Atomistica):
    name = "KumagaiScr"
    potential_class = native.KumagaiScr


class Brenner(Atomistica):
    name = "Brenner"
    potential_class = native.Brenner


class BrennerScr(Atomistica):
    name = "BrennerScr"
    potential_class = native.BrennerScr


class Juslin(Atomistica):
    name = "Juslin"
    potential_class = native.Juslin


class JuslinScr(Atomistica):
    name = "JuslinScr"
    potential_class = native.JuslinScr


class TabulatedEAM(Atomistica):
    name = "TabulatedEAM"
    potential_class = native.TabulatedEAM


class TabulatedAlloyEAM(Atomistica):
    name = "TabulatedAlloyEAM"
    potential_class = native.TabulatedAlloyEAM
