"""
Crystal builders and the seeded synthetic workloads of the force-path
benchmarks.

``Structure`` is a minimal stand-in for an ASE ``Atoms`` object: positions
(nat, 3) in Angstrom, cell rows = lattice vectors, pbc flags and atomic
numbers.  The builders reproduce the conventional cubic cells used by the
reference's tests (ase.lattice.cubic.Diamond / FaceCenteredCubic); atom order
within the supercell does not affect any energy, force or virial.
"""

import os
from dataclasses import dataclass, field

import numpy as np

from .parameters import atomic_numbers

AVOGADRO = 6.02214076e23
MASS_SI = 28.0855


@dataclass
class Structure:
    positions: np.ndarray
    cell: np.ndarray
    pbc: np.ndarray
    numbers: np.ndarray
    info: dict = field(default_factory=dict)

    def __len__(self):
        return len(self.positions)

    def copy(self):
        return Structure(self.positions.copy(), self.cell.copy(), self.pbc.copy(),
                         self.numbers.copy(), dict(self.info))

    def get_volume(self):
        return abs(np.linalg.det(self.cell))

    def set_cell(self, cell, scale_atoms=False):
        cell = np.asarray(cell, dtype=float)
        if cell.shape == (3,):
            cell = np.diag(cell)
        if scale_atoms:
            frac = np.linalg.solve(self.cell.T, self.positions.T).T
            self.positions = frac @ cell
        self.cell = cell.copy()

    def get_scaled_positions(self):
        return np.linalg.solve(self.cell.T, self.positions.T).T


_DIAMOND = np.array([[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0],
                     [.25, .25, .25], [.25, .75, .75], [.75, .25, .75], [.75, .75, .25]])
_FCC = np.array([[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0]])


def _lattice(basis, symbol, a, size):
    nx, ny, nz = size
    grid = np.stack(np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz),
                                indexing="ij"), axis=-1).reshape(-1, 3)
    frac = (grid[:, None, :] + basis[None, :, :]).reshape(-1, 3)
    pos = frac * a
    cell = np.diag([nx * a, ny * a, nz * a]).astype(float)
    z = atomic_numbers[symbol] if isinstance(symbol, str) else int(symbol)
    return Structure(pos.astype(float), cell, np.array([True, True, True]),
                     np.full(len(pos), z, dtype=np.int32))


def diamond(symbol="Si", a=5.431, size=(1, 1, 1)):
    """Diamond-cubic supercell, 8 atoms per conventional cell."""
    return _lattice(_DIAMOND, symbol, a, size)


def fcc(symbol="Cu", a=3.615, size=(1, 1, 1)):
    """Face-centred cubic supercell, 4 atoms per conventional cell."""
    return _lattice(_FCC, symbol, a, size)


def bcc(symbol="Fe", a=2.87, size=(1, 1, 1)):
    """Body-centred cubic supercell, 2 atoms per conventional cell."""
    return _lattice(np.array([[0, 0, 0], [.5, .5, .5]]), symbol, a, size)


def sc(symbol="Fe", a=2.4, size=(1, 1, 1)):
    """Simple cubic supercell, 1 atom per cell."""
    return _lattice(np.array([[0, 0, 0]]), symbol, a, size)


def b1(symbols=("Fe", "C"), a=3.9, size=(1, 1, 1)):
    """Rock-salt (B1) supercell: first symbol on the fcc sites, second on the
    fcc sites shifted by a/2 along x."""
    basis = np.concatenate([_FCC, (_FCC + np.array([.5, 0, 0])) % 1.0])
    s = _lattice(basis, symbols[0], a, size)
    s.numbers[np.arange(len(s)) % len(basis) >= 4] = atomic_numbers[symbols[1]]
    return s


def b2(symbols=("W", "C"), a=2.7, size=(1, 1, 1)):
    """CsCl (B2) supercell: first symbol at the cube corners, second at the
    centre."""
    s = bcc(symbols[0], a, size)
    s.numbers[np.arange(len(s)) % 2 == 1] = atomic_numbers[symbols[1]]
    return s


def b3(symbols=("Si", "C"), a=4.3596, size=(1, 1, 1)):
    """Zinc-blende (B3) supercell: first symbol on the fcc sites."""
    s = diamond(symbols[0], a, size)
    z2 = atomic_numbers[symbols[1]]
    nb = len(_DIAMOND)
    idx = np.arange(len(s)) % nb >= 4
    s.numbers[idx] = z2
    return s


# ---------------------------------------------------------------------------
# Benchmark workloads (seeded).
# ---------------------------------------------------------------------------

def si_number_density(rho_gcc=2.33):
    """Atoms per cubic Angstrom of Si at mass density ``rho_gcc``."""
    return rho_gcc * AVOGADRO / MASS_SI / 1e24


def tersoff_si_4096(seed=1):
    """Diamond Si, a=5.431, 8x8x8 cells (4096 atoms), uniform +-0.1 A noise."""
    rng = np.random.default_rng(seed)
    s = diamond("Si", 5.431, (8, 8, 8))
    s.positions += rng.uniform(-0.1, 0.1, size=s.positions.shape)
    s.info.update(workload="tersoff_si_4096", seed=seed)
    return s


def amorphous_carbon(nat=4096, density=3.0, seed=7, dmin=1.2):
    """Random carbon packing at ``density`` g/cm^3 (cubic box, minimum
    separation ``dmin`` over all images): a stand-in for amorphous carbon
    such as the reference's aC.cfg."""
    rng = np.random.default_rng(seed)
    L = (nat * 12.011 / (density * 6.02214076e23) * 1e24) ** (1.0 / 3.0)
    cell = np.eye(3) * L
    pos = _random_packing(rng, nat, cell, dmin)
    return Structure(pos, cell, np.array([True, True, True]), np.full(nat, 6, dtype=np.int32),
                     {"workload": "amorphous_carbon", "seed": seed, "density_gcc": density})


def eam_cu_131072(seed=2):
    """FCC Cu, a=3.615, 32^3 cells (131072 atoms), Gaussian sigma=0.05 A."""
    rng = np.random.default_rng(seed)
    s = fcc("Cu", 3.615, (32, 32, 32))
    s.positions += rng.normal(0.0, 0.05, size=s.positions.shape)
    s.info.update(workload="eam_cu_131072", seed=seed)
    return s


def tersoff_si_amorphous(natoms=1048576, seed=3, sigma=0.25, rho_gcc=2.33):
    """Si block of ``natoms`` atoms at ``rho_gcc`` in a cubic periodic box.

    Diamond sites of the smallest m^3 supercell holding ``natoms`` sites are
    scaled to the box edge L = (natoms/n)^(1/3) for the number density n; a
    seeded random subset of surplus sites is deleted so that exactly
    ``natoms`` remain, and each coordinate gets Gaussian noise ``sigma``.
    For natoms = 2^20: m = 51 (1,061,208 sites), 12,632 deleted, a = 5.410 A.
    """
    rng = np.random.default_rng(seed)
    n = si_number_density(rho_gcc)
    L = (natoms / n) ** (1.0 / 3.0)
    m = int(np.ceil((natoms / 8.0) ** (1.0 / 3.0) - 1e-9))
    while 8 * m ** 3 < natoms:
        m += 1
    s = diamond("Si", L / m, (m, m, m))
    nsites = len(s)
    keep = np.sort(rng.permutation(nsites)[:natoms])
    s.positions = s.positions[keep]
    s.numbers = s.numbers[keep]
    s.positions += rng.normal(0.0, sigma, size=s.positions.shape)
    s.info.update(workload="tersoff_si_amorphous_%d" % natoms, seed=seed,
                  sites=nsites, deleted=nsites - natoms, a=L / m, L=L)
    return s


def random_wch(nat=96, seed=0, frac=(0.4, 0.35, 0.25), density=3.0, dmin=1.1):
    """Random W-C-H packing: a random packing at the carbon number density of
    ``density`` g/cm^3 whose species are drawn W / C / H with the given
    fractions, so that every ordered pair and element triplet of the Juslin
    sets occurs."""
    s = amorphous_carbon(nat, density=density, seed=seed, dmin=dmin)
    rng = np.random.default_rng(seed + 1000)
    s.numbers = rng.choice([74, 6, 1], size=nat, p=list(frac)).astype(np.int32)
    return s


def _random_packing(rng, nat, cell, dmin, max_tries=50000000):
    """Uniform positions in ``cell`` with every pair (all periodic images)
    separated by at least ``dmin``: random sequential addition in the
    library's host code (gb_random_packing), seeded from ``rng``."""
    from . import _lib
    if not os.path.exists(_lib.LIB_PATH):
        from .build import build
        build()
    seed = int(rng.integers(0, 2 ** 63))
    cell = np.ascontiguousarray(cell, dtype=np.float64)
    pos = np.empty((nat, 3))
    _lib.check(_lib.load().gb_random_packing(int(nat), cell.ctypes.data, float(dmin), seed,
                                   int(max_tries), pos.ctypes.data), "random_packing")
    return pos


def si_batch(nstruct=2048, nmin=8, nmax=512, seed=4, strain=0.08, dmin=2.0,
             rho_gcc=2.33):
    """Independent triclinic Si structures: N ~ U{nmin..nmax}, cubic box for
    ``rho_gcc`` strained by (I+eps) with eps_ij ~ U(-strain, strain), uniform
    positions under a ``dmin`` minimum separation over all images."""
    rng = np.random.default_rng(seed)
    n = si_number_density(rho_gcc)
    out = []
    for s in range(nstruct):
        nat = int(rng.integers(nmin, nmax + 1))
        L = (nat / n) ** (1.0 / 3.0)
        eps = rng.uniform(-strain, strain, size=(3, 3))
        cell = (np.eye(3) * L) @ (np.eye(3) + eps).T
        pos = _random_packing(rng, nat, cell, dmin)
        out.append(Structure(pos, cell, np.array([True, True, True]),
                             np.full(nat, 14, dtype=np.int32),
                             {"workload": "si_batch", "seed": seed, "index": s}))
    return out


def si_fit_set(nstruct=256, seed=5, noise=0.15, a=5.431):
    """Diamond Si supercells of 64, 96, 144 or 216 atoms with uniform
    +-``noise`` A displacements."""
    rng = np.random.default_rng(seed)
    shapes = [(2, 2, 2), (2, 2, 3), (2, 3, 3), (3, 3, 3)]
    out = []
    for s in range(nstruct):
        size = shapes[int(rng.integers(0, len(shapes)))]
        st = diamond("Si", a, size)
        st.positions += rng.uniform(-noise, noise, size=st.positions.shape)
        st.info.update(workload="si_fit_set", seed=seed, index=s)
        out.append(st)
    return out
