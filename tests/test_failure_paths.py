"""Failure paths of the single-structure API on the GPU, and the list-build
fallbacks.  The reference reports a neighbour-list overflow as an error
(python_neighbors.f90:713-718) and refuses bond arrays that are too small
(bop_kernel.f90:47-53, 672-678); here every such condition is detected on
the device, read back by the host and returned as an error code with a
message, after which the objects stay usable.  Nothing here faults the GPU:
the bad inputs are values (non-finite or far-away positions) that the
kernels flag and skip."""

import re

import numpy as np
import pytest

import oracle
from atomistica_gb300 import native
from atomistica_gb300 import structures as S
from atomistica_gb300._lib import AtomisticaError

from helpers import TERSOFF, compare, rattled_diamond

pytestmark = pytest.mark.gpu

GB_ERROR_DOMAIN = -13


def _setup(s, precision="fp64"):
    p = native.from_atoms(s)
    nl = native.Neighbors(100)
    pot = native.Tersoff(precision=precision)
    pot.bind_to(p, nl)
    return p, nl, pot


def _eval(p, nl, pot):
    e, f, w = pot.energy_and_forces(p, nl)
    return {"epot": e, "f": f, "wpot": w}


def _expect_domain_error(p, nl, pot, pattern):
    with pytest.raises(AtomisticaError) as ei:
        pot.energy_and_forces(p, nl)
    msg = str(ei.value)
    assert "error %d" % GB_ERROR_DOMAIN in msg, msg
    assert re.search(pattern, msg), msg


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_nonfinite_position_is_a_domain_error(gpu, precision):
    s = rattled_diamond(size=(2, 2, 2), amp=0.2, seed=51)
    p, nl, pot = _setup(s, precision)
    _eval(p, nl, pot)
    for bad in (np.nan, np.inf, -np.inf):
        r = s.positions.copy()
        r[3, 1] = bad
        p.set_positions(r)
        _expect_domain_error(p, nl, pot, "Non-finite particle position")
    # the objects recover with valid positions
    p.set_positions(s.positions)
    tol = 1e-9 if precision == "fp64" else 1e-5
    compare(oracle.bop("tersoff", TERSOFF, s), _eval(p, nl, pot), len(s), ftol=tol, wtol=tol,
            etol=1e-10 if precision == "fp64" else 1e-6, per_at=False)


def test_image_shift_beyond_range_is_a_domain_error(gpu):
    s = rattled_diamond(size=(2, 2, 2), amp=0.2, seed=52)
    p, nl, pot = _setup(s)
    _eval(p, nl, pot)
    r = s.positions.copy()
    r[5] += 600 * s.cell[0]  # 600 cell lengths away: more than the 511 images supported
    p.set_positions(r)
    _expect_domain_error(p, nl, pot, "image shift outside the supported range")
    # 500 cell lengths away is within range and equals the wrapped structure
    t = s.copy()
    t.positions[5] += 500 * s.cell[0]
    p.set_positions(t.positions)
    compare(oracle.bop("tersoff", TERSOFF, t), _eval(p, nl, pot), len(s), per_at=False)


def test_eam_nonfinite_position(gpu, tmp_path):
    from atomistica_gb300 import io as gio
    fn = gio.cu_analytic_setfl(str(tmp_path / "cu.setfl"), nr=500, nrho=500)
    c = S.fcc("Cu", 3.615, (2, 2, 2))
    p = native.from_atoms(c)
    nl = native.Neighbors(100)
    pot = native.TabulatedAlloyEAM(fn)
    pot.bind_to(p, nl)
    pot.energy_and_forces(p, nl)
    r = c.positions.copy()
    r[0, 0] = np.nan
    p.set_positions(r)
    _expect_domain_error(p, nl, pot, "Non-finite particle position")


def test_staging_capacity_fallback(gpu):
    # The steady-state list build keeps each atom's first `cap` entries in a
    # staging buffer sized from the previous build (its maximum coordination
    # + 25 % + 4).  Compressing the structure between calls makes atoms
    # exceed that capacity: the build must notice and take the count + fill
    # passes, and still give the reference's list and forces.
    s = S.diamond("Si", 5.431, (3, 3, 3))
    s.positions += np.random.default_rng(53).uniform(-0.05, 0.05, s.positions.shape)
    p, nl, pot = _setup(s)
    for _ in range(2):  # first build (count + fill), then the staged single pass
        compare(oracle.bop("tersoff", TERSOFF, s), _eval(p, nl, pot), len(s), per_at=False)
    seed, _, _ = nl.get_list(p)
    assert np.diff(seed).max() == 4  # capacity of the next build: 12
    t = s.copy()
    t.positions = s.positions * 0.75
    t.cell = s.cell * 0.75  # second shell at 2.88 A < 3.0 A: 16 neighbours
    p.set_cell(t.cell, t.pbc)
    for _ in range(2):  # over capacity (count + fill), then staged again
        p.set_positions(t.positions)
        ref = oracle.bop("tersoff", TERSOFF, t)
        got = _eval(p, nl, pot)
        compare(ref, got, len(t), per_at=False)
        seed, j, dc = nl.get_list(p)
        ro = oracle.neighbors(t, 3.0)
        assert np.diff(seed).max() == 16
        assert np.array_equal(seed, ro.seed) and np.array_equal(j, ro.nbr)
        assert np.array_equal(dc, ro.dc)
