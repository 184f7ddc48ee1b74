"""Tabulated alloy EAM with many elements and an element filter, on the GPU
against the oracle (tabulated_alloy_eam.f90:60 MAX_EAM_ELS = 10, :72 and
:316-335 the `elements` filter), and the uniform 14-argument shim signature
of the EAM classes (factory.template.h:48-50, gen_factory.py:302-351)."""

import ctypes

import numpy as np
import pytest

import oracle
from atomistica_gb300 import io as gio
from atomistica_gb300 import native
from atomistica_gb300 import structures as S
from atomistica_gb300._lib import AtomisticaError

from helpers import compare, gpu_eam

pytestmark = pytest.mark.gpu

ALLOY = ["Cu", "Ag", "Au", "Ni", "Pd", "Pt"]
TEN = ["Cu", "Ag", "Au", "Ni", "Pd", "Pt", "Al", "Pb", "Rh", "Ir"]


def _alloy(zs, seed, size=(4, 4, 4)):
    s = S.fcc("Cu", 3.75, size)
    rng = np.random.default_rng(seed)
    s.numbers = np.array(rng.choice(zs, len(s)), dtype=np.int32)
    s.positions += rng.normal(0, 0.05, s.positions.shape)
    return s


def _gpu(fn, s, elements="*", mask=None):
    p = native.from_atoms(s)
    nl = native.Neighbors(100)
    pot = native.TabulatedAlloyEAM(fn, elements=elements)
    pot.bind_to(p, nl)
    e, f, w, epa, wpa = pot.energy_and_forces(p, nl, mask=mask, epot_per_at=True,
                                              wpot_per_at=True)
    return {"epot": e, "f": f, "wpot": w, "epot_per_at": epa, "wpot_per_at": wpa}


@pytest.mark.parametrize("nel", [6, 10])
def test_many_elements(gpu, tmp_path, nel):
    els = (ALLOY if nel == 6 else TEN)
    fn = gio.analytic_alloy_setfl(str(tmp_path / "a.setfl"), els, seed=nel)
    zs = [S.atomic_numbers[x] for x in els] + [14]  # Si: not in the file
    s = _alloy(zs, 70 + nel)
    ref = oracle.EAM(fn).compute(s, per_at=True)
    compare(ref, _gpu(fn, s), len(s))


@pytest.mark.parametrize("elements,zs", [("Cu,Ag,Ni", [29, 47, 28]), ("Au", [79]),
                                         ("pt,46,Cu", [78, 46, 29]), ("*", None)])
def test_element_filter(gpu, tmp_path, elements, zs):
    fn = gio.analytic_alloy_setfl(str(tmp_path / "a.setfl"), ALLOY, seed=3)
    s = _alloy([29, 47, 79, 28, 46, 78], 71)
    ref = oracle.EAM(fn).compute(s, per_at=True, elements=zs)
    compare(ref, _gpu(fn, s, elements=elements), len(s))


def test_element_filter_with_mask(gpu, tmp_path):
    fn = gio.analytic_alloy_setfl(str(tmp_path / "a.setfl"), ALLOY, seed=4)
    s = _alloy([29, 47, 79, 28, 46, 78], 72)
    mask = (np.arange(len(s)) % 3 != 1).astype(np.int32)
    ref = oracle.EAM(fn).compute(s, per_at=True, mask=mask, elements=[47, 79, 46])
    compare(ref, _gpu(fn, s, elements="Ag,Au,Pd", mask=mask), len(s))


def test_filter_change_between_calls(gpu, tmp_path):
    fn = gio.analytic_alloy_setfl(str(tmp_path / "a.setfl"), ALLOY, seed=5)
    s = _alloy([29, 47, 79, 28, 46, 78], 73, size=(3, 3, 3))
    p = native.from_atoms(s)
    nl = native.Neighbors(100)
    pot = native.TabulatedAlloyEAM(fn)
    pot.bind_to(p, nl)
    o = oracle.EAM(fn)
    for elements, zs in (("*", None), ("Cu,Pt", [29, 78]), ("*", None)):
        pot.set_elements(elements)
        e, f, w = pot.energy_and_forces(p, nl)
        compare(o.compute(s, elements=zs), {"epot": e, "f": f, "wpot": w}, len(s),
                per_at=False)


def test_unknown_element_in_filter(gpu, tmp_path):
    fn = gio.analytic_alloy_setfl(str(tmp_path / "a.setfl"), ALLOY, seed=6)
    with pytest.raises(AtomisticaError, match=r"error -11\): Unknown element 'Xq'"):
        native.TabulatedAlloyEAM(fn, elements="Cu,Xq")


def test_setfl_name_mismatch(gpu, tmp_path):
    fn = str(tmp_path / "bad.setfl")
    gio.analytic_alloy_setfl(fn, ["Cu", "Ag"], seed=7)
    lines = open(fn).read().split("\n")
    lines[3] = "2 Cu Au"  # the second element's atomic number (47) is Ag
    open(fn, "w").write("\n".join(lines))
    with pytest.raises(AtomisticaError, match="Atomic number 47 is element Ag and does not "
                                              "match element name Au"):
        native.TabulatedAlloyEAM(fn)


def test_more_than_ten_elements_refused(gpu, tmp_path):
    fn = gio.analytic_alloy_setfl(str(tmp_path / "a.setfl"), TEN + ["Fe"], seed=8)
    with pytest.raises(AtomisticaError, match="1 to 10 elements"):
        native.TabulatedAlloyEAM(fn)


def test_uniform_shim_signature(gpu, tmp_path):
    # gb_tabulated_alloy_eam_energy_and_forces has the 14 arguments of every
    # python_<mod>_energy_and_forces; per-bond outputs are refused with the
    # generated shim's message, the rest equals the generic call.
    from atomistica_gb300 import _lib
    L = _lib.load()
    fn = gio.analytic_alloy_setfl(str(tmp_path / "a.setfl"), ALLOY, seed=9)
    s = _alloy([29, 47, 79], 74, size=(2, 2, 2))
    p = native.from_atoms(s)
    nl = native.Neighbors(100)
    pot = native.TabulatedAlloyEAM(fn)
    pot.bind_to(p, nl)
    nat = len(s)
    epot = ctypes.c_double(0.0)
    f = np.zeros((nat, 3))
    w = np.zeros((3, 3))
    epa = np.zeros(nat)
    wpa = np.zeros((nat, 3, 3))
    err = ctypes.c_int(0)
    rc = L.gb_tabulated_alloy_eam_energy_and_forces(
        pot._h, p._h, nl._h, None, ctypes.byref(epot), f.ctypes.data, w.ctypes.data, None,
        epa.ctypes.data, None, None, wpa.ctypes.data, None, ctypes.byref(err))
    assert rc == 0, L.gb_get_error()
    ref = oracle.EAM(fn).compute(s, per_at=True)
    assert abs(epot.value - ref["epot"]) / nat < 1e-10
    assert np.max(np.abs(f - ref["f"])) < 1e-9
    bogus = np.zeros(1000)
    for k in range(3):
        args = [None, None, None]
        args[k] = bogus.ctypes.data
        rc = L.gb_tabulated_alloy_eam_energy_and_forces(
            pot._h, p._h, nl._h, None, ctypes.byref(epot), f.ctypes.data, w.ctypes.data, None,
            None, args[0], args[1], None, args[2], ctypes.byref(err))
        assert rc == -11
        name = ("epot_per_bond", "f_per_bond", "wpot_per_bond")[k]
        assert ("*%s* argument present but not supported by potential TabulatedAlloyEAM."
                % name).encode() in L.gb_get_error()


def test_funcfl_filter(gpu, tmp_path):
    # TabulatedEAM has the same filter: excluding its element leaves nothing
    fn = gio.cu_analytic_funcfl(str(tmp_path / "cu.funcfl"))
    c = S.fcc("Cu", 3.615, (3, 3, 3))
    c.positions += np.random.default_rng(75).normal(0, 0.05, c.positions.shape)
    p = native.from_atoms(c)
    nl = native.Neighbors(100)
    ref = oracle.FuncflEAM(fn).compute(c)
    for elements, zero in (("Cu", False), ("Ag", True)):
        pot = native.TabulatedEAM(fn, elements=elements)
        pot.bind_to(p, nl)
        e, f, w = pot.energy_and_forces(p, nl)
        if zero:
            assert e == 0.0 and np.all(f == 0.0)
        else:
            assert abs(e - ref["epot"]) / len(c) < 1e-10
            assert np.max(np.abs(f - ref["f"])) < 1e-9
