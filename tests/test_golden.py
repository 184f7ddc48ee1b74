"""Committed golden fixtures (tests/golden/*.npz, made by
tests/golden/make_golden.py): the oracle must reproduce them on CPU, and the
GPU path must match them within the parity tolerances."""

import glob
import os
import tempfile

import numpy as np
import pytest

import oracle
from atomistica_gb300 import io as gio
from atomistica_gb300.structures import Structure

from helpers import E_TOL, F_TOL, KUMAGAI, TERSOFF, W_TOL

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))
EAM_TABLE = dict(nr=800, nrho=800)


def load(fn):
    d = dict(np.load(fn))
    s = Structure(d["positions"], d["cell"], d["pbc"], d["numbers"])
    return str(d["kind"]), s, d


def test_fixtures_present():
    assert len(GOLDEN) >= 6


@pytest.mark.parametrize("fn", GOLDEN, ids=[os.path.basename(f) for f in GOLDEN])
def test_oracle_reproduces_golden(fn):
    kind, s, d = load(fn)
    with tempfile.TemporaryDirectory() as tmp:
        if kind == "eam":
            setfl = gio.cu_analytic_setfl(os.path.join(tmp, "cu.setfl"), **EAM_TABLE)
            o = oracle.EAM(setfl).compute(s, per_at=True, nthreads=1)
        else:
            o = oracle.bop(kind, TERSOFF if kind == "tersoff" else KUMAGAI, s, per_at=True,
                           nthreads=1)
    assert np.array_equal(o["nl"].seed, d["nl_seed"])
    assert np.array_equal(o["nl"].nbr, d["nl_j"]) and np.array_equal(o["nl"].dc, d["nl_dc"])
    assert abs(o["epot"] - d["epot"]) < 1e-12 * abs(d["epot"])
    assert np.max(np.abs(o["f"] - d["f"])) < 1e-12
    assert np.max(np.abs(o["wpot"] - d["wpot"])) < 1e-11
    assert np.max(np.abs(o["epot_per_at"] - d["epot_per_at"])) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("fn", GOLDEN, ids=[os.path.basename(f) for f in GOLDEN])
def test_gpu_matches_golden(gpu, fn):
    from helpers import gpu_bop, gpu_eam
    kind, s, d = load(fn)
    with tempfile.TemporaryDirectory() as tmp:
        if kind == "eam":
            setfl = gio.cu_analytic_setfl(os.path.join(tmp, "cu.setfl"), **EAM_TABLE)
            g = gpu_eam(setfl, s)
        else:
            g = gpu_bop(kind, s)
    seed, j, dc = g["nl"]
    assert np.array_equal(seed, d["nl_seed"]) and np.array_equal(j, d["nl_j"])
    assert np.array_equal(dc, d["nl_dc"])
    nat = len(s)
    assert abs(g["epot"] - d["epot"]) / nat < E_TOL
    assert np.max(np.abs(g["f"] - d["f"])) < F_TOL
    assert np.max(np.abs(g["wpot"] - d["wpot"])) < W_TOL * nat
    assert np.max(np.abs(g["epot_per_at"] - d["epot_per_at"])) < 10 * E_TOL
    assert np.max(np.abs(g["wpot_per_at"] - d["wpot_per_at"])) < 10 * W_TOL
