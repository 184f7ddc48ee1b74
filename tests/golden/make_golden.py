"""
Generates the golden fixtures tests/golden/*.npz: seeded input structures and
the FP64 oracle's outputs for them (energy, forces, virial, per-atom energy
and virial, and the neighbour list).  Run from the repository root:

    python tests/golden/make_golden.py

The fixtures pin the oracle (tests/test_golden.py re-runs it against them on
CPU) and give the GPU tests a stored reference that does not depend on the
oracle build on the GPU host.
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")]

import oracle  # noqa: E402
from atomistica_gb300 import io as gio  # noqa: E402
from atomistica_gb300 import structures as S  # noqa: E402
from helpers import KUMAGAI, TERSOFF, random_carbon, rattled_diamond, triclinic_si  # noqa: E402


def cases():
    yield "tersoff_si64", "tersoff", rattled_diamond("Si", 5.431, (2, 2, 2), 0.3, 101)
    yield "tersoff_sic64", "tersoff", (lambda s: (s.positions.__iadd__(
        np.random.default_rng(102).uniform(-0.3, 0.3, s.positions.shape)), s)[1])(
        S.b3(("Si", "C"), 4.3596, (2, 2, 2)))
    yield "tersoff_carbon80", "tersoff", random_carbon(80, seed=103)
    yield "tersoff_triclinic30", "tersoff", triclinic_si(30, seed=104)
    yield "kumagai_si64", "kumagai", rattled_diamond("Si", 5.429, (2, 2, 2), 0.3, 105)
    yield "eam_cu108", "eam", (lambda s: (s.positions.__iadd__(
        np.random.default_rng(106).normal(0, 0.05, s.positions.shape)), s)[1])(
        S.fcc("Cu", 3.615, (3, 3, 3)))


EAM_TABLE = dict(nr=800, nrho=800)


def eam_file(tmpdir):
    fn = os.path.join(tmpdir, "cu_golden.setfl")
    gio.cu_analytic_setfl(fn, **EAM_TABLE)
    return fn


def compute(kind, s, tmpdir):
    if kind == "eam":
        e = oracle.EAM(eam_file(tmpdir))
        return e.compute(s, per_at=True, nthreads=1)
    params = TERSOFF if kind == "tersoff" else KUMAGAI
    return oracle.bop(kind, params, s, per_at=True, nthreads=1)


def main():
    import tempfile
    with tempfile.TemporaryDirectory() as tmp:
        for name, kind, s in cases():
            o = compute(kind, s, tmp)
            np.savez_compressed(
                os.path.join(HERE, name + ".npz"), kind=kind, positions=s.positions,
                cell=s.cell, pbc=s.pbc, numbers=s.numbers, epot=o["epot"], f=o["f"],
                wpot=o["wpot"], epot_per_at=o["epot_per_at"], wpot_per_at=o["wpot_per_at"],
                nl_seed=o["nl"].seed, nl_j=o["nl"].nbr, nl_dc=o["nl"].dc)
            print(name, len(s), o["epot"])


if __name__ == "__main__":
    main()
