"""The allocation-free entry point gb_bop_energy_and_forces_noalloc.

It serves callers that cannot call cudaMalloc (a host framework that has
reserved the device memory for its own pool, or an MD loop that must not
allocate inside a time step): all its intermediate buffers live in one static
device array.  This test calls it through the C-ABI with device buffers and
checks, on two calls in a row, that it gives the same energy, forces and
virial as the regular entry point gb_potential_energy_and_forces, within the
parity tolerances used throughout the tests; and that inputs beyond its size
limit, and malformed neighbour lists, are refused with a clear error before
any kernel walks the list.  It is collected last on purpose."""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

E_TOL, F_TOL, W_TOL = 1e-10, 1e-9, 1e-9  # per atom, as in tests/helpers.py


def _noalloc_call(L, pot, nat, r, cell, Z, seed, j, dc, epot, f, wpot, stream):
    return L.gb_bop_energy_and_forces_noalloc(
        pot._h, nat, r.data_ptr(), cell.ctypes.data, Z.data_ptr(), seed.data_ptr(),
        j.data_ptr(), dc.data_ptr(), epot.data_ptr(), f.data_ptr(), wpot.data_ptr(), stream)


def _setup(kind, precision, s):
    import torch
    from atomistica_gb300 import native
    nat = len(s)
    p = native.from_atoms(s)
    nl = native.Neighbors(100)
    cls = {"tersoff": native.Tersoff, "kumagai": native.Kumagai,
           "brenner": native.Brenner}[kind]
    pot = cls(precision=precision)
    pot.bind_to(p, nl)
    e_ref, f_ref, w_ref = pot.energy_and_forces(p, nl)
    seed, j, dc = nl.get_list(p)
    dev = torch.device("cuda", torch.cuda.current_device())
    d = dict(
        pot=pot, nat=nat, dev=dev, ref=(e_ref, f_ref, w_ref), host=(seed, j, dc),
        r=torch.tensor(s.positions, dtype=torch.float64, device=dev),
        Z=torch.tensor(s.numbers, dtype=torch.int32, device=dev),
        cell=np.ascontiguousarray(s.cell, dtype=np.float64),
        f=torch.zeros((nat, 3), dtype=torch.float64, device=dev),
        epot=torch.zeros(1, dtype=torch.float64, device=dev),
        wpot=torch.zeros(9, dtype=torch.float64, device=dev))
    return d


def _run(L, d, seed, j, dc):
    import torch
    dev = d["dev"]
    seed_d = torch.tensor(seed, dtype=torch.int64, device=dev)
    j_d = torch.tensor(j, dtype=torch.int32, device=dev)
    dc_d = torch.tensor(dc, dtype=torch.int32, device=dev).contiguous()
    d["f"].zero_()
    d["wpot"].zero_()
    d["epot"].fill_(float("nan"))
    torch.cuda.synchronize()
    rc = _noalloc_call(L, d["pot"], d["nat"], d["r"], d["cell"], d["Z"], seed_d, j_d, dc_d,
                       d["epot"], d["f"], d["wpot"], torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return rc


@pytest.mark.parametrize("kind,precision", [("tersoff", "fp64"), ("tersoff", "mixed"),
                                            ("kumagai", "fp64"), ("brenner", "fp64"),
                                            ("brenner", "mixed")])
def test_noalloc_matches_regular_entry_point(gpu, kind, precision):
    from atomistica_gb300 import _lib, structures
    L = _lib.load()
    if kind == "brenner":
        s = structures.b3(("Si", "C"), 4.3596, (6, 6, 6))
        s.positions += np.random.default_rng(22).uniform(-0.1, 0.1, s.positions.shape)
    else:
        s = structures.tersoff_si_4096(seed=21)
    d = _setup(kind, precision, s)
    nat = d["nat"]
    e_ref, f_ref, w_ref = d["ref"]
    for call in range(2):
        rc = _run(L, d, *d["host"])
        assert rc == 0, L.gb_get_error()
        e = float(d["epot"].item())
        fh = d["f"].cpu().numpy()
        wh = d["wpot"].cpu().numpy().reshape(3, 3, order="F")
        assert abs(e - e_ref) / nat < E_TOL, (call, e, e_ref)
        assert np.max(np.abs(fh - f_ref)) < F_TOL, call
        assert np.max(np.abs(wh - w_ref)) < W_TOL * nat, call


def _bad_lists(seed, j, dc, nat):
    """(name, seed, j, dc, expected message fragment) of malformed lists.
    Every array is long enough for the offsets it claims, so the only fault
    is the one named."""
    n = int(seed[-1])
    out = []
    s2 = seed + 1
    out.append(("seed0", s2, np.concatenate([j, [0]]), np.concatenate([dc, [[0, 0, 0]]]),
                b"seed[0] != 0"))
    s2 = seed.copy()
    s2[5] = seed[7]
    out.append(("decreasing", s2, j, dc, b"decreasing offsets"))
    s2 = seed.copy()
    s2[3] = n + 10
    out.append(("beyond_end", s2, j, dc, b"offsets not within"))
    s2 = seed.copy()
    s2[4] = -3
    out.append(("negative", s2, j, dc, b"offsets not within"))
    j2 = j.copy()
    j2[0] = nat
    out.append(("j_range", seed, j2, dc, b"neighbour index out of range"))
    dc2 = dc.copy()
    dc2[0, 0] = 600
    out.append(("shift", seed, j, dc2, b"image shift beyond"))
    dc2 = dc.copy()
    dc2[0, 0] += 1
    out.append(("asymmetric", seed, j, dc2, b"list not symmetric"))
    return out


def test_noalloc_rejects_malformed_lists(gpu):
    from atomistica_gb300 import _lib, structures
    L = _lib.load()
    s = structures.diamond("Si", 5.431, (2, 2, 2))
    s.positions += np.random.default_rng(3).uniform(-0.1, 0.1, s.positions.shape)
    d = _setup("tersoff", "fp64", s)
    seed, j, dc = d["host"]
    for name, s2, j2, dc2, msg in _bad_lists(seed, j, dc, d["nat"]):
        rc = _run(L, d, s2, j2, dc2)
        assert rc == -11, (name, rc)  # GB_ERROR_ARGUMENT
        assert msg in L.gb_get_error(), (name, L.gb_get_error())
    # a good call after the rejected ones still matches
    assert _run(L, d, seed, j, dc) == 0, L.gb_get_error()
    assert np.max(np.abs(d["f"].cpu().numpy() - d["ref"][1])) < F_TOL


def test_noalloc_rejects_too_many_entries(gpu):
    from atomistica_gb300 import _lib, structures
    L = _lib.load()
    s = structures.diamond("Si", 5.431, (2, 2, 2))
    d = _setup("tersoff", "fp64", s)
    seed, j, dc = d["host"]
    s2 = seed.copy()
    s2[-1] = 262145  # only the total is read before the limit check
    rc = _run(L, d, s2, j, dc)
    assert rc == -12  # GB_ERROR_CAPACITY
    assert b"more than the maximum of 262144" in L.gb_get_error()


def test_noalloc_rejects_oversize(gpu):
    import torch
    from atomistica_gb300 import _lib, native
    L = _lib.load()
    pot = native.Tersoff()
    nat = 16385
    dev = torch.device("cuda", torch.cuda.current_device())
    r = torch.zeros((nat, 3), dtype=torch.float64, device=dev)
    Z = torch.full((nat,), 14, dtype=torch.int32, device=dev)
    seed = torch.zeros(nat + 1, dtype=torch.int64, device=dev)
    j = torch.zeros(1, dtype=torch.int32, device=dev)
    dc = torch.zeros((1, 3), dtype=torch.int32, device=dev)
    f = torch.zeros((nat, 3), dtype=torch.float64, device=dev)
    epot = torch.zeros(1, dtype=torch.float64, device=dev)
    wpot = torch.zeros(9, dtype=torch.float64, device=dev)
    cell = np.eye(3) * 100.0
    rc = _noalloc_call(L, pot, nat, r, cell, Z, seed, j, dc, epot, f, wpot,
                       torch.cuda.current_stream().cuda_stream)
    assert rc == -12  # GB_ERROR_CAPACITY
    assert b"exceeds the maximum" in L.gb_get_error()
