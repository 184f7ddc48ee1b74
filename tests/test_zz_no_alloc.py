"""The allocation-free entry point gb_bop_energy_and_forces_noalloc.

It serves callers that cannot call cudaMalloc (a host framework that has
reserved the device memory for its own pool, or an MD loop that must not
allocate inside a time step): all its intermediate buffers live in one static
device array.  This test calls it through the C-ABI with device buffers and
checks, on two calls in a row, that it gives the same energy, forces and
virial as the regular entry point gb_potential_energy_and_forces, within the
parity tolerances used throughout the tests; and that inputs beyond its size
limit are refused with a clear error.  It is collected last on purpose."""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

E_TOL, F_TOL, W_TOL = 1e-10, 1e-9, 1e-9  # per atom, as in tests/helpers.py


def _noalloc_call(L, pot, nat, r, cell, Z, seed, j, dc, epot, f, wpot, stream):
    return L.gb_bop_energy_and_forces_noalloc(
        pot._h, nat, r.data_ptr(), cell.ctypes.data, Z.data_ptr(), seed.data_ptr(),
        j.data_ptr(), dc.data_ptr(), epot.data_ptr(), f.data_ptr(), wpot.data_ptr(), stream)


@pytest.mark.parametrize("kind,precision", [("tersoff", "fp64"), ("tersoff", "mixed"),
                                            ("kumagai", "fp64")])
def test_noalloc_matches_regular_entry_point(gpu, kind, precision):
    import torch
    from atomistica_gb300 import _lib, native, structures
    L = _lib.load()
    s = structures.tersoff_si_4096(seed=21)
    nat = len(s)
    p = native.from_atoms(s)
    nl = native.Neighbors(100)
    cls = native.Tersoff if kind == "tersoff" else native.Kumagai
    pot = cls(precision=precision)
    pot.bind_to(p, nl)
    e_ref, f_ref, w_ref = pot.energy_and_forces(p, nl)
    seed, j, dc = nl.get_list(p)

    dev = torch.device("cuda", torch.cuda.current_device())
    r = torch.tensor(s.positions, dtype=torch.float64, device=dev)
    Z = torch.tensor(s.numbers, dtype=torch.int32, device=dev)
    seed_d = torch.tensor(seed, dtype=torch.int64, device=dev)
    j_d = torch.tensor(j, dtype=torch.int32, device=dev)
    dc_d = torch.tensor(dc, dtype=torch.int32, device=dev).contiguous()
    cell = np.ascontiguousarray(s.cell, dtype=np.float64)
    f = torch.zeros((nat, 3), dtype=torch.float64, device=dev)
    epot = torch.zeros(1, dtype=torch.float64, device=dev)
    wpot = torch.zeros(9, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        f.zero_()
        wpot.zero_()
        epot.fill_(float("nan"))
        torch.cuda.synchronize()
        rc = _noalloc_call(L, pot, nat, r, cell, Z, seed_d, j_d, dc_d, epot, f, wpot, stream)
        assert rc == 0, L.gb_get_error()
        torch.cuda.synchronize()
        e = float(epot.item())
        fh = f.cpu().numpy()
        wh = wpot.cpu().numpy().reshape(3, 3, order="F")
        assert abs(e - e_ref) / nat < E_TOL, (call, e, e_ref)
        assert np.max(np.abs(fh - f_ref)) < F_TOL, call
        assert np.max(np.abs(wh - w_ref)) < W_TOL * nat, call


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
