"""The C-ABI library loads and exports every function include/*.h declares; the
ctypes mirrors of the parameter structs match the C layout (CPU only: no
compute calls)."""

import glob
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[a-zA-Z_][\w\s\*]*?\b(gb_\w+)\s*\(", src, re.M):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    from atomistica_gb300 import build
    build.build()
    from atomistica_gb300 import _lib
    return _lib.load()


def test_header_declares_entry_points():
    names = declared_functions()
    assert "gb_potential_energy_and_forces" in names
    assert "gb_neighbors_update" in names
    assert len(names) >= 30


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", lib._name], capture_output=True,
                         text=True).stdout
    exported = set(re.findall(r"\b(gb_\w+)\b", out))
    assert set(declared_functions()) <= exported


def test_ctypes_signatures_cover_header():
    from atomistica_gb300 import _lib
    assert set(n for n, _, _ in _lib.SIGNATURES) == set(declared_functions())


def test_struct_layout_matches_c(tmp_path):
    from atomistica_gb300 import _lib
    import ctypes
    prog = tmp_path / "layout.c"
    prog.write_text("""
#include <stdio.h>
#include <stddef.h>
#include "atomistica_gb300.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu %zu\\n", sizeof(gb_tersoff_params_t),
         offsetof(gb_tersoff_params_t, m), offsetof(gb_tersoff_params_t, r2),
         sizeof(gb_kumagai_params_t), offsetof(gb_kumagai_params_t, beta),
         sizeof(gb_brenner_params_t), offsetof(gb_brenner_params_t, m),
         offsetof(gb_brenner_params_t, r2));
  return 0;
}
""")
    exe = tmp_path / "layout"
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(prog), "-o", str(exe)])
    vals = [int(x) for x in subprocess.check_output([str(exe)]).split()]
    T, K, B = _lib.TersoffParams, _lib.KumagaiParams, _lib.BrennerParams
    assert vals == [ctypes.sizeof(T), T.m.offset, T.r2.offset, ctypes.sizeof(K), K.beta.offset,
                    ctypes.sizeof(B), B.m.offset, B.r2.offset]


def test_library_reports_missing_gpu_cleanly(lib):
    # Without a GPU the compute entry points return an error code, never crash.
    if lib.gb_device_count() > 0:
        pytest.skip("a GPU is present")
    import ctypes
    h = ctypes.c_void_p()
    assert lib.gb_particles_new(ctypes.byref(h)) == 0
    assert lib.gb_particles_allocate(h, 8) == -10  # GB_ERROR_CUDA
    assert b"CUDA" in lib.gb_get_error() or b"cuda" in lib.gb_get_error()
    lib.gb_particles_free(h)
