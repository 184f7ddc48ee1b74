"""
ctypes binding of libatomistica_gb300.so (the C-ABI of
include/atomistica_gb300.h).  There is no CPU fallback: if the library is
missing or no CUDA device is present, every compute call raises.
"""

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libatomistica_gb300.so")

GB_PRECISION_FP64 = 0
GB_PRECISION_MIXED = 1
GB_FORCES_SET = 1

_P = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double

# Every symbol the header declares: (name, restype, argtypes).
SIGNATURES = [
    ("gb_get_error", ctypes.c_char_p, []),
    ("gb_version", ctypes.c_char_p, []),
    ("gb_device_count", _I, []),
    ("gb_particles_new", _I, [_P]),
    ("gb_particles_free", None, [_P]),
    ("gb_particles_allocate", _I, [_P, _I]),
    ("gb_particles_get_nat", _I, [_P]),
    ("gb_particles_set_cell", _I, [_P, _P, _P]),
    ("gb_particles_set_positions", _I, [_P, _P]),
    ("gb_particles_set_Z", _I, [_P, _P]),
    ("gb_particles_set_stream", _I, [_P, _P]),
    ("gb_neighbors_new", _I, [_P, _I]),
    ("gb_neighbors_free", None, [_P]),
    ("gb_neighbors_request_interaction_range", _I, [_P, _D]),
    ("gb_neighbors_get_interaction_range", _D, [_P]),
    ("gb_neighbors_update", _I, [_P, _P]),
    ("gb_neighbors_get_size", ctypes.c_int64, [_P]),
    ("gb_neighbors_get", _I, [_P, _P, _P, _P, _P]),
    ("gb_neighbors_set_stream", _I, [_P, _P]),
    ("gb_tersoff_new", _I, [_P, _P]),
    ("gb_kumagai_new", _I, [_P, _P]),
    ("gb_tersoff_scr_new", _I, [_P, _P, _P]),
    ("gb_tabulated_eam_new", _I, [_P, ctypes.c_char_p]),
    ("gb_potential_energy_and_forces_ghost", _I,
     [_P, _I, _I, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    ("gb_potential_energy_and_forces_lammps", _I,
     [_P, _I, _I, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    ("gb_kumagai_scr_new", _I, [_P, _P, _P]),
    ("gb_brenner_new", _I, [_P, _P]),
    ("gb_brenner_scr_new", _I, [_P, _P, _P]),
    ("gb_juslin_new", _I, [_P, _P]),
    ("gb_juslin_scr_new", _I, [_P, _P, _P]),
    ("gb_tabulated_alloy_eam_new", _I, [_P, ctypes.c_char_p]),
    ("gb_potential_free", None, [_P]),
    ("gb_potential_set_precision", _I, [_P, _I]),
    ("gb_potential_set_stream", _I, [_P, _P]),
    ("gb_potential_get_cutoff", _D, [_P]),
    ("gb_potential_bind_to", _I, [_P, _P, _P, _P]),
    ("gb_potential_energy_and_forces", _I, [_P] * 13 + [_P]),
    ("gb_potential_energy_and_forces_flags", _I, [_P] * 13 + [_I, _P]),
    ("gb_tersoff_bind_to", _I, [_P, _P, _P, _P]),
    ("gb_tersoff_energy_and_forces", _I, [_P] * 13 + [_P]),
    ("gb_kumagai_bind_to", _I, [_P, _P, _P, _P]),
    ("gb_kumagai_energy_and_forces", _I, [_P] * 13 + [_P]),
    ("gb_brenner_bind_to", _I, [_P, _P, _P, _P]),
    ("gb_brenner_energy_and_forces", _I, [_P] * 13 + [_P]),
    ("gb_juslin_bind_to", _I, [_P, _P, _P, _P]),
    ("gb_juslin_energy_and_forces", _I, [_P] * 13 + [_P]),
    ("gb_tabulated_alloy_eam_bind_to", _I, [_P, _P, _P, _P]),
    ("gb_tabulated_alloy_eam_energy_and_forces", _I, [_P] * 14),
    ("gb_tabulated_eam_bind_to", _I, [_P, _P, _P, _P]),
    ("gb_tabulated_eam_energy_and_forces", _I, [_P] * 14),
    ("gb_potential_set_elements", _I, [_P, ctypes.c_char_p]),
    ("gb_tabulated_alloy_eam_table", _I, [_P, _I, _I, _P, _P]),
    ("gb_batch_new", _I, [_P]),
    ("gb_batch_free", None, [_P]),
    ("gb_batch_set_stream", _I, [_P, _P]),
    ("gb_batch_set_structures", _I, [_P, _I, _P, _P, _P, _P]),
    ("gb_batch_set_positions", _I, [_P, _P]),
    ("gb_batch_get_nat", _I, [_P]),
    ("gb_batch_set_options", _I, [_P, _I, _I]),
    ("gb_random_packing", _I, [_I, _P, ctypes.c_double, ctypes.c_uint64, ctypes.c_int64, _P]),
    ("gb_batch_last_info", _I, [_P, _P]),
    ("gb_batch_energy_and_forces", _I, [_P, _P, _P, _P, _P]),
    ("gb_batch_md_set_state", _I, [_P, _P, _P]),
    ("gb_batch_md_run", _I, [_P, _P, ctypes.c_double, _I, _P, _P]),
    ("gb_batch_md_get_state", _I, [_P, _P, _P, _P]),
    ("gb_batch_tersoff_tangent", _I, [_P, _I, _I, _P, _P, _P, _P, _P, _P, _P]),
    ("gb_batch_tersoff_adjoint", _I, [_P, _I, _I, _P, _P, _P, _P, _P, _P, _P]),
    ("gb_potential_last_timing", _I, [_P, _P]),
    ("gb_potential_last_stats", _I, [_P, _P]),
    ("gb_potential_set_tile_atoms", _I, [_P, _I]),
    ("gb_potential_set_graph", _I, [_P, _I]),
    ("gb_bop_energy_and_forces_noalloc", _I, [_P, _I, _P, _P, _P, _P, _P, _P, _P, _P, _P,
                                              _P]),
    ("gb_kernel_launches", ctypes.c_uint64, []),
    ("gb_bench_fma_peak", _I, [_I, _P]),
    ("gb_diag_sqrt_check", _I, [ctypes.c_int64, ctypes.c_double, ctypes.c_double, _P]),
]


class TersoffParams(ctypes.Structure):
    """gb_tersoff_params_t"""
    _fields_ = [("nel", _I), ("Z", _I * 3)] + \
        [(k, _D * 6) for k in ("A", "B", "xi", "lambda_", "mu", "omega", "mubo")] + \
        [("m", _I * 6)] + \
        [(k, _D * 3) for k in ("beta", "n", "c", "d", "h")] + \
        [("r1", _D * 6), ("r2", _D * 6)]


class KumagaiParams(ctypes.Structure):
    """gb_kumagai_params_t"""
    _fields_ = [("nel", _I), ("Z", _I * 1)] + \
        [(k, _D * 1) for k in ("A", "B", "lambda1", "lambda2", "eta", "delta", "alpha")] + \
        [("beta", _I * 1)] + \
        [(k, _D * 1) for k in ("c1", "c2", "c3", "c4", "c5", "h", "r1", "r2")]


class BrennerParams(ctypes.Structure):
    """gb_brenner_params_t"""
    _fields_ = [("nel", _I), ("Z", _I * 3)] + \
        [(k, _D * 6) for k in ("D0", "r0", "S", "beta", "gamma", "c", "d", "h", "mu", "n")] + \
        [("m", _I * 6), ("r1", _D * 6), ("r2", _D * 6)]


class JuslinParams(ctypes.Structure):
    """gb_juslin_params_t"""
    _fields_ = [("nel", _I), ("Z", _I * 3)] + \
        [(k, _D * 9) for k in ("D0", "r0", "S", "beta", "gamma", "c", "d", "h", "n")] + \
        [("alpha", _D * 27), ("omega", _D * 27), ("m", _I * 27), ("r1", _D * 9),
         ("r2", _D * 9)]


class ScreeningParams(ctypes.Structure):
    """gb_screening_params_t"""
    _fields_ = [(k, _D * 9) for k in ("or1", "or2", "bor1", "bor2", "Cmin", "Cmax")]


_lib = None


class AtomisticaError(RuntimeError):
    pass


def load():
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise AtomisticaError(
            "libatomistica_gb300.so is not built (expected at %s); run "
            "atomistica_gb300.build.build() — there is no CPU fallback." % LIB_PATH)
    L = ctypes.CDLL(LIB_PATH)
    for name, res, args in SIGNATURES:
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(rc, what=""):
    if rc != 0:
        msg = load().gb_get_error().decode(errors="replace")
        raise AtomisticaError("%s failed (error %d): %s" % (what or "call", rc, msg))
    return rc


def device_count():
    return load().gb_device_count()
