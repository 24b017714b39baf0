"""ctypes binding of ``lib/libbib_gb300.so`` (the C ABI in ``include/bib/bib.h``).

There is no CPU fallback: if the CUDA library is missing or cannot be loaded every
entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libbib_gb300.so")

P_COUNT = 12


class LatticeParams(C.Structure):
    _fields_ = [
        ("periodic", C.c_int32 * 3),
        ("collision", C.c_int32),
        ("storage", C.c_int32),
        ("wall_y", C.c_int32),
        ("wall_z", C.c_int32),
        ("use_phase", C.c_int32),
        ("reserved", C.c_int32),
        ("omega", C.c_double),
        ("omega_inner", C.c_double),
        ("trt_magic", C.c_double),
        ("wall_u", (C.c_double * 3) * 4),
        ("body_force", C.c_double * 3),
        ("f16_scale", C.c_double),
    ]


class IbParams(C.Structure):
    _fields_ = [("dirac", C.c_int32), ("spread_mode", C.c_int32), ("field_offset", C.c_double)]


class Tuning(C.Structure):
    _fields_ = [("collide_kernel", C.c_int32), ("tile_cells", C.c_int32), ("stages", C.c_int32),
                ("membrane_block", C.c_int32), ("force_reset", C.c_int32), ("wait_limit_us", C.c_int32),
                ("withhold_tile", C.c_int32), ("reserved", C.c_int32 * 1)]


class BatchTuning(C.Structure):
    _fields_ = [("tile_cells", C.c_int32), ("stages", C.c_int32), ("membrane_block", C.c_int32),
                ("reserved", C.c_int32 * 5)]


class Potential(C.Structure):
    _fields_ = [("kind", C.c_int32), ("search", C.c_int32), ("r0", C.c_double), ("beta", C.c_double),
                ("strength", C.c_double)]


class Growth(C.Structure):
    _fields_ = [("box", C.c_int64 * 6), ("periodic", C.c_int32 * 3), ("has_wall", C.c_int32),
                ("wall", C.c_double * 3), ("min_dist", C.c_double), ("strength", C.c_double),
                ("initial_scale", C.c_double), ("density", C.c_double), ("damping", C.c_double),
                ("n_it", C.c_int64), ("rescale_every", C.c_int64), ("it_end", C.c_int64)]


class Config(C.Structure):
    _fields_ = [("device", C.c_int32), ("flags", C.c_int32)]


# name -> (restype, argtypes)
_dp, _ip, _i32p, _vp = C.POINTER(C.c_double), C.POINTER(C.c_int64), C.POINTER(C.c_int32), C.c_void_p
SIGNATURES = {
    "bib_abi_version": (C.c_int32, []),
    "bib_status_string": (C.c_char_p, [C.c_int32]),
    "bib_create": (C.c_int32, [C.POINTER(Config), C.POINTER(C.c_void_p)]),
    "bib_destroy": (None, [_vp]),
    "bib_sync": (C.c_int32, [_vp]),
    "bib_last_error": (C.c_size_t, [_vp, C.c_char_p, C.c_size_t]),
    "bib_set_graph_mode": (C.c_int32, [_vp, C.c_int32]),
    "bib_set_profiling": (C.c_int32, [_vp, C.c_int32]),
    "bib_profile_read": (C.c_int32, [_vp, _dp, C.c_int32]),
    "bib_lattice_add_domain": (C.c_int32, [_vp, C.c_int64, C.c_int64, C.c_int64, C.POINTER(LatticeParams), _i32p]),
    "bib_coprocessor_domain_params": (C.c_int32, [C.c_double, C.c_int32, C.c_int32, C.POINTER(LatticeParams)]),
    "bib_lattice_cells": (C.c_int32, [_vp, C.c_int32, _ip]),
    "bib_lattice_send": (C.c_int32, [_vp, C.c_int32, _vp, C.c_size_t, C.c_int32]),
    "bib_lattice_receive": (C.c_int32, [_vp, C.c_int32, _vp, C.c_size_t, C.c_int32]),
    "bib_lattice_collide_and_stream": (C.c_int32, [_vp, C.c_int32, C.c_int64]),
    "bib_lattice_init_equilibrium": (C.c_int32, [_vp, C.c_int32, _dp, _dp]),
    "bib_lattice_set_force": (C.c_int32, [_vp, C.c_int32, _dp]),
    "bib_lattice_get_force": (C.c_int32, [_vp, C.c_int32, _dp]),
    "bib_lattice_set_phase": (C.c_int32, [_vp, C.c_int32, _dp]),
    "bib_lattice_get_phase": (C.c_int32, [_vp, C.c_int32, _dp]),
    "bib_lattice_get_velocity": (C.c_int32, [_vp, C.c_int32, _dp]),
    "bib_shape_store": (C.c_int32, [_vp, _dp, _ip, C.c_int64, C.c_int64, _i32p]),
    "bib_shape_info": (C.c_int32, [_vp, C.c_int32, _dp]),
    "bib_shape_set_tag": (C.c_int32, [_vp, C.c_int32, C.c_char_p]),
    "bib_ib_configure": (C.c_int32, [_vp, C.c_int32, C.POINTER(IbParams)]),
    "bib_particle_add": (C.c_int32, [_vp, C.c_int32, C.c_int32, C.c_int32, _dp, _dp, _i32p]),
    "bib_particle_count": (C.c_int32, [_vp, C.c_int32, _i32p]),
    "bib_particle_get": (C.c_int32, [_vp, C.c_int32, C.c_int32, _dp, _dp, _dp]),
    "bib_particle_set_positions": (C.c_int32, [_vp, C.c_int32, C.c_int32, _dp]),
    "bib_particle_stats": (C.c_int32, [_vp, C.c_int32, C.c_int32, _dp]),
    "bib_particles_download": (C.c_int32, [_vp, C.c_int32, _dp, _dp]),
    "bib_particles_download_async": (C.c_int32, [_vp, C.c_int32, _dp, _dp, C.c_int32]),
    "bib_download_wait": (C.c_int32, [_vp, C.c_int32]),
    "bib_particles_upload": (C.c_int32, [_vp, C.c_int32, _dp]),
    "bib_total_vertices": (C.c_int32, [_vp, C.c_int32, _ip]),
    "bib_total_volume": (C.c_int32, [_vp, C.c_int32, _dp]),
    "bib_ibm_step": (C.c_int32, [_vp, C.c_int32]),
    "bib_ibm_init": (C.c_int32, [_vp, C.c_int32]),
    "bib_ib_set_pipe_boundary": (C.c_int32, [_vp, C.c_int32, C.c_double, C.c_double, C.c_double]),
    "bib_lattice_set_pipe_walls": (C.c_int32, [_vp, C.c_int32, C.c_double, C.c_double, C.c_double, C.c_int32]),
    "bib_add_wall_interaction": (C.c_int32, [_vp, C.c_int32, C.c_int32, C.c_double, C.c_double, C.POINTER(Potential)]),
    "bib_add_pipe_wall_interaction": (C.c_int32, [_vp, C.c_int32, C.c_double, C.c_double, C.c_double,
                                                  C.POINTER(Potential)]),
    "bib_add_pp_interaction": (C.c_int32, [_vp, C.c_int32, C.POINTER(Potential)]),
    "bib_clear_interactions": (C.c_int32, [_vp, C.c_int32]),
    "bib_particle_info": (C.c_int32, [_vp, C.c_int32, C.c_int32, _i32p]),
    "bib_lattice_iteration": (C.c_int32, [_vp, C.c_int32, _ip]),
    "bib_checkpoint_save": (C.c_int32, [_vp, C.c_int32, C.c_char_p]),
    "bib_particles_save_plb": (C.c_int32, [_vp, C.c_int32, C.c_char_p, C.c_char_p]),
    "bib_particles_load_plb": (C.c_int32, [_vp, C.c_int32, C.c_char_p, C.c_char_p]),
    "bib_particles_write_vtu": (C.c_int32, [_vp, C.c_int32, C.c_char_p, C.c_uint64]),
    "bib_particle_write_vtu": (C.c_int32, [_vp, C.c_int32, C.c_int32, C.c_char_p]),
    "bib_particles_write_lightweight": (C.c_int32, [_vp, C.c_int32, C.c_char_p, C.c_uint64]),
    "bib_lattice_save_plb": (C.c_int32, [_vp, C.c_int32, C.c_char_p, C.c_char_p]),
    "bib_rbc_params": (C.c_int32, [_vp, C.c_int32, C.c_double, C.c_double, C.c_double, _dp]),
    "bib_rbc_shrink_volume": (C.c_int32, [_vp, C.c_int32, _dp, C.c_double, C.c_int64, C.c_double, _dp, _dp]),
    "bib_align_minor_axis": (C.c_int32, [_vp, C.c_int32, _dp, _dp]),
    "bib_grow_particles": (C.c_int32, [_vp, C.POINTER(Growth), C.c_int32, _i32p, _dp, _dp, _dp, _dp]),
    "bib_place_particle": (C.c_int32, [_vp, C.c_int32, _dp, _dp, _dp, _dp]),
    "bib_initial_distribution": (C.c_int32, [C.POINTER(C.c_int64), _dp, C.c_int32, C.POINTER(C.c_int64), _dp,
                                             C.c_double, C.c_uint32, C.c_int64, _dp, _dp]),
    "bib_lattice_load_plb": (C.c_int32, [_vp, C.c_int32, C.c_char_p, C.c_char_p]),
    "bib_checkpoint_load": (C.c_int32, [_vp, C.c_int32, C.c_char_p]),
    "bib_step": (C.c_int32, [_vp, C.c_int32, C.c_int64]),
    "bib_step_timed": (C.c_int32, [_vp, C.c_int32, C.c_int64, _dp]),
    "bib_step_kernel_count": (C.c_int32, [_vp, C.c_int32, _i32p]),
    "bib_check_health": (C.c_int32, [_vp, C.c_int32]),
    "bib_lattice_set_tuning": (C.c_int32, [_vp, C.c_int32, C.POINTER(Tuning)]),
    "bib_lattice_set_cell_types": (C.c_int32, [_vp, C.c_int32, _vp]),
    "bib_spread_forces_noalloc": (C.c_int32, [_vp, C.c_int32, _vp, _vp, C.c_int64, _vp]),
    "bib_batch_create": (C.c_int32, [_vp, _i32p, C.c_int32, _i32p]),
    "bib_batch_destroy": (C.c_int32, [_vp, C.c_int32]),
    "bib_batch_step": (C.c_int32, [_vp, C.c_int32, C.c_int64]),
    "bib_batch_step_timed": (C.c_int32, [_vp, C.c_int32, C.c_int64, _dp]),
    "bib_batch_set_tuning": (C.c_int32, [_vp, C.c_int32, C.POINTER(BatchTuning)]),
    "bib_batch_autotune": (C.c_int32, [_vp, C.c_int32, C.c_int32, C.POINTER(BatchTuning)]),
}

_lib = None


class BibError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s (%d): %s" % (status_string(status), status, message))
        self.status = status


def load(path: str = LIB_PATH):
    """Load the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            "biblbm_gb300 CUDA library not found at %s; build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'` or `python biblbm_gb300/build.py`" % path)
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def status_string(s: int) -> str:
    try:
        return load().bib_status_string(s).decode()
    except Exception:  # pragma: no cover - used while formatting another error
        return "status"


def exported_symbols():
    return list(SIGNATURES)
