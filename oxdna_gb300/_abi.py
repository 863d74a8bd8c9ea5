"""ctypes bindings of include/oxgb.h (the library's C ABI).

The library must be built (oxdna_gb300.build.build()); loading fails loudly otherwise -- there
is no CPU fallback anywhere in this package.
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

OK = 0
ERRORS = {1: "invalid argument", 2: "CUDA error", 3: "FENE bond broken", 4: "neighbour row overflow",
          5: "non-finite coordinates", 6: "out of device memory"}

THERMOSTATS = {"no": 0, "none": 0, "john": 1, "brownian": 1, "bussi": 2}
# limits of oxgb_verlet_build_noalloc (OXGB_NOALLOC_MAX_N / OXGB_NOALLOC_MAX_CELLS in oxgb.h)
NOALLOC_MAX_N = 65536
NOALLOC_MAX_CELLS = 32768


class OxgbError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"oxgb error {code} ({ERRORS.get(code, '?')}): {msg}")
        self.code = code


class DNA2Settings(C.Structure):
    _fields_ = [
        ("T", C.c_double), ("salt", C.c_double), ("average", C.c_int), ("seq_stck", (C.c_double * 4) * 4),
        ("seq_stck_fact_eps", C.c_double), ("seq_hydr_at", C.c_double), ("seq_hydr_gc", C.c_double),
        ("hb_multiplier", C.c_double), ("dh_half_charged_ends", C.c_int), ("dh_lambda", C.c_double),
        ("dh_strength", C.c_double), ("use_mbf", C.c_int), ("mbf_fmax", C.c_double), ("mbf_finf", C.c_double),
        ("reference_cuda_eps", C.c_int),
    ]


class ExtForce(C.Structure):
    _fields_ = [
        ("type", C.c_int), ("particle", C.c_int), ("ref_particle", C.c_int), ("flags", C.c_int),
        ("F0", C.c_double), ("rate", C.c_double), ("stiff", C.c_double), ("stiff_rate", C.c_double),
        ("r0", C.c_double), ("position", C.c_double), ("dir", C.c_double * 3), ("pos0", C.c_double * 3),
        ("sigma", C.c_double), ("cutoff", C.c_double), ("p1", C.c_double), ("p2", C.c_double),
        ("n", C.c_int), ("pad", C.c_int), ("v1", C.c_double * 3), ("v2", C.c_double * 3),
    ]


FORCE_TYPES = {"constant": 0, "string": 0, "mutual_trap": 1, "trap": 2, "moving_trap": 2, "lowdim_trap": 3,
               "repulsion_plane": 4, "attraction_plane": 5, "sphere": 6, "sphere_smooth": 7, "LJ_wall": 8,
               "generic_central_force": 9, "repulsion_plane_moving": 10, "LJ_cone": 11, "twist": 12, "ellipsoid": 13,
               "com": 14, "yukawa_sphere": 15, "repulsive_sphere_moving": 16}


class MDSettings(C.Structure):
    _fields_ = [
        ("dt", C.c_double), ("verlet_skin", C.c_double), ("thermostat", C.c_int), ("newtonian_steps", C.c_int),
        ("pt", C.c_double), ("diff_coeff", C.c_double), ("bussi_tau", C.c_double), ("seed", C.c_uint64),
        ("precision", C.c_int), ("cells_auto_optimisation", C.c_int), ("max_neigh", C.c_int),
        ("steps_per_graph", C.c_int), ("list_rebuild_node", C.c_int), ("sort_every", C.c_int),
        ("autotune", C.c_int),
        ("use_edge", C.c_int),
        ("sort_order", C.c_int),
        ("list_kernel", C.c_int),
    ]


_lib = None

# every entry point include/oxgb.h declares, with its ctypes signature
_VP = C.c_void_p
_DP = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_IP = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
SIGNATURES = {
    "oxgb_version": (C.c_char_p, []),
    "oxgb_last_error": (C.c_char_p, []),
    "oxgb_dna2_default_settings": (None, [C.POINTER(DNA2Settings), C.c_double, C.c_double]),
    "oxgb_md_default_settings": (None, [C.POINTER(MDSettings)]),
    "oxgb_dna2_create": (C.c_int, [C.POINTER(DNA2Settings), C.POINTER(_VP)]),
    "oxgb_dna2_get_rcut": (C.c_int, [_VP, C.POINTER(C.c_double)]),
    "oxgb_dna2_set_temperature": (C.c_int, [_VP, C.c_double]),
    "oxgb_dna2_compute_forces": (C.c_int, [_VP, C.c_int, C.c_double, _VP, _VP, _VP, _VP, _VP, _VP, _VP, C.c_int,
                                           C.c_longlong, C.c_longlong, _VP]),
    "oxgb_dna2_hb_op_precalc": (C.c_int, [_VP, C.c_double, _VP, _VP, _VP, _VP, C.c_int, _VP, _VP]),
    "oxgb_dna2_near_hb_op_precalc": (C.c_int, [_VP, C.c_double, _VP, _VP, _VP, _VP, C.c_int, _VP, _VP]),
    "oxgb_dna2_dist_op_precalc": (C.c_int, [_VP, C.c_double, _VP, _VP, _VP, _VP, C.c_int, _VP, _VP]),
    "oxgb_dna2_destroy": (C.c_int, [_VP]),
    "oxgb_verlet_create": (C.c_int, [C.c_int, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, C.POINTER(_VP)]),
    "oxgb_verlet_update": (C.c_int, [_VP, _VP, _VP, _VP, _VP]),
    "oxgb_verlet_build_noalloc": (C.c_int, [C.c_int, C.c_double, C.c_double, C.c_double, C.c_int, _VP, _VP, _VP, _VP, _VP,
                                            C.c_int, _VP]),
    "oxgb_verlet_buffers": (C.c_int, [_VP, C.POINTER(_VP), C.POINTER(_VP), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "oxgb_verlet_status": (C.c_int, [_VP]),
    "oxgb_verlet_destroy": (C.c_int, [_VP]),
    "oxgb_md_create": (C.c_int, [C.c_int, _IP, _DP, C.POINTER(DNA2Settings), C.POINTER(MDSettings), C.POINTER(_VP)]),
    "oxgb_md_set_topology": (C.c_int, [_VP, _IP, _IP, _IP, _IP]),
    "oxgb_md_set_state": (C.c_int, [_VP, _DP, _DP, _DP, _DP]),
    "oxgb_md_get_state": (C.c_int, [_VP, _VP, _VP, _VP, _VP]),
    "oxgb_md_run": (C.c_int, [_VP, C.c_int, C.c_int]),
    "oxgb_md_compute_forces": (C.c_int, [_VP, _VP, _VP, _VP, _VP]),
    "oxgb_md_get_forces": (C.c_int, [_VP, _VP, _VP, _VP]),
    "oxgb_md_scale_momenta": (C.c_int, [_VP, C.c_int, C.c_double]),
    "oxgb_md_set_external_forces": (C.c_int, [_VP, C.c_int, C.POINTER(ExtForce)]),
    "oxgb_md_set_force_groups": (C.c_int, [_VP, C.c_int, _VP, _VP]),
    "oxgb_md_energies": (C.c_int, [_VP, _VP, _VP, _VP]),
    "oxgb_md_force_shape": (C.c_int, [_VP, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                      C.POINTER(C.c_double)]),
    "oxgb_md_set_force_shape": (C.c_int, [_VP, C.c_int]),
    "oxgb_force_shape_table": (C.c_int, [C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "oxgb_md_list_kernel": (C.c_int, [_VP, C.POINTER(C.c_int)]),
    "oxgb_md_set_temperature": (C.c_int, [_VP, C.c_int, C.c_double]),
    "oxgb_md_neighbours": (C.c_int, [_VP, _VP, _VP, C.c_int, _VP, _VP]),
    "oxgb_md_info": (C.c_int, [_VP, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong), C.POINTER(C.c_int)]),
    "oxgb_md_storage_order": (C.c_int, [_VP, _VP]),
    "oxgb_md_status": (C.c_int, [_VP]),
    "oxgb_md_device_buffers": (C.c_int, [_VP, C.POINTER(_VP), C.POINTER(_VP), C.POINTER(_VP), C.POINTER(_VP),
                                         C.POINTER(_VP), C.POINTER(_VP)]),
    "oxgb_md_stream": (_VP, [_VP]),
    "oxgb_md_launch_forces": (C.c_int, [_VP]),
    "oxgb_probe_fp32_peak": (C.c_int, [C.POINTER(C.c_double)]),
    "oxgb_md_destroy": (C.c_int, [_VP]),
}


def library_path() -> str:
    return _build.LIB


def lib(build_if_missing: bool = True):
    """Load liboxgb.so (building it first if needed)."""
    global _lib
    if _lib is None:
        path = _build.build() if build_if_missing else _build.LIB
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: build the CUDA library first (oxdna_gb300.build.build())")
        L = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(rc: int):
    if rc != OK:
        msg = lib().oxgb_last_error()
        raise OxgbError(rc, msg.decode() if msg else "")


def ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None
