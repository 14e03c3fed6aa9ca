"""ctypes declarations of include/medyan_mech.h and the loader of libmedyan_mech.so.

There is no CPU fallback: if the library is missing or no CUDA device is
visible, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import build as _build

_dp = C.POINTER(C.c_double)
_i32p = C.POINTER(C.c_int32)
_i64p = C.POINTER(C.c_int64)

MECH_OK = 0
ERRORS = {
    -1: "MECH_ERR_ARG", -2: "MECH_ERR_TOPOLOGY", -3: "MECH_ERR_CUDA", -4: "MECH_ERR_NONFINITE",
    -5: "MECH_ERR_LINESEARCH", -6: "MECH_ERR_ITER_LIMIT", -7: "MECH_ERR_CAPACITY", -8: "MECH_ERR_NO_DEVICE",
    -9: "MECH_ERR_STATE",
}
PREC_FP64 = 0
PREC_MIXED = 1
NUM_FF = 6
FF_NAMES = ["FilamentStretching", "FilamentBending", "LinkerStretching", "MotorStretching",
            "CylinderExcludeVolume", "BoundaryCylinderRepulsion"]

# Every symbol include/medyan_mech.h declares.
EXPORTS = [
    "mech_abi_version", "mech_last_error", "mech_ctx_create", "mech_ctx_destroy", "mech_set_networks",
    "mech_set_coords", "mech_get_coords", "mech_rebuild_neighbors", "mech_get_pairs", "mech_energy",
    "mech_forces", "mech_minimize", "mech_get_forces", "mech_get_stretch_forces", "mech_get_timing",
    "mech_reset_coords", "mech_profile", "mech_filament_energy_device", "mech_hvp", "mech_set_linker_params",
    "mech_adjoint", "mech_newton_refine", "mech_autotune", "mech_set_tuning", "mech_set_graph_mode", "mech_get_boundary_list",
    "mech_load_forces", "mech_energy_terms",
]


class MechNetwork(C.Structure):
    _fields_ = [
        ("n_beads", C.c_int32), ("coord", _dp),
        ("n_filaments", C.c_int32), ("fil_cyl_start", _i32p),
        ("n_cylinders", C.c_int32), ("cyl_bead", _i32p), ("cyl_id", _i64p), ("cyl_filament_id", _i32p),
        ("cyl_position", _i32p), ("cyl_type", _i32p), ("cyl_eq_length", _dp), ("cyl_k_stretch", _dp),
        ("cyl_k_bend", _dp), ("cyl_eq_theta", _dp), ("cyl_k_exvol", _dp),
        ("n_linkers", C.c_int32), ("lk_cyl", _i32p), ("lk_pos", _dp), ("lk_k", _dp), ("lk_eq_length", _dp),
        ("n_motors", C.c_int32), ("mt_cyl", _i32p), ("mt_pos", _dp), ("mt_k", _dp), ("mt_eq_length", _dp),
        ("n_planes", C.c_int32), ("planes", _dp), ("plane_k", _dp), ("plane_screen", _dp),
        ("box", C.c_double * 3), ("exvol_cutoff", C.c_double), ("boundary_cutoff", C.c_double),
    ]


class MechCGParams(C.Structure):
    _fields_ = [("method", C.c_int32), ("max_dist", C.c_double), ("lambda_max", C.c_double),
                ("grad_tol", C.c_double), ("energy_rel_tol", C.c_double), ("energy_call_limit", C.c_int32),
                ("force_call_limit", C.c_int32), ("report_on_call_limit", C.c_int32),
                ("try_to_recover", C.c_int32)]


class MechResult(C.Structure):
    _fields_ = [("error_flags", C.c_uint32), ("status", C.c_int32), ("num_energy_call", C.c_int32),
                ("energy_call_limit", C.c_int32), ("num_force_call", C.c_int32), ("force_call_limit", C.c_int32),
                ("num_iter", C.c_int32), ("num_safe_mode", C.c_int32), ("num_recover", C.c_int32),
                ("num_line_search_trials", C.c_int32), ("num_energy_eval", C.c_int32), ("used_backup", C.c_int32),
                ("grad_inf_norm", C.c_double), ("grad_tol", C.c_double), ("energy_rel_change", C.c_double),
                ("energy_rel_tol", C.c_double), ("energies_before", C.c_double * (NUM_FF + 1)),
                ("energies_after", C.c_double * (NUM_FF + 1)), ("seconds", C.c_double)]

    def as_dict(self) -> dict:
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            out[name] = list(v) if isinstance(v, C.Array) else v
        return out


class MechListInfo(C.Structure):
    _fields_ = [("n_exvol_pairs", C.c_int64), ("n_boundary_beads", C.c_int64), ("n_boundary_cyl", C.c_int64),
                ("cell_size", C.c_double), ("n_cells", C.c_int64)]


class MechTiming(C.Structure):
    _fields_ = [("ms_total", C.c_double), ("ms_line_search", C.c_double), ("ms_force", C.c_double),
                ("ms_direction", C.c_double), ("ms_rebuild", C.c_double), ("launches", C.c_int64),
                ("graph_launches", C.c_int64)]


class MechProfile(C.Structure):
    _fields_ = [("ms_energy_eval", C.c_double), ("ms_force_eval", C.c_double), ("ms_fil_energy", C.c_double),
                ("ms_fil_force", C.c_double), ("ms_bond_energy", C.c_double), ("ms_bond_force", C.c_double),
                ("ms_exvol_energy", C.c_double), ("ms_exvol_force", C.c_double), ("n_beads", C.c_int64),
                ("n_exvol_pairs", C.c_int64), ("n_boundary", C.c_int64), ("n_linkers", C.c_int64),
                ("n_motors", C.c_int64), ("n_slots", C.c_int64), ("n_exvol_ext_energy", C.c_int64),
                ("n_exvol_ext_force", C.c_int64), ("ms_iteration_idle", C.c_double),
                ("ms_trial_energy_eval", C.c_double), ("n_exvol_fallback_energy", C.c_int64),
                ("n_exvol_fallback_force", C.c_int64), ("ms_fil_energy_trial", C.c_double),
                ("ms_fil_force_kernel", C.c_double), ("ms_force_gather", C.c_double)]


class MechSolveParams(C.Structure):
    _fields_ = [("rel_tol", C.c_double), ("max_iter", C.c_int32), ("shift", C.c_double)]


class MechSolveInfo(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("converged", C.c_int32), ("rel_residual", C.c_double),
                ("launches", C.c_int64), ("newton_steps", C.c_int32), ("max_force", C.c_double),
                ("negative_curvature", C.c_int32)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class MechTuning(C.Structure):
    _fields_ = [("energy_tiles_per_block", C.c_int32), ("force_tiles_per_block", C.c_int32),
                ("cell_scale", C.c_double), ("ms_energy", C.c_double), ("ms_force", C.c_double),
                ("ms_rebuild", C.c_double), ("energy_blocks_per_sm", C.c_int32),
                ("force_blocks_per_sm", C.c_int32)]


_lock = threading.Lock()
_lib = None


class MechError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


def load(build_if_missing: bool = False):
    """Load libmedyan_mech.so (in-tree).  Raises if it is not built."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.lib_path()
        if not os.path.exists(path):
            if not build_if_missing:
                raise RuntimeError(f"{path} is not built; run picgo_gb300.build.build() (there is no CPU fallback)")
            _build.build()
        L = C.CDLL(path)
        vp = C.c_void_p
        L.mech_abi_version.restype = C.c_int32
        L.mech_last_error.restype = C.c_char_p
        L.mech_ctx_create.argtypes = [C.c_int32, C.c_int32, C.POINTER(vp)]
        L.mech_ctx_destroy.argtypes = [vp]
        L.mech_set_networks.argtypes = [vp, C.c_int32, C.POINTER(MechNetwork)]
        L.mech_set_coords.argtypes = [vp, C.c_int32, _dp]
        L.mech_get_coords.argtypes = [vp, C.c_int32, _dp]
        L.mech_rebuild_neighbors.argtypes = [vp, C.c_double, C.POINTER(MechListInfo)]
        L.mech_get_pairs.argtypes = [vp, C.c_int32, _i32p, C.c_int64, _i64p]
        L.mech_get_boundary_list.argtypes = [vp, C.c_int32, _i32p, C.c_int64, _i64p]
        L.mech_energy_terms.argtypes = [vp, C.c_int32, _dp, _dp]
        L.mech_load_forces.argtypes = [vp, C.c_int32, C.c_int32, _dp, _i32p, C.c_int32, _dp, _dp]
        L.mech_energy.argtypes = [vp, C.c_int32, _dp, _dp, _dp, _dp]
        L.mech_forces.argtypes = [vp, C.c_int32, _dp, _dp]
        L.mech_minimize.argtypes = [vp, C.POINTER(MechCGParams), C.POINTER(MechResult)]
        L.mech_get_forces.argtypes = [vp, C.c_int32, _dp]
        L.mech_get_stretch_forces.argtypes = [vp, C.c_int32, _dp, _dp]
        L.mech_get_timing.argtypes = [vp, C.POINTER(MechTiming)]
        L.mech_reset_coords.argtypes = [vp]
        L.mech_profile.argtypes = [vp, C.c_int32, C.POINTER(MechProfile)]
        L.mech_filament_energy_device.argtypes = [C.c_int32, C.c_int32, vp, vp, vp, vp, vp, vp, vp, vp]
        L.mech_hvp.argtypes = [vp, C.c_int32, C.c_int32, _dp, _dp]
        L.mech_autotune.argtypes = [vp, C.c_int32, C.POINTER(MechTuning)]
        L.mech_set_tuning.argtypes = [vp, C.POINTER(MechTuning)]
        L.mech_set_graph_mode.argtypes = [vp, C.c_int32]
        L.mech_set_linker_params.argtypes = [vp, C.c_int32, _dp, _dp]
        L.mech_adjoint.argtypes = [vp, C.c_int32, _dp, C.c_double, C.POINTER(MechSolveParams), _dp, _dp,
                                   C.POINTER(MechSolveInfo)]
        L.mech_newton_refine.argtypes = [vp, C.c_int32, C.c_double, C.POINTER(MechSolveParams),
                                         C.POINTER(MechSolveInfo)]
        for name in EXPORTS:
            f = getattr(L, name)
            if f.restype is None or f.restype is C.c_int:
                f.restype = C.c_int32 if name not in ("mech_last_error",) else C.c_char_p
        _lib = L
        return L


def check(rc: int):
    if rc != MECH_OK:
        msg = load().mech_last_error()
        raise MechError(rc, msg.decode() if msg else "")
    return rc
