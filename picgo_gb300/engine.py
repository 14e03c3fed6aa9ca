"""Python front end of the C ABI: one :class:`Engine` owns one device context.

The calls mirror the reference's force-field manager and minimizer seam
(medyan-5.4.0/src/Mechanics/ForceField/ForceFieldManager.h:64-123 and
Mechanics/Minimizer/CGMethod.hpp:826-836): ``energies`` is
computeIndividualEnergies / computeEnergy, ``forces`` is computeForces,
``minimize`` is CGMethod::minimize with MController's recovery move.
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from . import _lib
from ._lib import (MechCGParams, MechListInfo, MechNetwork, MechProfile, MechResult, MechSolveInfo, MechSolveParams,
                   MechTiming, MechTuning, check)

_dp = C.POINTER(C.c_double)
_i32p = C.POINTER(C.c_int32)
_i64p = C.POINTER(C.c_int64)


def _ptr(a, t):
    return a.ctypes.data_as(t) if a is not None and a.size else None


def network_struct(net, keep: list) -> MechNetwork:
    """MechNetwork view of a :class:`picgo_gb300.network.Network` (arrays kept alive in ``keep``)."""
    def arr(x, dt):
        a = np.ascontiguousarray(x, dtype=dt)
        keep.append(a)
        return a
    s = MechNetwork()
    coord = arr(net.coord, np.float64)
    s.n_beads = net.n_beads
    s.coord = _ptr(coord, _dp)
    s.n_filaments = net.n_filaments
    s.fil_cyl_start = _ptr(arr(net.fil_cyl_start, np.int32), _i32p)
    s.n_cylinders = net.n_cyl
    s.cyl_bead = _ptr(arr(np.stack([net.cyl_b1, net.cyl_b2], 1), np.int32), _i32p)
    s.cyl_id = _ptr(arr(net.cyl_id, np.int64), _i64p)
    s.cyl_filament_id = _ptr(arr(net.cyl_fil, np.int32), _i32p)
    s.cyl_position = _ptr(arr(net.cyl_pos, np.int32), _i32p)
    s.cyl_type = _ptr(arr(net.cyl_type, np.int32), _i32p)
    s.cyl_eq_length = _ptr(arr(net.cyl_l0, np.float64), _dp)
    s.cyl_k_stretch = _ptr(arr(net.cyl_kstr, np.float64), _dp)
    s.cyl_k_bend = _ptr(arr(net.cyl_kbend, np.float64), _dp)
    s.cyl_eq_theta = _ptr(arr(net.cyl_theta0, np.float64), _dp)
    s.cyl_k_exvol = _ptr(arr(net.cyl_kexvol, np.float64), _dp)
    s.n_linkers = int(net.lk_cyl.shape[0])
    s.lk_cyl = _ptr(arr(net.lk_cyl, np.int32), _i32p)
    s.lk_pos = _ptr(arr(net.lk_pos, np.float64), _dp)
    s.lk_k = _ptr(arr(net.lk_k, np.float64), _dp)
    s.lk_eq_length = _ptr(arr(net.lk_l0, np.float64), _dp)
    s.n_motors = int(net.mt_cyl.shape[0])
    s.mt_cyl = _ptr(arr(net.mt_cyl, np.int32), _i32p)
    s.mt_pos = _ptr(arr(net.mt_pos, np.float64), _dp)
    s.mt_k = _ptr(arr(net.mt_k, np.float64), _dp)
    s.mt_eq_length = _ptr(arr(net.mt_l0, np.float64), _dp)
    s.n_planes = int(net.planes.shape[0])
    s.planes = _ptr(arr(net.planes, np.float64), _dp)
    s.plane_k = _ptr(arr(net.plane_k, np.float64), _dp)
    s.plane_screen = _ptr(arr(net.plane_slen, np.float64), _dp)
    for k in range(3):
        s.box[k] = float(net.box)
    s.exvol_cutoff = float(net.exvol_cutoff)
    s.boundary_cutoff = float(net.boundary_cutoff)
    return s


def cg_params(method: int = 2, max_dist: float = 1.0, lambda_max: float = 0.01, grad_tol: float = 1.0,
              energy_rel_tol: float = 1e-9, energy_call_limit: int = 0, force_call_limit: int = 10000,
              report_on_call_limit: int = 1, try_to_recover: int = 1) -> MechCGParams:
    """Defaults: MController's CG parameters with the example input's LAMBDAMAX
    (medyan-5.4.0/src/Controller/MController.cpp:34-63, SysParams.h:112-129)."""
    return MechCGParams(method, max_dist, lambda_max, grad_tol, energy_rel_tol, energy_call_limit,
                        force_call_limit, report_on_call_limit, try_to_recover)


class Engine:
    def __init__(self, precision: str | int = "fp64", device: int = 0):
        self._L = _lib.load()
        prec = {"fp64": _lib.PREC_FP64, "mixed": _lib.PREC_MIXED}.get(precision, precision)
        self._ctx = C.c_void_p()
        check(self._L.mech_ctx_create(int(prec), int(device), C.byref(self._ctx)))
        self.precision = prec
        self.nbeads: list[int] = []
        self.nlinkers: list[int] = []
        self.nmotors: list[int] = []

    # -- lifecycle ---------------------------------------------------------
    def close(self):
        if self._ctx:
            self._L.mech_ctx_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- network -----------------------------------------------------------
    def set_networks(self, nets: Sequence) -> None:
        keep: list = []
        arr = (MechNetwork * len(nets))(*[network_struct(n, keep) for n in nets])
        check(self._L.mech_set_networks(self._ctx, len(nets), arr))
        self.nbeads = [n.n_beads for n in nets]
        self.nlinkers = [int(n.lk_cyl.shape[0]) for n in nets]
        self.nmotors = [int(n.mt_cyl.shape[0]) for n in nets]
        self._nfil = [int(n.n_filaments) for n in nets]
        self._ncyl = [int(n.n_cyl) for n in nets]

    def set_network(self, net) -> None:
        self.set_networks([net])

    def set_coords(self, coord: np.ndarray, replica: int = 0) -> None:
        x = np.ascontiguousarray(coord, dtype=np.float64).reshape(-1)
        check(self._L.mech_set_coords(self._ctx, replica, _ptr(x, _dp)))

    def coords(self, replica: int = 0) -> np.ndarray:
        out = np.empty((self.nbeads[replica], 3))
        check(self._L.mech_get_coords(self._ctx, replica, _ptr(out, _dp)))
        return out

    # -- neighbor lists ----------------------------------------------------
    def rebuild(self, cell_size: float = 0.0) -> dict:
        info = MechListInfo()
        check(self._L.mech_rebuild_neighbors(self._ctx, float(cell_size), C.byref(info)))
        return {k: getattr(info, k) for k, _ in info._fields_}

    def pairs(self, replica: int = 0) -> np.ndarray:
        cnt = C.c_int64()
        check(self._L.mech_get_pairs(self._ctx, replica, None, 0, C.byref(cnt)))
        out = np.empty((max(cnt.value, 1), 2), np.int32)
        check(self._L.mech_get_pairs(self._ctx, replica, _ptr(out, _i32p), cnt.value, C.byref(cnt)))
        return out[:cnt.value]

    def boundary_list(self, replica: int = 0) -> np.ndarray:
        """BoundaryCylinderNL entries (plane, cylinder) of the last rebuild, plane by plane."""
        cnt = C.c_int64()
        check(self._L.mech_get_boundary_list(self._ctx, replica, None, 0, C.byref(cnt)))
        out = np.empty((max(cnt.value, 1), 2), np.int32)
        check(self._L.mech_get_boundary_list(self._ctx, replica, _ptr(out, _i32p), cnt.value, C.byref(cnt)))
        return out[:cnt.value]

    def load_forces(self, mon_size=(2.7,), n_mon=(40,), replica: int = 0):
        """Boundary load forces on the filament ends (plus, minus), each [n_filaments, max n_mon]."""
        ms = np.ascontiguousarray(mon_size, dtype=np.float64)
        nm = np.ascontiguousarray(n_mon, dtype=np.int32)
        nfil = self._nfil[replica]
        stride = int(nm.max())
        plus = np.zeros((nfil, stride))
        minus = np.zeros((nfil, stride))
        check(self._L.mech_load_forces(self._ctx, replica, len(ms), _ptr(ms, _dp), _ptr(nm, _i32p), stride,
                                       _ptr(plus, _dp), _ptr(minus, _dp)))
        return plus, minus

    def energy_terms(self, replica: int = 0):
        """Per-cylinder stretching and bending energy terms in the engine's arithmetic (before summing)."""
        n = self._ncyl[replica]
        st = np.zeros(n)
        bd = np.zeros(n)
        check(self._L.mech_energy_terms(self._ctx, replica, _ptr(st, _dp), _ptr(bd, _dp)))
        return st, bd

    # -- evaluation --------------------------------------------------------
    def energies(self, coord: np.ndarray | None = None, replica: int = 0):
        """(per-FF energies, plain total, computeEnergy value)."""
        per = np.zeros(_lib.NUM_FF)
        tot = C.c_double()
        en = C.c_double()
        x = None if coord is None else np.ascontiguousarray(coord, dtype=np.float64).reshape(-1)
        check(self._L.mech_energy(self._ctx, replica, _ptr(x, _dp), _ptr(per, _dp), C.byref(tot), C.byref(en)))
        return per, tot.value, en.value

    def forces(self, coord: np.ndarray | None = None, replica: int = 0) -> np.ndarray:
        out = np.empty((self.nbeads[replica], 3))
        x = None if coord is None else np.ascontiguousarray(coord, dtype=np.float64).reshape(-1)
        check(self._L.mech_forces(self._ctx, replica, _ptr(x, _dp), _ptr(out, _dp)))
        return out

    def last_forces(self, replica: int = 0) -> np.ndarray:
        out = np.empty((self.nbeads[replica], 3))
        check(self._L.mech_get_forces(self._ctx, replica, _ptr(out, _dp)))
        return out

    def stretch_forces(self, replica: int = 0):
        lk = np.zeros(self.nlinkers[replica])
        mt = np.zeros(self.nmotors[replica])
        check(self._L.mech_get_stretch_forces(self._ctx, replica, _ptr(lk, _dp), _ptr(mt, _dp)))
        return lk, mt

    # -- minimization ------------------------------------------------------
    def minimize(self, params: MechCGParams | None = None) -> list[dict]:
        params = params or cg_params()
        res = (MechResult * len(self.nbeads))()
        rc = self._L.mech_minimize(self._ctx, C.byref(params), res)
        if rc not in (_lib.MECH_OK, -5):
            check(rc)
        return [r.as_dict() for r in res]

    def reset_coords(self) -> None:
        check(self._L.mech_reset_coords(self._ctx))

    def set_graph_mode(self, mode: str) -> None:
        """'unrolled' (default): relaunched graphs of 8 unrolled iteration blocks;
        'unrolled_pdl': the same with programmatic dependent launch around the reductions;
        'conditional': one graph whose device while loop runs only the phases in use;
        'unrolled_coop': the unrolled graph with each iteration's tail (gather, reductions, direction, reset) as one
        cooperative launch (mixed, one replica; otherwise as 'unrolled').  Same results."""
        check(self._L.mech_set_graph_mode(self._ctx, {"conditional": 0, "unrolled": 1, "unrolled_pdl": 2,
                                                     "unrolled_coop": 3}[mode]))

    # -- second order (FP64 contexts) -----------------------------------------
    def hvp(self, v: np.ndarray, replica: int = 0, jacobian: bool = False) -> np.ndarray:
        """H v at the current coordinates (caller bead order): the energy's Hessian,
        or with ``jacobian`` minus the Jacobian of the force routine."""
        x = np.ascontiguousarray(v, dtype=np.float64).reshape(-1)
        out = np.empty((self.nbeads[replica], 3))
        check(self._L.mech_hvp(self._ctx, replica, 1 if jacobian else 0, _ptr(x, _dp), _ptr(out, _dp)))
        return out

    def set_linker_params(self, k=None, l0=None, replica: int = 0) -> None:
        kk = None if k is None else np.ascontiguousarray(k, dtype=np.float64)
        ll = None if l0 is None else np.ascontiguousarray(l0, dtype=np.float64)
        check(self._L.mech_set_linker_params(self._ctx, replica, _ptr(kk, _dp), _ptr(ll, _dp)))

    def adjoint(self, dL_dx: np.ndarray, dL_dE: float = 0.0, rel_tol: float = 1e-10, max_iter: int = 20000,
                shift: float = 0.0, replica: int = 0):
        """(dL/dk, dL/dl0, info) per linker at the current (equilibrium) coordinates."""
        g = np.ascontiguousarray(dL_dx, dtype=np.float64).reshape(-1)
        n = self.nlinkers[replica]
        dk = np.zeros(n)
        dl = np.zeros(n)
        sp = MechSolveParams(rel_tol, max_iter, shift)
        info = MechSolveInfo()
        rc = self._L.mech_adjoint(self._ctx, replica, _ptr(g, _dp), float(dL_dE), C.byref(sp), _ptr(dk, _dp),
                                  _ptr(dl, _dp), C.byref(info))
        if rc not in (_lib.MECH_OK, -6):
            check(rc)
        return dk, dl, info.as_dict()

    def newton_refine(self, max_steps: int = 20, force_tol: float = 1e-9, rel_tol: float = 1e-8,
                      max_iter: int = 20000, shift: float = 0.0) -> dict:
        sp = MechSolveParams(rel_tol, max_iter, shift)
        info = MechSolveInfo()
        check(self._L.mech_newton_refine(self._ctx, int(max_steps), float(force_tol), C.byref(sp), C.byref(info)))
        return info.as_dict()

    def autotune(self, kernels: bool = True, cell: bool = True, force: bool = False) -> dict:
        """Time candidate launch geometries / bin edges on this context's networks and keep the fastest."""
        t = MechTuning()
        flags = (1 if kernels else 0) | (2 if cell else 0) | (4 if force else 0)
        check(self._L.mech_autotune(self._ctx, flags, C.byref(t)))
        return {k: getattr(t, k) for k, _ in t._fields_}

    def set_tuning(self, tuning: dict) -> None:
        t = MechTuning(*[tuning[k] for k, _ in MechTuning._fields_])
        check(self._L.mech_set_tuning(self._ctx, C.byref(t)))

    def profile(self, iters: int = 20) -> dict:
        p = MechProfile()
        check(self._L.mech_profile(self._ctx, int(iters), C.byref(p)))
        return {k: getattr(p, k) for k, _ in p._fields_}

    def timing(self) -> dict:
        t = MechTiming()
        check(self._L.mech_get_timing(self._ctx, C.byref(t)))
        return {k: getattr(t, k) for k, _ in t._fields_}
