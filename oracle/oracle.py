"""ctypes front end of the C++ oracle (``mech_oracle.cpp``) plus the
reference-view vectorization of a network.

TEST INFRASTRUCTURE ONLY (see the package docstring).

``vectorize`` mirrors what MEDYAN's force fields build in ``vectorize()``:
coordinate offsets (3 x bead index) and per-interaction constants, in the
reference's interaction order:

* stretching: one entry per cylinder in database order
  (medyan-5.4.0/src/Mechanics/ForceField/Filament/FilamentStretching.cpp:26-44);
* bending: per filament, per consecutive cylinder pair, beads
  (b1 of previous, b1 of current, b2 of current) and the current cylinder's
  constants (FilamentBending.cpp:30-65);
* linker / motor: beads (b1, b2) of the first cylinder then of the second
  (LinkerStretching.cpp:29-60);
* excluded volume: per cylinder in database order, per neighbor in its half
  list, beads of the cylinder then of the neighbor, k = VolumeK (max of the two
  for mixed types) and both rest lengths (CylinderExclVolume.cpp:33-139);
* boundary: per plane, per neighboring cylinder, the first bead when the
  cylinder is a filament minus end, then the second bead
  (BoundaryCylinderRepulsion.cpp:33-88).
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIBPATH = os.path.join(_HERE, "liboracle.so")
_lock = threading.Lock()
_lib = None

FF_NAMES = ["FilamentStretching", "FilamentBending", "LinkerStretching", "MotorStretching",
            "CylinderExcludeVolume", "BoundaryCylinderRepulsion"]

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_i32p = C.POINTER(C.c_int32)
_i64p = C.POINTER(C.c_int64)


def build(force: bool = False) -> str:
    """Compile liboracle.so from mech_oracle.cpp (make)."""
    src = os.path.join(_HERE, "mech_oracle.cpp")
    if force or not os.path.exists(_LIBPATH) or os.path.getmtime(_LIBPATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIBPATH


class System(C.Structure):
    _fields_ = [
        ("n_stretch", C.c_int), ("st_bs", _ip), ("st_k", _dp), ("st_l0", _dp),
        ("n_bend", C.c_int), ("bd_bs", _ip), ("bd_k", _dp), ("bd_t0", _dp),
        ("n_linker", C.c_int), ("lk_bs", _ip), ("lk_k", _dp), ("lk_l0", _dp), ("lk_s1", _dp), ("lk_s2", _dp),
        ("n_motor", C.c_int), ("mt_bs", _ip), ("mt_k", _dp), ("mt_l0", _dp), ("mt_s1", _dp), ("mt_s2", _dp),
        ("n_exvol", C.c_int), ("ev_bs", _ip), ("ev_k", _dp), ("ev_len", _dp),
        ("n_planes", C.c_int), ("planes", _dp), ("bd_nn", _ip), ("bb_bs", _ip), ("bb_k", _dp), ("bb_slen", _dp),
    ]


class CGParams(C.Structure):
    _fields_ = [("method", C.c_int), ("maxDist", C.c_double), ("lambdaMax", C.c_double),
                ("gradTol", C.c_double), ("energyRelTol", C.c_double), ("energyCallLimit", C.c_int),
                ("forceCallLimit", C.c_int), ("reportOnCallLimit", C.c_int), ("tryToRecover", C.c_int)]


class CGResult(C.Structure):
    _fields_ = [("errorFlags", C.c_uint32), ("numEnergyCall", C.c_int), ("energyCallLimit", C.c_int),
                ("numForceCall", C.c_int), ("forceCallLimit", C.c_int), ("numIter", C.c_int),
                ("numSafeMode", C.c_int), ("numRecover", C.c_int), ("numLineSearchTrials", C.c_int),
                ("gradInfNorm", C.c_double), ("gradTol", C.c_double), ("energyRelChange", C.c_double),
                ("energyRelTol", C.c_double), ("energiesBefore", C.c_double * 7),
                ("energiesAfter", C.c_double * 7), ("usedBackup", C.c_int), ("status", C.c_int)]


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(_LIBPATH)
            L.orc_system_energy.restype = C.c_double
            L.orc_system_energy.argtypes = [C.POINTER(System), _dp]
            L.orc_system_energies.restype = C.c_double
            L.orc_system_energies.argtypes = [C.POINTER(System), _dp, _dp]
            L.orc_system_forces.restype = C.c_int
            L.orc_system_forces.argtypes = [C.POINTER(System), _dp, _dp, C.c_int, _dp, _dp]
            L.orc_minimize.restype = C.c_int
            L.orc_minimize.argtypes = [C.POINTER(System), C.POINTER(CGParams), _dp, C.c_int, C.c_int, _dp,
                                       C.POINTER(CGResult)]
            L.orc_minimize_quadratic.restype = C.c_int
            L.orc_minimize_quadratic.argtypes = [C.c_int, _dp, _dp, C.POINTER(CGParams), _dp, _dp,
                                                 C.POINTER(CGResult)]
            L.orc_cyl_pairs.restype = C.c_int64
            L.orc_cyl_pairs.argtypes = [C.c_int, _dp, _i64p, _ip, _ip, _ip, C.c_double, C.c_double, _i32p,
                                        C.c_int64]
            L.orc_cyl_pairs_binned.restype = C.c_int64
            L.orc_cyl_pairs_binned.argtypes = [C.c_int, _dp, _i64p, _ip, _ip, _ip, C.c_double, C.c_double,
                                               C.c_double, C.c_double, _i32p, C.c_int64]
            L.orc_boundary_list.restype = C.c_int64
            L.orc_boundary_list.argtypes = [C.c_int, _dp, _ip, _ip, C.c_int, _dp, C.c_double, _ip, _i32p,
                                            C.c_int64]
            for nm in ("orc_exvol_energy", "orc_boundary_energy", "orc_stretch_energy", "orc_bend_energy",
                       "orc_bond_energy", "orc_exvol_pair_energy", "orc_plane_distance"):
                getattr(L, nm).restype = C.c_double
            L.orc_exvol_energy.argtypes = [_dp, C.c_int, _ip, _dp, _dp]
            L.orc_exvol_forces.restype = C.c_int
            L.orc_exvol_forces.argtypes = [_dp, _dp, C.c_int, _ip, _dp, _dp]
            L.orc_boundary_energy.argtypes = [_dp, C.c_int, _dp, _ip, _ip, _dp, _dp]
            L.orc_boundary_forces.argtypes = [_dp, _dp, C.c_int, _dp, _ip, _ip, _dp, _dp]
            L.orc_set_exvol_force_nodes.argtypes = [C.c_int]
            L.orc_set_series_atan.argtypes = [C.c_int]
            L.orc_series_atan.restype = C.c_double
            L.orc_series_atan.argtypes = [C.c_double]
            L.orc_system_force_scale.argtypes = [C.POINTER(System), _dp, _dp, C.c_int]
            L.orc_set_threads.argtypes = [C.c_int]
            L.orc_boundary_load_forces.restype = C.c_int
            L.orc_boundary_load_forces.argtypes = [C.c_int, _ip, _ip, _ip, _ip, _dp, C.c_int, _dp, _dp, _dp, _ip,
                                                   _i32p, _dp, _ip, C.c_int, _dp, _dp]
            L.orc_get_threads.restype = C.c_int
            _lib = L
    return _lib


def _p(a, t=_dp):
    return a.ctypes.data_as(t)


@dataclasses.dataclass
class Vectorized:
    """Reference-view arrays of one network; keeps the numpy buffers alive."""
    arrays: dict
    system: System
    ndof: int
    nbeads: int
    pairs: np.ndarray          # (P, 2) cylinder indices of the excluded-volume half list
    bnd_cyl: np.ndarray        # boundary-list cylinder indices, plane by plane
    bnd_nn: np.ndarray         # cylinders per plane


def cyl_midpoints(coord: np.ndarray, b1: np.ndarray, b2: np.ndarray) -> np.ndarray:
    """0.5 * (b1 + b2), the cylinder database coordinate (Cylinder.cpp:45-46)."""
    return 0.5 * (coord[b1] + coord[b2])


def cyl_pairs(net, coord=None, binned: bool = False, cell: float | None = None) -> np.ndarray:
    """Half cylinder-pair list (c, n), id_c > id_n, sorted by c then n."""
    L = lib()
    coord = net.coord if coord is None else coord
    mid = np.ascontiguousarray(cyl_midpoints(coord, net.cyl_b1, net.cyl_b2))
    ids = np.ascontiguousarray(net.cyl_id, dtype=np.int64)
    fil = np.ascontiguousarray(net.cyl_fil, dtype=np.int32)
    pos = np.ascontiguousarray(net.cyl_pos, dtype=np.int32)
    typ = np.ascontiguousarray(net.cyl_type, dtype=np.int32)
    cap = 1 << 16
    while True:
        out = np.empty((cap, 2), np.int32)
        if binned:
            n = L.orc_cyl_pairs_binned(net.n_cyl, _p(mid), _p(ids, _i64p), _p(fil, _ip), _p(pos, _ip),
                                       _p(typ, _ip), net.exvol_cutoff, 0.0, net.box,
                                       float(cell or 1.125 * net.exvol_cutoff), _p(out, _i32p), cap)
        else:
            n = L.orc_cyl_pairs(net.n_cyl, _p(mid), _p(ids, _i64p), _p(fil, _ip), _p(pos, _ip), _p(typ, _ip),
                                net.exvol_cutoff, 0.0, _p(out, _i32p), cap)
        if n <= cap:
            return out[:n].copy()
        cap = int(n)


def cyl_pairs_fast(net, coord=None) -> np.ndarray:
    """Same set as :func:`cyl_pairs` from a KD-tree (for networks too large for O(n^2)).

    Candidates come from a radius query slightly larger than the cutoff; the
    reference predicate is then applied exactly (d^2 in double against the
    float-rounded rMax^2).
    """
    from scipy.spatial import cKDTree
    coord = net.coord if coord is None else coord
    mid = cyl_midpoints(coord, net.cyl_b1, net.cyl_b2)
    rmaxsq = float(np.float32(net.exvol_cutoff * net.exvol_cutoff))
    cand = cKDTree(mid).query_pairs(net.exvol_cutoff * (1 + 1e-6) + 1e-6, output_type="ndarray")
    if cand.size == 0:
        return np.zeros((0, 2), np.int32)
    i, j = cand[:, 0], cand[:, 1]
    c = np.where(net.cyl_id[i] > net.cyl_id[j], i, j)
    n = np.where(net.cyl_id[i] > net.cyl_id[j], j, i)
    same = (net.cyl_fil[c] == net.cyl_fil[n]) & (np.abs(net.cyl_pos[c] - net.cyl_pos[n]) <= 2)
    ok = ~same
    dx = mid[n] - mid[c]
    d2 = ((0.0 + dx[:, 0] * dx[:, 0]) + dx[:, 1] * dx[:, 1]) + dx[:, 2] * dx[:, 2]
    ok &= (d2 >= 0.0) & (d2 <= rmaxsq)
    pairs = np.stack([c[ok], n[ok]], axis=1).astype(np.int32)
    order = np.lexsort((pairs[:, 1], pairs[:, 0]))
    return pairs[order]


def boundary_list(net, coord=None):
    L = lib()
    coord = np.ascontiguousarray(net.coord if coord is None else coord)
    b1 = np.ascontiguousarray(net.cyl_b1, dtype=np.int32)
    b2 = np.ascontiguousarray(net.cyl_b2, dtype=np.int32)
    planes = np.ascontiguousarray(net.planes, dtype=np.float64)
    nn = np.zeros(planes.shape[0], np.int32)
    cap = max(1024, 6 * net.n_cyl)
    out = np.empty(cap, np.int32)
    m = L.orc_boundary_list(net.n_cyl, _p(coord), _p(b1, _ip), _p(b2, _ip), planes.shape[0], _p(planes),
                            net.boundary_cutoff, _p(nn, _ip), _p(out, _i32p), cap)
    return out[:m].copy(), nn


def vectorize(net, coord=None, pairs=None, bnd=None) -> Vectorized:
    """Build the reference-view FF arrays of ``net`` at ``coord`` (default: its coordinates).

    The neighbor lists are rebuilt at ``coord`` unless given, as MEDYAN does
    once before each minimization (Controller.cpp:1617-1625).
    """
    coord = net.coord if coord is None else coord
    b1 = net.cyl_b1.astype(np.int64)
    b2 = net.cyl_b2.astype(np.int64)
    A = {}
    A["st_bs"] = np.ascontiguousarray(np.stack([3 * b1, 3 * b2], 1).reshape(-1), dtype=np.int32)
    A["st_k"] = np.ascontiguousarray(net.cyl_kstr, dtype=np.float64)
    A["st_l0"] = np.ascontiguousarray(net.cyl_l0, dtype=np.float64)
    # bending triples per filament
    prev, cur = [], []
    for f in range(net.n_filaments):
        s, e = int(net.fil_cyl_start[f]), int(net.fil_cyl_start[f + 1])
        if e - s > 1:
            prev.append(np.arange(s, e - 1))
            cur.append(np.arange(s + 1, e))
    prev = np.concatenate(prev) if prev else np.zeros(0, np.int64)
    cur = np.concatenate(cur) if cur else np.zeros(0, np.int64)
    A["bd_bs"] = np.ascontiguousarray(np.stack([3 * b1[prev], 3 * b1[cur], 3 * b2[cur]], 1).reshape(-1), dtype=np.int32)
    A["bd_k"] = np.ascontiguousarray(net.cyl_kbend[cur], dtype=np.float64)
    A["bd_t0"] = np.ascontiguousarray(net.cyl_theta0[cur], dtype=np.float64)

    def bond(cyl, pos, k, l0, tag):
        c1, c2 = cyl[:, 0].astype(np.int64), cyl[:, 1].astype(np.int64)
        A[tag + "_bs"] = np.ascontiguousarray(np.stack([3 * b1[c1], 3 * b2[c1], 3 * b1[c2], 3 * b2[c2]], 1).reshape(-1),
                                              dtype=np.int32)
        A[tag + "_k"] = np.ascontiguousarray(k, dtype=np.float64)
        A[tag + "_l0"] = np.ascontiguousarray(l0, dtype=np.float64)
        A[tag + "_s1"] = np.ascontiguousarray(pos[:, 0], dtype=np.float64)
        A[tag + "_s2"] = np.ascontiguousarray(pos[:, 1], dtype=np.float64)

    bond(net.lk_cyl, net.lk_pos, net.lk_k, net.lk_l0, "lk")
    bond(net.mt_cyl, net.mt_pos, net.mt_k, net.mt_l0, "mt")

    if pairs is None:
        pairs = cyl_pairs(net, coord) if net.n_cyl <= 20000 else cyl_pairs_fast(net, coord)
    c, n = pairs[:, 0].astype(np.int64), pairs[:, 1].astype(np.int64)
    A["ev_bs"] = np.ascontiguousarray(np.stack([3 * b1[c], 3 * b2[c], 3 * b1[n], 3 * b2[n]], 1).reshape(-1),
                                      dtype=np.int32)
    same = net.cyl_type[c] == net.cyl_type[n]
    A["ev_k"] = np.ascontiguousarray(np.where(same, net.cyl_kexvol[c], np.maximum(net.cyl_kexvol[c], net.cyl_kexvol[n])),
                                     dtype=np.float64)
    A["ev_len"] = np.ascontiguousarray(np.stack([net.cyl_l0[c], net.cyl_l0[n]], 1).reshape(-1), dtype=np.float64)

    if bnd is None:
        bnd = boundary_list(net, coord)
    bcyl, bnn = bnd
    minus = np.zeros(net.n_cyl, bool)
    minus[net.fil_cyl_start[:-1]] = True
    beads, kk, ss, nn = [], [], [], []
    off = 0
    for p in range(net.planes.shape[0]):
        cs = bcyl[off:off + bnn[p]].astype(np.int64)
        off += int(bnn[p])
        m = minus[cs]
        cnt = np.where(m, 2, 1)
        pos = np.repeat(np.arange(cs.size), cnt)
        first = np.ones(pos.size, bool)
        first[1:] = pos[1:] != pos[:-1]
        bb = np.where(first & m[pos], b1[cs[pos]], b2[cs[pos]])
        beads.append(3 * bb)
        kk.append(np.full(bb.size, net.plane_k[p]))
        ss.append(np.full(bb.size, net.plane_slen[p]))
        nn.append(bb.size)
    A["bb_bs"] = np.ascontiguousarray(np.concatenate(beads) if beads else np.zeros(0), dtype=np.int32)
    A["bb_k"] = np.ascontiguousarray(np.concatenate(kk) if kk else np.zeros(0), dtype=np.float64)
    A["bb_slen"] = np.ascontiguousarray(np.concatenate(ss) if ss else np.zeros(0), dtype=np.float64)
    A["bd_nn"] = np.ascontiguousarray(nn, dtype=np.int32)
    A["planes"] = np.ascontiguousarray(net.planes.reshape(-1), dtype=np.float64)

    S = System()
    S.n_stretch = net.n_cyl
    S.st_bs, S.st_k, S.st_l0 = _p(A["st_bs"], _ip), _p(A["st_k"]), _p(A["st_l0"])
    S.n_bend = int(cur.size)
    S.bd_bs, S.bd_k, S.bd_t0 = _p(A["bd_bs"], _ip), _p(A["bd_k"]), _p(A["bd_t0"])
    S.n_linker = int(net.lk_cyl.shape[0])
    S.lk_bs, S.lk_k, S.lk_l0, S.lk_s1, S.lk_s2 = (_p(A["lk_bs"], _ip), _p(A["lk_k"]), _p(A["lk_l0"]),
                                                  _p(A["lk_s1"]), _p(A["lk_s2"]))
    S.n_motor = int(net.mt_cyl.shape[0])
    S.mt_bs, S.mt_k, S.mt_l0, S.mt_s1, S.mt_s2 = (_p(A["mt_bs"], _ip), _p(A["mt_k"]), _p(A["mt_l0"]),
                                                  _p(A["mt_s1"]), _p(A["mt_s2"]))
    S.n_exvol = int(pairs.shape[0])
    S.ev_bs, S.ev_k, S.ev_len = _p(A["ev_bs"], _ip), _p(A["ev_k"]), _p(A["ev_len"])
    S.n_planes = int(net.planes.shape[0])
    S.planes, S.bd_nn, S.bb_bs, S.bb_k, S.bb_slen = (_p(A["planes"]), _p(A["bd_nn"], _ip), _p(A["bb_bs"], _ip),
                                                     _p(A["bb_k"]), _p(A["bb_slen"]))
    return Vectorized(arrays=A, system=S, ndof=3 * net.n_beads, nbeads=net.n_beads, pairs=pairs,
                      bnd_cyl=bcyl, bnd_nn=bnn)


def energies(vec: Vectorized, coord: np.ndarray):
    """(total, per-FF array) with computeIndividualEnergies semantics."""
    x = np.ascontiguousarray(coord, dtype=np.float64).reshape(-1)
    per = np.zeros(6)
    tot = lib().orc_system_energies(C.byref(vec.system), _p(x), _p(per))
    return tot, per


def energy(vec: Vectorized, coord: np.ndarray) -> float:
    """Total with computeEnergy semantics (+inf when an FF fails)."""
    x = np.ascontiguousarray(coord, dtype=np.float64).reshape(-1)
    return lib().orc_system_energy(C.byref(vec.system), _p(x))


def forces(vec: Vectorized, coord: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(coord, dtype=np.float64).reshape(-1)
    f = np.zeros_like(x)
    lib().orc_system_forces(C.byref(vec.system), _p(x), _p(f), x.size, None, None)
    return f.reshape(-1, 3)


def stretch_forces(vec: Vectorized, coord: np.ndarray):
    """Per-linker and per-motor stretch force of the force routine
    (LinkerStretching::assignforcemags, LinkerStretching.cpp:117-123; motors alike)."""
    x = np.ascontiguousarray(coord, dtype=np.float64).reshape(-1)
    f = np.zeros_like(x)
    lk = np.zeros(max(1, vec.system.n_linker))
    mt = np.zeros(max(1, vec.system.n_motor))
    lib().orc_system_forces(C.byref(vec.system), _p(x), _p(f), x.size, _p(lk), _p(mt))
    return lk[:vec.system.n_linker], mt[:vec.system.n_motor]


def load_forces(net, coord=None, bnd=None, mon_size=(2.7,), n_mon=(40,)):
    """Boundary load forces on filament ends, (plus, minus) each [n_filaments, max n_mon]
    (ForceFieldManager.cpp:292-311, BoundaryCylinderRepulsion.cpp:122-192)."""
    coord = np.ascontiguousarray(net.coord if coord is None else coord, dtype=np.float64)
    if bnd is None:
        bnd = boundary_list(net, coord)
    bcyl, bnn = bnd
    ms = np.ascontiguousarray(mon_size, dtype=np.float64)
    nm = np.ascontiguousarray(n_mon, dtype=np.int32)
    stride = int(nm.max())
    nfil = int(net.n_filaments)
    plus = np.zeros((nfil, stride))
    minus = np.zeros((nfil, stride))
    fcs = np.ascontiguousarray(net.fil_cyl_start, dtype=np.int32)
    b1 = np.ascontiguousarray(net.cyl_b1, dtype=np.int32)
    b2 = np.ascontiguousarray(net.cyl_b2, dtype=np.int32)
    ty = np.ascontiguousarray(net.cyl_type, dtype=np.int32)
    planes = np.ascontiguousarray(net.planes, dtype=np.float64)
    pk = np.ascontiguousarray(net.plane_k, dtype=np.float64)
    ps = np.ascontiguousarray(net.plane_slen, dtype=np.float64)
    nn = np.ascontiguousarray(bnn, dtype=np.int32)
    lst = np.ascontiguousarray(bcyl, dtype=np.int32)
    lib().orc_boundary_load_forces(nfil, _p(fcs, _ip), _p(b1, _ip), _p(b2, _ip), _p(ty, _ip), _p(coord),
                                   planes.shape[0], _p(planes), _p(pk), _p(ps), _p(nn, _ip), _p(lst, _i32p),
                                   _p(ms), _p(nm, _ip), stride, _p(plus), _p(minus))
    return plus, minus


def force_scale(vec: Vectorized, coord: np.ndarray) -> np.ndarray:
    """Per component, the sum over interactions of |contribution|."""
    x = np.ascontiguousarray(coord, dtype=np.float64).reshape(-1)
    s = np.zeros_like(x)
    lib().orc_system_force_scale(C.byref(vec.system), _p(x), _p(s), x.size)
    return s.reshape(-1, 3)


class series_atan_mode:
    """Context manager: the excluded-volume formula uses the oracle's series
    arctangent (the one the GPU's FP64 kernel uses) instead of the C library's."""
    def __enter__(self):
        lib().orc_set_series_atan(1)
        return self

    def __exit__(self, *exc):
        lib().orc_set_series_atan(0)


class threads:
    """Context manager: the oracle's force fields and CG vector loops on `n`
    host threads (OpenMP).  Only for timing the CPU baseline: with more than
    one thread the sums round differently from the reference's serial order,
    so parity checks run with the default single thread."""
    def __init__(self, n: int):
        self.n = max(1, int(n))

    def __enter__(self):
        self.prev = lib().orc_get_threads()
        lib().orc_set_threads(self.n)
        return self

    def __exit__(self, *exc):
        lib().orc_set_threads(self.prev)


def cg_params(method=2, maxDist=1.0, lambdaMax=0.01, gradTol=1.0, energyRelTol=1e-9, energyCallLimit=0,
              forceCallLimit=10000, reportOnCallLimit=1, tryToRecover=1) -> CGParams:
    return CGParams(method, maxDist, lambdaMax, gradTol, energyRelTol, energyCallLimit, forceCallLimit,
                    reportOnCallLimit, tryToRecover)


def minimize(vec: Vectorized, coord: np.ndarray, params: CGParams | None = None):
    """Run the restated CGMethod::minimize; returns (coord, force, CGResult)."""
    params = params or cg_params()
    x = np.ascontiguousarray(coord, dtype=np.float64).reshape(-1).copy()
    f = np.zeros_like(x)
    res = CGResult()
    lib().orc_minimize(C.byref(vec.system), C.byref(params), _p(x), x.size, vec.nbeads, _p(f), C.byref(res))
    return x.reshape(-1, 3), f.reshape(-1, 3), res


def minimize_quadratic(w, o, x0, params: CGParams):
    w = np.ascontiguousarray(w, dtype=np.float64)
    o = np.ascontiguousarray(o, dtype=np.float64)
    x = np.ascontiguousarray(x0, dtype=np.float64).copy()
    f = np.zeros_like(x)
    res = CGResult()
    lib().orc_minimize_quadratic(x.size, _p(w), _p(o), C.byref(params), _p(x), _p(f), C.byref(res))
    return x, f, res
