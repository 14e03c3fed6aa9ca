"""Seeded synthetic actin networks for the mechanical-equilibration path.

A network is what MEDYAN's ``MController::run`` hands to the minimizer after
``serializeDof`` (medyan-5.4.0/src/Structure/DofSerializer.hpp:64-187) and the
force fields' ``vectorize`` calls: bead coordinates plus the topology and
constants of filaments, cylinders, linkers, motors and boundary planes.

The generator follows MEDYAN's own recipes where they exist:

* filaments are straight rods from a uniform start point along an isotropic
  direction, rejected unless both ends sit at least ``BoundaryCutoff / 4``
  inside the boundary (medyan-5.4.0/src/FilamentInitializer.cpp:105-135);
  beads are spaced at the cylinder rest length, so every cylinder starts at
  rest;
* cylinder constants follow ``MCylinder::setEqLength``
  (medyan-5.4.0/src/Structure/MCylinder.cpp:35-43): k_str = K_str * size/l0,
  k_bend = K_bend * size/l0;
* linkers and motors join two cylinders of different filaments whose
  midpoints are closer than a binding range, at relative positions drawn
  uniformly on [0, 1]; linker rest lengths are the distance at creation
  (medyan-5.4.0/src/Structure/Linker.cpp:71), motor rest lengths are drawn
  uniformly from a range;
* the boundary is MEDYAN's cube: six planes 25 nm inside the box with inward
  normals (medyan-5.4.0/src/Structure/BoundaryImpl.cpp:25-53).

Everything is numpy and seeded; the same seed gives the same network on any
machine with the same numpy.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

# Workloads with the sizes and constants named by the benchmark configuration.
CONFIGS = {
    # 200 actin filaments x 20 cylinders in a 2 um box, 500 linkers.
    "c1": dict(n_filaments=200, n_cyl_per_filament=20, box=2000.0,
               n_linkers=500, linker_k=8.0, n_motors=0),
    # 20,000 filaments x 50 cylinders in a 10 um box, 50,000 linkers and
    # 5,000 motors with rest lengths drawn from 175-225 nm.
    "c2": dict(n_filaments=20000, n_cyl_per_filament=50, box=10000.0,
               n_linkers=50000, linker_k=8.0, n_motors=5000, motor_k=2.5,
               motor_l0=(175.0, 225.0)),
    # 2,000 filaments x 30 cylinders with 5,000 linkers whose stiffness and
    # rest length are the adjoint parameters.
    "c5": dict(n_filaments=2000, n_cyl_per_filament=30, box=None,
               n_linkers=5000, linker_k=(4.0, 12.0), linker_l0=(20.0, 40.0),
               n_motors=0, linker_tension=True),
}

CYLINDER_SIZE = 108.0          # nm, full actin cylinder
F_STRETCHING_K = 100.0         # pN/nm
F_BENDING_K = 672.0            # pN nm
F_BENDING_THETA = 0.0          # rad
VOLUME_K = 1.0e5               # excluded-volume constant
VOLUME_CUTOFF = 27.0           # nm, midpoint cutoff of the cylinder pair list
BOUNDARY_K = 41.0              # pN nm
BOUNDARY_SCREEN = 2.7          # nm
BOUNDARY_CUTOFF = 100.0        # nm
BOUNDARY_INSET = 25.0          # nm, planes sit this far inside the box
LINK_RANGE = 40.0              # nm, midpoint distance of linkable cylinder pairs
DENSITY_C1 = 4000 / 2000.0 ** 3  # cylinders per nm^3 at the 2 um / 4000 cylinder point


@dataclasses.dataclass
class Network:
    """Bead coordinates and the topology/constants of one network.

    Index conventions follow MEDYAN's database order: ``coord`` is the
    serialized DOF vector reshaped (n_beads, 3); cylinders are listed filament
    by filament from minus to plus end; linkers/motors refer to cylinders by
    index into the cylinder arrays.
    """
    box: float
    coord: np.ndarray             # (n_beads, 3) float64
    fil_cyl_start: np.ndarray     # (n_filaments + 1,) int32
    cyl_b1: np.ndarray            # (n_cyl,) int32 first (minus-side) bead
    cyl_b2: np.ndarray            # (n_cyl,) int32 second (plus-side) bead
    cyl_id: np.ndarray            # (n_cyl,) int64 unique cylinder ID
    cyl_fil: np.ndarray           # (n_cyl,) int32 filament ID
    cyl_pos: np.ndarray           # (n_cyl,) int32 position on filament
    cyl_type: np.ndarray          # (n_cyl,) int32 filament type
    cyl_l0: np.ndarray            # (n_cyl,) float64 equilibrium length
    cyl_kstr: np.ndarray          # (n_cyl,) float64
    cyl_kbend: np.ndarray         # (n_cyl,) float64
    cyl_theta0: np.ndarray        # (n_cyl,) float64
    cyl_kexvol: np.ndarray        # (n_cyl,) float64
    lk_cyl: np.ndarray            # (n_linkers, 2) int32
    lk_pos: np.ndarray            # (n_linkers, 2) float64
    lk_k: np.ndarray              # (n_linkers,) float64
    lk_l0: np.ndarray             # (n_linkers,) float64
    mt_cyl: np.ndarray            # (n_motors, 2) int32
    mt_pos: np.ndarray            # (n_motors, 2) float64
    mt_k: np.ndarray              # (n_motors,) float64
    mt_l0: np.ndarray             # (n_motors,) float64
    planes: np.ndarray            # (n_planes, 4) float64: a, b, c, d of a x + b y + c z + d = 0
    plane_k: np.ndarray           # (n_planes,) float64 repulsion constant
    plane_slen: np.ndarray        # (n_planes,) float64 screening length
    boundary_cutoff: float = BOUNDARY_CUTOFF
    exvol_cutoff: float = VOLUME_CUTOFF
    seed: int = 0
    stats: dict = dataclasses.field(default_factory=dict)

    @property
    def n_beads(self) -> int:
        return int(self.coord.shape[0])

    @property
    def n_cyl(self) -> int:
        return int(self.cyl_b1.shape[0])

    @property
    def n_filaments(self) -> int:
        return int(self.fil_cyl_start.shape[0] - 1)

    def copy(self) -> "Network":
        return dataclasses.replace(
            self, **{f.name: (getattr(self, f.name).copy()
                              if isinstance(getattr(self, f.name), np.ndarray) else getattr(self, f.name))
                     for f in dataclasses.fields(self)})


def cube_planes(box: float, k: float = BOUNDARY_K, slen: float = BOUNDARY_SCREEN):
    """MEDYAN's cubic boundary: x, y, z planes at 25 nm and box - 25 nm, normals inward.

    The plane constant is d = -(n . p0) for a point p0 on the plane
    (medyan-5.4.0/src/Structure/BoundaryElementImpl.h:40-47).
    """
    lo, hi = BOUNDARY_INSET, box - BOUNDARY_INSET
    planes = []
    for axis in range(3):
        for pos, sgn in ((lo, 1.0), (hi, -1.0)):
            n = [0.0, 0.0, 0.0]
            n[axis] = sgn
            p0 = [hi / 2, hi / 2, hi / 2]
            p0[axis] = pos
            d = -n[0] * p0[0] - n[1] * p0[1] - n[2] * p0[2]
            planes.append(n + [d])
    planes = np.array(planes, dtype=np.float64)
    return planes, np.full(6, k), np.full(6, slen)


def _place_filaments(rng, n_fil, length, box, max_tries):
    """Straight rods accepted when both ends are >= cutoff/4 inside the planes."""
    lo = BOUNDARY_INSET + BOUNDARY_CUTOFF / 4.0
    hi = box - BOUNDARY_INSET - BOUNDARY_CUTOFF / 4.0
    starts = np.empty((n_fil, 3))
    dirs = np.empty((n_fil, 3))
    got = 0
    tries = 0
    batch = max(1024, 4 * n_fil)
    while got < n_fil:
        if tries >= max_tries:
            raise RuntimeError(f"filament placement gave up after {tries} tries "
                               f"({got}/{n_fil} placed; rod {length} nm in a {box} nm box)")
        p = rng.uniform(0.0, box, size=(batch, 3))
        phi = rng.uniform(0.0, 2.0 * math.pi, size=batch)
        cz = rng.uniform(-1.0, 1.0, size=batch)
        sz = np.sqrt(1.0 - cz * cz)
        u = np.stack([sz * np.cos(phi), sz * np.sin(phi), cz], axis=1)
        q = p + length * u
        ok = np.all((p >= lo) & (p <= hi) & (q >= lo) & (q <= hi), axis=1)
        tries += batch
        idx = np.nonzero(ok)[0][: n_fil - got]
        starts[got:got + idx.size] = p[idx]
        dirs[got:got + idx.size] = u[idx]
        got += idx.size
    return starts, dirs, n_fil / tries


def _place_chains(rng, n_fil, n_cyl, box, bend_sigma=0.35):
    """Filaments as confined persistent random walks of n_cyl 108 nm steps: the
    direction of each step is the previous one plus N(0, bend_sigma) per
    component, renormalised; a step that would leave the box (inset like the
    straight rods) has the offending direction components reflected.  Used
    where straight rods cannot fit, e.g. 50-cylinder filaments (5.4 um) in
    boxes shrunk to keep the 2 um / 4000-cylinder density."""
    lo = BOUNDARY_INSET + BOUNDARY_CUTOFF / 4.0
    hi = box - BOUNDARY_INSET - BOUNDARY_CUTOFF / 4.0
    if hi - lo < 3 * CYLINDER_SIZE:
        raise ValueError(f"box {box} nm too small for chains of {CYLINDER_SIZE} nm cylinders")
    pts = np.empty((n_fil, n_cyl + 1, 3))
    pts[:, 0] = rng.uniform(lo, hi, size=(n_fil, 3))
    phi = rng.uniform(0.0, 2.0 * math.pi, size=n_fil)
    cz = rng.uniform(-1.0, 1.0, size=n_fil)
    sz = np.sqrt(1.0 - cz * cz)
    u = np.stack([sz * np.cos(phi), sz * np.sin(phi), cz], axis=1)
    for j in range(1, n_cyl + 1):
        if j > 1:
            u = u + rng.normal(0.0, bend_sigma, size=u.shape)
            u /= np.linalg.norm(u, axis=1)[:, None]
        q = pts[:, j - 1] + CYLINDER_SIZE * u
        out = (q < lo) | (q > hi)
        u = np.where(out, -u, u)
        pts[:, j] = pts[:, j - 1] + CYLINDER_SIZE * u
    return pts.reshape(-1, 3)


def _link_pairs(rng, mid, cyl_fil, n_need, r):
    """Cylinder pairs of different filaments with midpoint distance < r."""
    from scipy.spatial import cKDTree
    if n_need == 0:
        return np.zeros((0, 2), np.int32), 0
    tree = cKDTree(mid)
    pairs = tree.query_pairs(r, output_type="ndarray")
    pairs = pairs[cyl_fil[pairs[:, 0]] != cyl_fil[pairs[:, 1]]]
    n_cand = int(pairs.shape[0])
    if n_cand == 0:
        raise RuntimeError("no linkable cylinder pairs")
    # Distinct pairs when there are enough; otherwise several linkers share a
    # cylinder pair at different binding positions, as MEDYAN allows.
    replace = n_cand < n_need
    pick = rng.choice(n_cand, size=n_need, replace=replace)
    sel = pairs[pick]
    # random orientation of each pair
    flip = rng.random(n_need) < 0.5
    sel[flip] = sel[flip][:, ::-1]
    return sel.astype(np.int32), n_cand


def make_network(config: str | dict = "c1", seed: int | None = None, *, n_filaments=None,
                 n_cyl_per_filament=None, box=None, n_linkers=None, n_motors=None,
                 shuffle_beads: bool = False, shuffle_ids: bool = False,
                 max_tries: int = 200_000_000) -> Network:
    """Build a seeded network.

    ``config`` names one of :data:`CONFIGS` or is a dict of the same keys;
    keyword arguments override it.  ``shuffle_beads`` permutes the bead
    storage order and ``shuffle_ids`` permutes cylinder IDs, to exercise
    callers whose database order is not filament order.
    """
    cfg = dict(CONFIGS[config]) if isinstance(config, str) else dict(config)
    for key, val in (("n_filaments", n_filaments), ("n_cyl_per_filament", n_cyl_per_filament),
                     ("box", box), ("n_linkers", n_linkers), ("n_motors", n_motors)):
        if val is not None:
            cfg[key] = val
    cfg.setdefault("n_motors", 0)
    nf = int(cfg["n_filaments"])
    nc = int(cfg["n_cyl_per_filament"])
    if cfg.get("box") is None:
        # hold the 2 um / 4000-cylinder density
        cfg["box"] = (nf * nc / DENSITY_C1) ** (1.0 / 3.0)
    L = float(cfg["box"])
    if seed is None:
        seed = 20261203
    rng = np.random.default_rng(seed)

    length = nc * CYLINDER_SIZE
    if cfg.get("shape", "straight") == "chain":
        coord = _place_chains(rng, nf, nc, L)
        acc = 1.0
    else:
        starts, dirs, acc = _place_filaments(rng, nf, length, L, max_tries)
        k = np.arange(nc + 1, dtype=np.float64) * CYLINDER_SIZE
        coord = (starts[:, None, :] + k[None, :, None] * dirs[:, None, :]).reshape(-1, 3)
    nb = coord.shape[0]
    bead_of = np.arange(nb, dtype=np.int64).reshape(nf, nc + 1)
    b1 = bead_of[:, :-1].reshape(-1)
    b2 = bead_of[:, 1:].reshape(-1)
    ncyl = nf * nc
    cyl_fil = np.repeat(np.arange(nf, dtype=np.int32), nc)
    cyl_pos = np.tile(np.arange(nc, dtype=np.int32), nf)
    cyl_id = np.arange(ncyl, dtype=np.int64)
    if shuffle_ids:
        cyl_id = rng.permutation(ncyl).astype(np.int64) * 3 + 7
    if shuffle_beads:
        perm = rng.permutation(nb)          # new index of old bead
        new_coord = np.empty_like(coord)
        new_coord[perm] = coord
        coord = new_coord
        b1 = perm[b1]
        b2 = perm[b2]

    l0 = np.full(ncyl, CYLINDER_SIZE)
    frac = CYLINDER_SIZE / l0
    mid = 0.5 * (coord[b1] + coord[b2])

    def bonds(n, kval, l0spec, kind):
        if n == 0:
            z = np.zeros
            return z((0, 2), np.int32), z((0, 2)), z(0), z(0), 0
        cyl, n_cand = _link_pairs(rng, mid, cyl_fil, n, LINK_RANGE)
        pos = rng.uniform(0.0, 1.0, size=(n, 2))
        kk = (rng.uniform(kval[0], kval[1], size=n) if isinstance(kval, tuple)
              else np.full(n, float(kval)))
        c1a, c1b = coord[b1[cyl[:, 0]]], coord[b2[cyl[:, 0]]]
        c2a, c2b = coord[b1[cyl[:, 1]]], coord[b2[cyl[:, 1]]]

        def attach_dist(ps):
            p1 = c1a * (1 - ps[:, :1]) + ps[:, :1] * c1b
            p2 = c2a * (1 - ps[:, 1:]) + ps[:, 1:] * c2b
            return np.sqrt(np.sum((p2 - p1) ** 2, axis=1))

        if l0spec is None:   # rest length = distance at creation
            ll = attach_dist(pos)
        else:
            ll = rng.uniform(l0spec[0], l0spec[1], size=n)
            if kind == "linker" and cfg.get("linker_tension"):
                # attachment points redrawn until the linker starts stretched
                # (distance >= rest length); a compressed harmonic linker
                # has negative transverse stiffness and makes the energy
                # non-convex where it sits.  Linkers still compressed after
                # 64 draws start at rest (rest length = distance).
                for _ in range(64):
                    bad = attach_dist(pos) < ll
                    if not bad.any():
                        break
                    pos[bad] = rng.uniform(0.0, 1.0, size=(int(bad.sum()), 2))
                ll = np.minimum(ll, attach_dist(pos))
        return cyl, pos, kk, ll, n_cand

    lk_cyl, lk_pos, lk_k, lk_l0, lk_cand = bonds(int(cfg["n_linkers"]), cfg.get("linker_k", 8.0),
                                                  cfg.get("linker_l0"), "linker")
    mt_cyl, mt_pos, mt_k, mt_l0, mt_cand = bonds(int(cfg["n_motors"]), cfg.get("motor_k", 2.5),
                                                  cfg.get("motor_l0", (175.0, 225.0)), "motor")
    planes, pk, ps = cube_planes(L)
    net = Network(
        box=L, coord=np.ascontiguousarray(coord, dtype=np.float64),
        fil_cyl_start=(np.arange(nf + 1, dtype=np.int32) * nc),
        cyl_b1=b1.astype(np.int32), cyl_b2=b2.astype(np.int32), cyl_id=cyl_id,
        cyl_fil=cyl_fil, cyl_pos=cyl_pos, cyl_type=np.zeros(ncyl, np.int32),
        cyl_l0=l0, cyl_kstr=F_STRETCHING_K * frac, cyl_kbend=F_BENDING_K * frac,
        cyl_theta0=np.full(ncyl, F_BENDING_THETA), cyl_kexvol=np.full(ncyl, VOLUME_K),
        lk_cyl=lk_cyl, lk_pos=lk_pos, lk_k=lk_k, lk_l0=lk_l0,
        mt_cyl=mt_cyl, mt_pos=mt_pos, mt_k=mt_k, mt_l0=mt_l0,
        planes=planes, plane_k=pk, plane_slen=ps, seed=int(seed),
        stats=dict(placement_acceptance=acc, linker_candidates=lk_cand, motor_candidates=mt_cand),
    )
    return net


def jitter(net: Network, sigma: float, seed: int = 1) -> Network:
    """Copy of ``net`` with every bead displaced by N(0, sigma) per component."""
    out = net.copy()
    rng = np.random.default_rng(seed)
    out.coord = out.coord + rng.normal(0.0, sigma, size=out.coord.shape)
    return out


def make_ensemble(n_replicas: int = 512, seed: int = 20261203 + 4, fil_range=(50, 5000), cyl_range=(20, 50),
                  linkers_per_cylinder: float = 500 / 4000) -> list:
    """Independent replica networks of uneven size: filament counts log-uniform
    on ``fil_range``, cylinders per filament uniform on ``cyl_range``, box side
    scaled to hold the 2 um / 4000-cylinder density, linkers at the 200 x 20
    network's ratio; filaments as confined chains (:func:`_place_chains`),
    since straight rods do not fit the shrunk boxes."""
    rng = np.random.default_rng(seed)
    nfs = np.rint(np.exp(rng.uniform(math.log(fil_range[0]), math.log(fil_range[1]), size=n_replicas))).astype(int)
    ncs = rng.integers(cyl_range[0], cyl_range[1] + 1, size=n_replicas)
    nets = []
    for i in range(n_replicas):
        ncyl = int(nfs[i] * ncs[i])
        cfg = dict(n_filaments=int(nfs[i]), n_cyl_per_filament=int(ncs[i]), box=None,
                   n_linkers=int(round(linkers_per_cylinder * ncyl)), linker_k=8.0, n_motors=0, shape="chain")
        nets.append(make_network(cfg, seed=seed * 1000 + i))
    return nets
