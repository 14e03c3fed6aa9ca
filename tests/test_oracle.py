"""The oracle pinned against the reference's own unit cases and known answers.

The reference (MEDYAN 5.4.0) cannot be built here; its Catch2 cases for this
path are re-run on the oracle from the inputs in the reference's test sources,
read at test time by tests/golden/make_reference_fixtures.py:

* TestCylinderExclVolume.cpp:13-47, :49-101, :103-244
* TestBoundaryBeadRepulsion.cpp:13-96
* TestCGMethod.cpp:9-93

Filament stretching/bending, linkers, motors and the neighbor lists have no
reference test; they are pinned by analytic values, energy/force consistency
and brute force.
"""
import ctypes as C
import math

import numpy as np
import pytest

import oracle
from oracle.oracle import _dp, _ip, _p
from picgo_gb300.network import make_network, jitter


def _ef_consistent(energy_fn, force_fn, c0, move_mag, rel_eps, reps, need, seed=0):
    """Restatement of testEnergyForceConsistency (TestFFCommon.hpp:101-171)."""
    rng = np.random.default_rng(seed)
    passed = 0
    for _ in range(reps):
        dc = rng.normal(0.0, move_mag, size=c0.shape)
        de_actual = energy_fn(c0 + dc) - energy_fn(c0 - dc)
        de_expected = -2.0 * float(np.dot(dc, force_fn(c0)))
        if abs(de_actual - de_expected) <= min(abs(de_actual), abs(de_expected)) * rel_eps:
            passed += 1
    return passed >= need, passed


def _exvol_E(coord, bs, k, ln):
    L = oracle.lib()
    x = np.ascontiguousarray(coord, dtype=np.float64)
    bs = np.ascontiguousarray(bs, dtype=np.int32)
    k = np.ascontiguousarray(k, dtype=np.float64)
    ln = np.ascontiguousarray(ln, dtype=np.float64)
    return L.orc_exvol_energy(_p(x), k.size, _p(bs, _ip), _p(k), _p(ln))


def _exvol_F(coord, bs, k, ln):
    L = oracle.lib()
    x = np.ascontiguousarray(coord, dtype=np.float64)
    f = np.zeros_like(x)
    bs = np.ascontiguousarray(bs, dtype=np.int32)
    k = np.ascontiguousarray(k, dtype=np.float64)
    ln = np.ascontiguousarray(ln, dtype=np.float64)
    L.orc_exvol_forces(_p(x), _p(f), k.size, _p(bs, _ip), _p(k), _p(ln))
    return f


def _ceildiv(a, b):
    return -((-a) // b)


def monomer_energy(info, coord):
    """Monomer-based excluded volume (CylinderVolumeMon.hpp, energy()): sum over
    monomer pairs of kvol * seg1 * seg2 / d^4, monomers at (m - lo + 0.5)/numMon."""
    c = np.asarray(coord, dtype=np.float64)
    c1 = info["cyl1"]
    c2 = info["cyl2"]
    p11, p12 = c[c1["c1Index"]:c1["c1Index"] + 3], c[c1["c2Index"]:c1["c2Index"] + 3]
    p21, p22 = c[c2["c1Index"]:c2["c1Index"] + 3], c[c2["c2Index"]:c2["c2Index"] + 3]
    n1 = c1["monIndexPastPlus"] - c1["monIndexAtMinus"]
    n2 = c2["monIndexPastPlus"] - c2["monIndexAtMinus"]
    s1 = _ceildiv(c1["monIndexAtMinus"], c1["monInterval"]) * c1["monInterval"]
    s2 = _ceildiv(c2["monIndexAtMinus"], c2["monInterval"]) * c2["monInterval"]
    coeff = info["kvol"] * (c1["monInterval"] * c1["monEqLen"]) * (c2["monInterval"] * c2["monEqLen"])
    en = 0.0
    for m1 in range(s1, c1["monIndexPastPlus"], c1["monInterval"]):
        l1 = (m1 - c1["monIndexAtMinus"] + 0.5) / n1
        q1 = p11 + l1 * (p12 - p11)
        for m2 in range(s2, c2["monIndexPastPlus"], c2["monInterval"]):
            l2 = (m2 - c2["monIndexAtMinus"] + 0.5) / n2
            q2 = p21 + l2 * (p22 - p21)
            d2 = float(np.sum((q2 - q1) ** 2))
            en += coeff / (d2 * d2)
    return en


# --------------------------------------------------------------------------- reference cases

def test_exvol_scaling_reference_case(reference_cases):
    """One 120 nm pair vs the same pair split in sub-segments (TestCylinderExclVolume.cpp:13-47)."""
    s = reference_cases["exvol"]["scaling"]
    e0 = _exvol_E(s["coord"], s["beadSet0"], s["k0"], s["eqLength0"])
    e1 = _exvol_E(s["coord"], s["beadSet1"], s["k1"], s["eqLength1"])
    # Catch's Approx default: |a - b| <= 100 * FLT_EPSILON * |b|
    assert abs(e0 - e1) <= 100 * np.finfo(np.float32).eps * abs(e1)
    assert e0 > 0


def test_exvol_integral_vs_monomer_reference_case(reference_cases):
    """Integral formula vs monomer sum within 1e-2 (TestCylinderExclVolume.cpp:49-101)."""
    s = reference_cases["exvol"]["consistency"]
    ei = _exvol_E(s["coord"], s["beadSet"], [s["kvol"]], [s["eqLen"], s["eqLen"]])
    em = monomer_energy(s, s["coord"])
    assert abs(ei - em) <= min(abs(ei), abs(em)) * s["relEps"], (ei, em)


@pytest.mark.parametrize("case", [0, 1])
def test_exvol_energy_force_reference_case(reference_cases, case):
    """Energy/force consistency, 9 of 10 repetitions (TestCylinderExclVolume.cpp:103-244)."""
    ev = reference_cases["exvol"]
    ti = ev["energy_force"][case]
    c0 = np.array(ti["coord"], dtype=np.float64)
    ok, n = _ef_consistent(lambda c: _exvol_E(c, ti["beadSet"], ti["k"], ti["eqLength"]),
                           lambda c: _exvol_F(c, ti["beadSet"], ti["k"], ti["eqLength"]),
                           c0, ev["moveMag"], ev["relEps"], ev["repsTot"], ev["repsPassReq"], seed=case)
    assert ok, (ti["name"], n)


def test_boundary_energy_force_reference_case(reference_cases):
    """Plane at z = 3, beads on/above/below it (TestBoundaryBeadRepulsion.cpp:13-96)."""
    b = reference_cases["boundary"]
    n = np.array(b["normal"])
    p0 = np.array(b["point"])
    plane = np.array([n[0], n[1], n[2], -n[0] * p0[0] - n[1] * p0[1] - n[2] * p0[2]])
    L = oracle.lib()
    nn = np.array(b["numNeighbors"], np.int32)
    bs = np.array(b["beadSet"], np.int32)
    kr = np.array(b["kreps"])
    sl = np.array(b["slens"])

    def E(c):
        x = np.ascontiguousarray(c, dtype=np.float64)
        return L.orc_boundary_energy(_p(x), 1, _p(plane), _p(nn, _ip), _p(bs, _ip), _p(kr), _p(sl))

    def F(c):
        x = np.ascontiguousarray(c, dtype=np.float64)
        f = np.zeros_like(x)
        L.orc_boundary_forces(_p(x), _p(f), 1, _p(plane), _p(nn, _ip), _p(bs, _ip), _p(kr), _p(sl))
        return f

    ok, cnt = _ef_consistent(E, F, np.array(b["coords"]), b["moveMag"], b["relEps"], b["repsTot"], b["repsPassReq"])
    assert ok, cnt
    # distance is signed: the bead below the plane is at r = -10
    assert math.isclose(L.orc_plane_distance(_p(plane), _p(np.array([-1.0, -1e8, -7.0]))), -10.0)


@pytest.mark.parametrize("method", [0, 1, 2])
def test_cg_harmonic_reference_case(reference_cases, method):
    """10-D weighted bowl from three starts (TestCGMethod.cpp:9-93): success and all |F| < gradTol."""
    cg = reference_cases["cg"]
    p = cg["params"]
    prm = oracle.cg_params(method=method, maxDist=p["maxDist"], lambdaMax=p["lambdaMax"], gradTol=p["gradTol"],
                           energyRelTol=p["energyRelTol"], forceCallLimit=p["forceCallLimit"], tryToRecover=0)
    for x0 in cg["inits"]:
        x, f, res = oracle.minimize_quadratic(cg["weight"], cg["optCoord"], x0, prm)
        assert res.errorFlags == 0
        assert np.all(np.abs(f) <= p["gradTol"]), (method, np.abs(f).max())


# --------------------------------------------------------------------------- known answers

def _tiny_filament(coords, l0=108.0, k=100.0, kb=672.0):
    """A single filament network from explicit bead coordinates."""
    from picgo_gb300.network import Network, cube_planes
    coords = np.asarray(coords, dtype=np.float64)
    nb = coords.shape[0]
    nc = nb - 1
    planes, pk, ps = cube_planes(1e6)
    z = np.zeros
    return Network(box=1e6, coord=coords, fil_cyl_start=np.array([0, nc], np.int32),
                   cyl_b1=np.arange(nc, dtype=np.int32), cyl_b2=np.arange(1, nb, dtype=np.int32),
                   cyl_id=np.arange(nc, dtype=np.int64), cyl_fil=z(nc, np.int32), cyl_pos=np.arange(nc, dtype=np.int32),
                   cyl_type=z(nc, np.int32), cyl_l0=np.full(nc, l0), cyl_kstr=np.full(nc, k),
                   cyl_kbend=np.full(nc, kb), cyl_theta0=z(nc), cyl_kexvol=np.full(nc, 1e5),
                   lk_cyl=z((0, 2), np.int32), lk_pos=z((0, 2)), lk_k=z(0), lk_l0=z(0),
                   mt_cyl=z((0, 2), np.int32), mt_pos=z((0, 2)), mt_k=z(0), mt_l0=z(0),
                   planes=planes, plane_k=pk, plane_slen=ps)


def test_straight_filament_at_rest_has_zero_energy_and_force():
    c = np.array([[5e5 + 108.0 * i, 5e5, 5e5] for i in range(6)])
    net = _tiny_filament(c)
    v = oracle.vectorize(net)
    tot, per = oracle.energies(v, net.coord)
    assert per[0] == 0.0 and abs(per[1]) < 1e-12
    assert np.abs(oracle.forces(v, net.coord)).max() < 1e-9


def test_stretch_and_bend_analytic():
    L1, th = 120.0, 0.3
    c = np.array([[5e2, 5e2, 5e2], [5e2 + L1, 5e2, 5e2],
                  [5e2 + L1 + 108 * math.cos(th), 5e2 + 108 * math.sin(th), 5e2]])
    net = _tiny_filament(c)
    v = oracle.vectorize(net)
    _, per = oracle.energies(v, net.coord)
    assert math.isclose(per[0], 0.5 * 100.0 * (L1 - 108.0) ** 2, rel_tol=1e-12)
    assert math.isclose(per[1], 672.0 * (1 - math.cos(th)), rel_tol=1e-11)
    # net force and net torque of internal forces vanish
    f = oracle.forces(v, net.coord)
    assert np.abs(f.sum(0)).max() < 1e-9
    assert np.abs(np.cross(net.coord - net.coord.mean(0), f).sum(0)).max() < 1e-6


@pytest.mark.parametrize("ff", ["n_stretch", "n_bend", "n_linker", "n_motor", "n_planes"])
def test_forcefield_gradients_match_finite_differences(ff):
    """Each FF's force is minus the gradient of its energy (central differences)."""
    net = jitter(make_network("c1", n_motors=200), 0.5)
    v = oracle.vectorize(net)
    S2 = oracle.System.from_buffer_copy(v.system)
    for nm in ("n_stretch", "n_bend", "n_linker", "n_motor", "n_exvol", "n_planes"):
        if nm != ff:
            setattr(S2, nm, 0)
    vv = oracle.Vectorized(v.arrays, S2, v.ndof, v.nbeads, v.pairs, v.bnd_cyl, v.bnd_nn)
    f = oracle.forces(vv, net.coord)
    rng = np.random.default_rng(3)
    for _ in range(4):
        dc = rng.normal(0, 1e-5, net.coord.shape)
        de = oracle.energy(vv, net.coord + dc) - oracle.energy(vv, net.coord - dc)
        ex = -2 * float((dc * f).sum())
        assert abs(de - ex) <= 1e-6 * abs(ex) + 1e-12, (ff, de, ex)


def _fd_force(coord, bs, k, ln, h=1e-6):
    """-dE/dx by central differences of the oracle's pair energy."""
    g = np.zeros_like(coord)
    for i in range(coord.size):
        cp, cm = coord.copy(), coord.copy()
        cp[i] += h
        cm[i] -= h
        g[i] = -(_exvol_E(cp, bs, k, ln) - _exvol_E(cm, bs, k, ln)) / (2 * h)
    return g


def _moved_c2(c):
    """c with bead 2 moved 0.01 nm along unit((c2 - c1) x (c3 - c1)): the reference's
    movePointOutOfPlane for a pair judged coplanar (MathFunctions.h:1221-1273,
    CylinderExclVolRepulsion.cpp:610-626)."""
    p = c.reshape(4, 3)
    n = np.cross(p[1] - p[0], p[2] - p[0])
    q = p.copy()
    q[1] = p[1] + n / np.linalg.norm(n) * 0.01
    return q.reshape(-1)


def test_exvol_force_nudge_only_in_force_path():
    """A pair judged coplanar (|cos| < 0.1): its forces are those of the pair with c2
    moved 0.01 nm off the plane, its energy is that of the pair as given; a pair far
    from coplanar gets the plain gradient."""
    bs, k, ln = [0, 3, 6, 9], [1.0], [10.0, 10.0]
    # a 10 nm segment and a 2.8 nm one 1-3 nm from it, tilted by ~0.1 deg out of a common plane
    c = np.array([0, 0, 0, 10, 0, 0, 3, 3, 0.002, 5, 1, -0.002], dtype=np.float64)
    f = _exvol_F(c, bs, k, ln)
    # h = 3e-4 nm balances the truncation error against the round-off of the
    # energy, which is ill-conditioned this close to coplanar (FD error ~3e-7)
    g_here = _fd_force(c, bs, k, ln, 3e-4)
    g_moved = _fd_force(_moved_c2(c), bs, k, ln, 3e-4)
    scale = np.abs(f).max()
    assert np.abs(f - g_moved).max() <= 2e-6 * scale, (f, g_moved)
    assert np.abs(f - g_here).max() >= 1e-3 * scale, (f, g_here)    # the move is visible in the forces
    # the energy path does not move: E(c) differs from E(moved) and is smooth through c
    e = _exvol_E(c, bs, k, ln)
    assert abs(e - _exvol_E(_moved_c2(c), bs, k, ln)) >= 1e-6 * abs(e)
    dz = np.zeros_like(c)
    dz[5] = 1e-4
    mid = 0.5 * (_exvol_E(c + dz, bs, k, ln) + _exvol_E(c - dz, bs, k, ln))
    assert abs(mid - e) <= 1e-7 * abs(e)
    # far from coplanar (|cos| ~ 0.7): forces are the plain gradient
    c3 = np.array([0, 0, 0, 10, 0, 0, 3, 3, 2.0, 5, -3, -3.0], dtype=np.float64)
    f3 = _exvol_F(c3, bs, k, ln)
    g3 = _fd_force(c3, bs, k, ln, 3e-4)
    assert np.abs(f3 - g3).max() <= 1e-6 * np.abs(f3).max(), (f3, g3)


# --------------------------------------------------------------------------- neighbor lists

@pytest.mark.parametrize("cell", [27.0, 30.375, 60.0, 150.0])
def test_pair_list_is_cell_size_invariant(cell):
    net = make_network("c1", shuffle_ids=True)
    brute = oracle.cyl_pairs(net)
    assert brute.shape[0] > 50
    assert np.array_equal(oracle.cyl_pairs(net, binned=True, cell=cell), brute)
    assert np.array_equal(oracle.cyl_pairs_fast(net), brute)
    ids = net.cyl_id
    assert np.all(ids[brute[:, 0]] > ids[brute[:, 1]])


def test_boundary_list_matches_distance_rule():
    net = make_network("c1")
    cyl, nn = oracle.boundary_list(net)
    mid = 0.5 * net.coord[net.cyl_b1] + 0.5 * net.coord[net.cyl_b2]
    off = 0
    for p in range(6):
        a, b, c, d = net.planes[p]
        r = (a * mid[:, 0] + b * mid[:, 1] + c * mid[:, 2] + d) / math.sqrt(a * a + b * b + c * c)
        expect = np.nonzero(r < net.boundary_cutoff)[0]
        assert np.array_equal(cyl[off:off + nn[p]], expect)
        off += nn[p]


# --------------------------------------------------------------------------- minimizer on a network

def test_cg_reduces_energy_and_stops_on_a_criterion():
    net = make_network("c1", n_filaments=40, n_linkers=60, box=1200.0, n_cyl_per_filament=8)
    v = oracle.vectorize(net)
    x, f, res = oracle.minimize(v, net.coord, oracle.cg_params())
    assert res.status == 0 and res.errorFlags == 0
    assert res.energiesAfter[6] < res.energiesBefore[6]
    assert res.gradInfNorm < res.gradTol or res.energyRelChange < res.energyRelTol
    assert np.isclose(np.abs(f).max(), res.gradInfNorm)


def test_series_atan_accuracy():
    """The series arctangent shared with the GPU FP64 kernel is within 3 ulp of numpy's."""
    L = oracle.lib()
    xs = np.concatenate([np.linspace(-40, 40, 40001), np.logspace(-300, 300, 4001), -np.logspace(-8, 8, 401),
                         [0.0, 1.0, np.tan(np.pi / 12), 1e308]])
    ys = np.array([L.orc_series_atan(float(x)) for x in xs])
    ref = np.arctan(xs)
    ulp = np.abs(ys - ref) / np.spacing(np.abs(ref) + 1e-300)
    assert ulp.max() <= 3.0
    assert L.orc_series_atan(float("inf")) == np.pi / 2


def test_oracle_atan_sensitivity():
    """C-library vs series arctangent in the excluded-volume formula: the
    reference's own libm sensitivity (energies ~1e-14, forces up to ~1e-9 of
    the contribution scale on nearly coplanar pairs)."""
    net = make_network("c1")
    v = oracle.vectorize(net)
    e1, p1 = oracle.energies(v, net.coord)
    f1 = oracle.forces(v, net.coord)
    with oracle.series_atan_mode():
        e2, p2 = oracle.energies(v, net.coord)
        f2 = oracle.forces(v, net.coord)
    s = oracle.force_scale(v, net.coord)
    assert abs(p1[4] - p2[4]) <= 1e-12 * abs(p1[4])
    assert np.all(np.abs(f1 - f2) <= 1e-8 * s + 1e-9)


def test_force_scale_bounds_forces():
    net = jitter(make_network("c1", n_motors=50), 0.4)
    v = oracle.vectorize(net)
    f = oracle.forces(v, net.coord)
    s = oracle.force_scale(v, net.coord)
    assert np.all(np.abs(f) <= s * (1 + 1e-12) + 1e-12)


def test_threaded_oracle_agrees_with_serial():
    """The all-cores CPU baseline computes the same energies, forces and CG run
    as the serial oracle, up to summation order."""
    net = jitter(make_network("c1"), 0.5, seed=3)
    vec = oracle.vectorize(net)
    e1, p1 = oracle.energies(vec, net.coord)
    f1 = oracle.forces(vec, net.coord)
    x1, _, r1 = oracle.minimize(vec, net.coord, oracle.cg_params(energyCallLimit=60))
    with oracle.threads(4):
        e4, p4 = oracle.energies(vec, net.coord)
        f4 = oracle.forces(vec, net.coord)
        x4, _, r4 = oracle.minimize(vec, net.coord, oracle.cg_params(energyCallLimit=60))
    assert oracle.lib().orc_get_threads() == 1
    assert np.all(np.abs(p4 - p1) <= 1e-12 * np.abs(p1) + 1e-12)
    scale = oracle.force_scale(vec, net.coord)
    assert np.all(np.abs(f4 - f1) <= 1e-12 * scale + 1e-12)
    # same line-search branches for the first iterations: same call counts, nearly the same positions
    assert r4.numEnergyCall == r1.numEnergyCall and r4.numForceCall == r1.numForceCall
    assert np.abs(x4 - x1).max() < 1e-6
