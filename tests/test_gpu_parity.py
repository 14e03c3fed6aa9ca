"""GPU path against the oracle, through the C ABI.

Tolerances (FP64 path):
* energies: per force field |E_gpu - E_oracle| <= 1e-12 * |E_oracle| + 1e-10 pN nm;
* forces: per component |F_gpu - F_oracle| <= 1e-12 * S + 1e-9 pN, with S the
  sum over all interactions of |contribution| to that component;
* neighbor lists: the sorted cylinder-pair set is integer-exact.
The excluded-volume formula is compared with the oracle's series arctangent,
the arctangent the FP64 kernel uses (the C library's differs by an ulp, which
nearly coplanar pairs amplify; see test_oracle_atan_sensitivity).
Mixed precision: total energy within 1e-6 relative of the FP64 oracle, forces
within 2e-4 * (S + X) + 5e-3 pN, where X adds, for each excluded-volume pair
touching the bead, the largest force component of that pair (the pair's four
bead forces come from shared terms, so their error scales with the pair's
largest force), and 5 mpN is the single-precision resolution of a 108 nm bond
length times the 100 pN/nm stretching constant, with margin.
"""
import ctypes as C
import numpy as np
import pytest

import oracle
from picgo_gb300 import Engine, cg_params, jitter, make_network

pytestmark = pytest.mark.gpu

FF_FIELDS = ("n_stretch", "n_bend", "n_linker", "n_motor", "n_exvol", "n_planes")


def exvol_pair_scale(vec, coord):
    """Per component: sum over excluded-volume pairs touching the bead of the pair's largest force component."""
    L = oracle.lib()
    L.orc_exvol_pair_forces.restype = C.c_int
    L.orc_exvol_pair_forces.argtypes = [C.POINTER(C.c_double)] * 4 + [C.c_double] * 3 + [C.POINTER(C.c_double)]
    x = np.ascontiguousarray(coord, dtype=np.float64).reshape(-1)
    bs = vec.arrays["ev_bs"].reshape(-1, 4)
    k = vec.arrays["ev_k"]
    ln = vec.arrays["ev_len"].reshape(-1, 2)
    out = np.zeros(12)
    T = np.zeros_like(x)
    dp = C.POINTER(C.c_double)
    for i in range(bs.shape[0]):
        ptrs = [x[b:b + 3].ctypes.data_as(dp) for b in bs[i]]
        L.orc_exvol_pair_forces(*ptrs, float(k[i]), float(ln[i, 0]), float(ln[i, 1]), out.ctypes.data_as(dp))
        m = np.abs(out).max()
        for b in bs[i]:
            T[b:b + 3] += m
    return T.reshape(-1, 3)


def check_energies(per_gpu, per_orc, vec=None):
    """Per force field 1e-12 relative + 1e-10 pN nm.  With `vec`, the bending energy
    also gets 4 eps64 sum(k_bend): k (1 - cos theta) of a nearly straight triple is
    round-off of k, so a network of straight filaments has a bending energy made of
    cancellation only (1e-8 pN nm over a million triples), which no two
    implementations share to 1e-12 of itself."""
    for k in range(6):
        tol = 1e-12 * abs(per_orc[k]) + 1e-10
        if vec is not None and k == 1:
            tol += 4 * 2.2e-16 * float(np.sum(vec.arrays["bd_k"]))
        assert abs(per_gpu[k] - per_orc[k]) <= tol, (k, per_gpu[k], per_orc[k])


def check_forces(f_gpu, f_orc, scale):
    err = np.abs(f_gpu - f_orc)
    tol = 1e-12 * scale + 1e-9
    bad = err > tol
    assert not bad.any(), (err[bad][:5], tol[bad][:5], np.argwhere(bad)[:5])


NETS = {
    "c1": dict(config="c1"),
    "c1_shuffled": dict(config="c1", shuffle_beads=True, shuffle_ids=True, seed=11),
    "small_motors": dict(config="c1", n_filaments=60, n_cyl_per_filament=12, box=1500.0, n_linkers=80, n_motors=40,
                         seed=3),
}
# networks for the mixed-precision error checks only (the FP64 checks above cover the formulas)
MIXED_NETS = [("c1", 0.5), ("small_motors", 1.5), ("c5", 0.5)]


def _net(name, sigma=0.0):
    kw = dict(NETS[name]) if name in NETS else dict(config=name)
    cfg = kw.pop("config")
    net = make_network(cfg, **kw)
    return jitter(net, sigma, seed=7) if sigma else net


@pytest.mark.parametrize("name", list(NETS))
@pytest.mark.parametrize("sigma", [0.0, 0.7])
def test_fp64_energies_and_forces_match_oracle(name, sigma):
    net = _net(name, sigma)
    vec = oracle.vectorize(net)
    with Engine("fp64") as eng:
        eng.set_network(net)
        assert np.array_equal(eng.pairs(), vec.pairs)
        per, tot, en = eng.energies()
        f = eng.forces()
    with oracle.series_atan_mode():
        o_tot, o_per = oracle.energies(vec, net.coord)
        fo = oracle.forces(vec, net.coord)
        check_energies(per, o_per)
        assert abs(en - oracle.energy(vec, net.coord)) <= 1e-12 * abs(o_tot)
        check_forces(f, fo, oracle.force_scale(vec, net.coord))


@pytest.mark.parametrize("cell", [0.0, 27.0, 30.375, 55.0, 140.0])
def test_pair_list_is_exact_for_any_bin_edge(cell):
    net = _net("c1_shuffled", 2.0)
    ref = oracle.cyl_pairs(net)
    with Engine("fp64") as eng:
        eng.set_network(net)
        info = eng.rebuild(cell)
        assert info["n_exvol_pairs"] == ref.shape[0]
        assert np.array_equal(eng.pairs(), ref)


def test_coordinates_round_trip_in_caller_order():
    net = _net("c1_shuffled")
    with Engine("fp64") as eng:
        eng.set_network(net)
        assert np.array_equal(eng.coords(), net.coord)
        x2 = net.coord + 0.25
        eng.set_coords(x2)
        assert np.array_equal(eng.coords(), x2)


def test_fp64_minimizer_tracks_oracle_for_first_iterations():
    """Same decisions in the first CG iterations: coordinates agree to round-off."""
    net = _net("small_motors", 0.3)
    vec = oracle.vectorize(net)
    prm = dict(energy_call_limit=40)
    x_o, f_o, r_o = oracle.minimize(vec, net.coord, oracle.cg_params(energyCallLimit=40))
    with Engine("fp64") as eng:
        eng.set_network(net)
        r = eng.minimize(cg_params(**prm))[0]
        x = eng.coords()
    assert r["num_iter"] == r_o.numIter
    assert r["num_force_call"] == r_o.numForceCall
    assert r["num_energy_call"] == r_o.numEnergyCall
    assert np.abs(x - x_o).max() <= 1e-9 * (1 + np.abs(x_o).max())
    assert abs(r["energies_after"][6] - r_o.energiesAfter[6]) <= 1e-10 * abs(r_o.energiesAfter[6])


def test_fp64_minimizer_converges_like_oracle():
    net = _net("small_motors")
    vec = oracle.vectorize(net)
    x_o, f_o, r_o = oracle.minimize(vec, net.coord)
    with Engine("fp64") as eng:
        eng.set_network(net)
        r = eng.minimize(cg_params())[0]
        f = eng.last_forces()
    assert r["status"] == 0 and r["error_flags"] == 0
    assert r["grad_inf_norm"] < r["grad_tol"] or r["energy_rel_change"] < r["energy_rel_tol"]
    assert np.isclose(np.abs(f).max(), r["grad_inf_norm"])
    # both descend from the same start to a nearby stationary state
    assert r["energies_after"][6] < r["energies_before"][6]
    assert abs(r["energies_after"][6] - r_o.energiesAfter[6]) <= 2e-2 * abs(r_o.energiesAfter[6])


@pytest.mark.parametrize("name,sigma", MIXED_NETS)
def test_mixed_energy_error_against_fp64(name, sigma):
    net = _net(name, sigma)
    vec = oracle.vectorize(net)
    o_tot, o_per = oracle.energies(vec, net.coord)
    fo = oracle.forces(vec, net.coord)
    with Engine("mixed") as eng:
        eng.set_network(net)
        assert np.array_equal(eng.pairs(), vec.pairs)
        assert np.abs(eng.coords() - net.coord).max() <= 1e-11 * np.abs(net.coord).max()
        per, tot, _ = eng.energies()
        f = eng.forces()
    assert abs(tot - o_tot) <= 1e-6 * abs(o_tot), (tot, o_tot)
    S = oracle.force_scale(vec, net.coord)
    X = exvol_pair_scale(vec, net.coord)
    err = np.abs(f - fo)
    ratio = err / (2e-4 * (S + X) + 5e-3)
    i = np.unravel_index(np.argmax(ratio), ratio.shape)
    assert ratio.max() <= 1.0, dict(worst=i, ratio=ratio[i], err=err[i], S=S[i], X=X[i], f=f[i], fo=fo[i])


def test_mixed_minimizer_reaches_tolerance():
    net = _net("small_motors")
    with Engine("mixed") as eng:
        eng.set_network(net)
        r = eng.minimize(cg_params(energy_rel_tol=0.0, force_call_limit=200000))[0]
        f = eng.last_forces()
    assert r["status"] == 0
    assert r["grad_inf_norm"] < 1.0
    assert np.abs(f).max() < 1.0
    assert r["energies_after"][6] < r["energies_before"][6]
