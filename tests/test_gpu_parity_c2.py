"""GPU path against the oracle on the 1M-cylinder network (20,000 filaments x 50
cylinders, 50,000 linkers, 5,000 motors, 10 um box, seed 20261205), through
the C ABI, at the seeded start and after 200 mixed-precision CG iterations.

Tolerances:
* neighbor lists: the cylinder pair list and the boundary-cylinder list are
  integer-exact;
* FP64 against the oracle with the series arctangent the FP64 kernel uses:
  per force field |dE| <= 1e-12 |E| + 1e-10 pN nm (bending also + 4 eps64 sum k_bend,
  the round-off of straight triples), forces |dF| <= 1e-12 S + 1e-9 pN
  per component (S = sum of |contributions| to that component);
* FP64 against the oracle with the C library's arctangent (the reference's
  arithmetic): the same energy bound; forces |dF| <= 1e-7 S + 1e-9 pN.  Nearly
  coplanar excluded-volume pairs amplify a one-ulp arctangent difference by
  ~1e6-1e8 (measured: up to 2.3e-8 S on this network's start);
* mixed precision: total energy within 1e-6 relative of the oracle, forces
  within 2e-4 (S + X) + 5e-3 pN (X as in test_gpu_parity).
"""
import numpy as np
import pytest

import oracle
from picgo_gb300 import Engine, cg_params, jitter, make_network

from test_gpu_parity import check_energies, check_forces, exvol_pair_scale

pytestmark = pytest.mark.gpu

SEED = 20261205


@pytest.fixture(scope="module")
def c2_start():
    return make_network("c2", seed=SEED)


@pytest.fixture(scope="module")
def c2_relaxed(c2_start):
    """The network after 200 mixed CG iterations from the seeded start."""
    with Engine("mixed") as eng:
        eng.set_network(c2_start)
        r = eng.minimize(cg_params(energy_rel_tol=0.0, energy_call_limit=540))[0]
        x = eng.coords()
    assert r["num_iter"] >= 150
    net = c2_start.copy()
    net.coord = x
    return net


@pytest.fixture(scope="module", params=["start", "relaxed"])
def c2(request, c2_start, c2_relaxed):
    net = c2_start if request.param == "start" else c2_relaxed
    return net, oracle.vectorize(net)


def boundary_pairs(net, coord=None):
    """The oracle's BoundaryCylinderNL as (plane, cylinder) rows, plane by plane."""
    cyl, nn = oracle.boundary_list(net, coord)
    return np.stack([np.repeat(np.arange(len(nn)), nn), cyl], axis=1).astype(np.int32)


def test_c2_pair_list_is_exact(c2):
    net, vec = c2
    ref = oracle.cyl_pairs_fast(net)
    assert np.array_equal(ref, vec.pairs)
    assert ref.shape[0] > 20000
    with Engine("fp64") as eng:
        eng.set_network(net)
        assert np.array_equal(eng.pairs(), ref)


def test_c2_boundary_list_is_exact(c2):
    net, vec = c2
    ref = boundary_pairs(net)
    with Engine("fp64") as eng:
        eng.set_network(net)
        info = eng.rebuild()
        got = eng.boundary_list()
    assert info["n_boundary_cyl"] == ref.shape[0]
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("sigma", [0.0, 2.0])
def test_c1_boundary_list_is_exact(sigma):
    net = make_network("c1")
    net = jitter(net, sigma, seed=5) if sigma else net
    with Engine("mixed") as eng:
        eng.set_network(net)
        got = eng.boundary_list()
    assert np.array_equal(got, boundary_pairs(net))


def test_c2_fp64_matches_oracle_series_atan(c2):
    net, vec = c2
    with Engine("fp64") as eng:
        eng.set_network(net)
        per, tot, en = eng.energies()
        f = eng.forces()
    with oracle.series_atan_mode():
        o_tot, o_per = oracle.energies(vec, net.coord)
        fo = oracle.forces(vec, net.coord)
        check_energies(per, o_per, vec)
        assert abs(tot - o_tot) <= 1e-12 * abs(o_tot)
        check_forces(f, fo, oracle.force_scale(vec, net.coord))


def test_c2_fp64_matches_oracle_libm_atan(c2):
    """The reference's own arithmetic (C library arctangent): stated looser force bound."""
    net, vec = c2
    with Engine("fp64") as eng:
        eng.set_network(net)
        per, tot, en = eng.energies()
        f = eng.forces()
    o_tot, o_per = oracle.energies(vec, net.coord)
    fo = oracle.forces(vec, net.coord)
    check_energies(per, o_per, vec)
    S = oracle.force_scale(vec, net.coord)
    err = np.abs(f - fo)
    tol = 1e-7 * S + 1e-9
    assert (err <= tol).all(), (err / (S + 1e-300)).max()


def test_c2_mixed_per_evaluation_error(c2):
    net, vec = c2
    o_tot, o_per = oracle.energies(vec, net.coord)
    fo = oracle.forces(vec, net.coord)
    with Engine("mixed") as eng:
        eng.set_network(net)
        assert np.array_equal(eng.pairs(), vec.pairs)
        per, tot, _ = eng.energies()
        f = eng.forces()
    assert abs(tot - o_tot) <= 1e-6 * abs(o_tot), (tot, o_tot)
    S = oracle.force_scale(vec, net.coord)
    X = exvol_pair_scale(vec, net.coord)
    ratio = np.abs(f - fo) / (2e-4 * (S + X) + 5e-3)
    assert ratio.max() <= 1.0, ratio.max()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_load_forces_match_oracle(precision, c2_relaxed):
    """Boundary load forces on filament ends after a minimization, at the engine's own
    coordinates with the lists of the last rebuild."""
    for net in (jitter(make_network("c1"), 1.0, seed=9), c2_relaxed):
        with Engine(precision) as eng:
            eng.set_network(net)
            eng.minimize(cg_params(energy_rel_tol=0.0, energy_call_limit=60))
            x = eng.coords()
            plus, minus = eng.load_forces((2.7,), (40,))
        # the lists are those of the rebuild at the network's coordinates
        bnd = oracle.boundary_list(net)
        po, mo = oracle.load_forces(net, x, bnd, (2.7,), (40,))
        assert np.count_nonzero(po) > 0 and np.count_nonzero(mo) > 0
        for got, ref in ((plus, po), (minus, mo)):
            assert np.all(np.abs(got - ref) <= 1e-12 * np.abs(ref) + 1e-12), np.abs(got - ref).max()


def test_load_forces_per_filament_type():
    """Two filament types with their own monomer sizes and counts; entries past a
    type's monomer count stay zero."""
    net = jitter(make_network("c1", n_filaments=60, n_cyl_per_filament=8, box=1200.0, n_linkers=40), 0.5, seed=2)
    fil_of = np.repeat(np.arange(net.n_filaments), np.diff(net.fil_cyl_start))
    net.cyl_type = (fil_of % 2).astype(np.int32)
    with Engine("fp64") as eng:
        eng.set_network(net)
        plus, minus = eng.load_forces((2.7, 4.0), (40, 27))
    po, mo = oracle.load_forces(net, net.coord, None, (2.7, 4.0), (40, 27))
    assert np.all(plus[1::2, 27:] == 0) and np.all(minus[1::2, 27:] == 0)
    for got, ref in ((plus, po), (minus, mo)):
        assert np.all(np.abs(got - ref) <= 1e-12 * np.abs(ref) + 1e-12)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_stretch_forces_match_oracle(precision):
    """LinkerStretching::assignforcemags (and motors) after a force evaluation."""
    net = jitter(make_network("c1", n_filaments=60, n_cyl_per_filament=12, box=1500.0, n_linkers=80, n_motors=40,
                              seed=3), 0.8, seed=4)
    vec = oracle.vectorize(net)
    lk_o, mt_o = oracle.stretch_forces(vec, net.coord)
    with Engine(precision) as eng:
        eng.set_network(net)
        eng.forces()
        lk, mt = eng.stretch_forces()
    tol = 1e-12 if precision == "fp64" else 2e-4
    for got, ref in ((lk, lk_o), (mt, mt_o)):
        assert got.shape == ref.shape and np.count_nonzero(ref) > 0
        assert np.all(np.abs(got - ref) <= tol * (np.abs(ref) + 1.0)), np.abs(got - ref).max()
