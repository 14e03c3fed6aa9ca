"""Batched replicas: independent networks of uneven size in one context,
minimized together, give each replica what a context of its own gives."""
import numpy as np
import pytest

from picgo_gb300 import Engine, cg_params
from picgo_gb300.network import make_ensemble

pytestmark = pytest.mark.gpu


def small_ensemble(n=4):
    return make_ensemble(n, seed=77, fil_range=(20, 120), cyl_range=(10, 24))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batched_evaluation_equals_single(precision):
    nets = small_ensemble()
    with Engine(precision) as eb:
        eb.set_networks(nets)
        got = [(eb.energies(replica=r)[0], eb.forces(replica=r)) for r in range(len(nets))]
        pairs = [eb.pairs(r) for r in range(len(nets))]
    for r, net in enumerate(nets):
        with Engine(precision) as es:
            es.set_network(net)
            per, f = es.energies()[0], es.forces()
            assert np.array_equal(pairs[r], es.pairs())
        assert np.allclose(got[r][0], per, rtol=1e-12, atol=1e-10), (r, got[r][0], per)
        assert np.allclose(got[r][1], f, rtol=1e-12, atol=1e-9), r


def test_batched_fp64_minimization_equals_single():
    nets = small_ensemble()
    prm = cg_params(energy_rel_tol=0.0, force_call_limit=200000)
    with Engine("fp64") as eb:
        eb.set_networks(nets)
        res = eb.minimize(prm)
        xs = [eb.coords(r) for r in range(len(nets))]
    for r, net in enumerate(nets):
        with Engine("fp64") as es:
            es.set_network(net)
            one = es.minimize(prm)[0]
            x1 = es.coords()
        assert res[r]["status"] == 0 and res[r]["grad_inf_norm"] < 1.0
        assert res[r]["num_iter"] == one["num_iter"], (r, res[r]["num_iter"], one["num_iter"])
        assert res[r]["energies_after"][6] == pytest.approx(one["energies_after"][6], rel=1e-12)
        assert np.abs(xs[r] - x1).max() <= 1e-9


def test_batched_mixed_minimization_converges_every_replica():
    nets = small_ensemble(6)
    with Engine("mixed") as eb:
        eb.set_networks(nets)
        res = eb.minimize(cg_params(energy_rel_tol=0.0, force_call_limit=200000))
    for r in res:
        assert r["status"] == 0 and r["grad_inf_norm"] < 1.0
        assert r["energies_after"][6] < r["energies_before"][6]
