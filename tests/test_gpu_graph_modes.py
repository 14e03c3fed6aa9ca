"""The minimizer's graph modes against each other.

All run the same active kernels in the same order (the conditional graph only
skips the phases no replica is in; the programmatic-launch variant of the
unrolled graph only lets kernels be scheduled before their predecessor ends;
the cooperative tail runs the same work units and reductions in one launch),
so minimizations must agree bit for bit: iteration and call counts, energies,
final coordinates.
"""
import numpy as np
import pytest

from picgo_gb300 import Engine, cg_params, jitter, make_network
from picgo_gb300.network import make_ensemble

pytestmark = pytest.mark.gpu


def _run(precision, nets, mode, params):
    with Engine(precision) as eng:
        eng.set_graph_mode(mode)
        if len(nets) == 1:
            eng.set_network(nets[0])
        else:
            eng.set_networks(nets)
        res = eng.minimize(params)
        coords = [eng.coords(r) for r in range(len(nets))]
    return res, coords


def _same(a, b):
    (ra, ca), (rb, cb) = a, b
    for x, y in zip(ra, rb):
        for k in ("status", "num_iter", "num_force_call", "num_energy_eval", "num_line_search_trials",
                  "num_safe_mode", "num_recover"):
            assert x[k] == y[k], (k, x[k], y[k])
        assert x["grad_inf_norm"] == y["grad_inf_norm"]
        assert list(x["energies_after"]) == list(y["energies_after"])
    for u, v in zip(ca, cb):
        assert np.array_equal(u, v)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_conditional_graph_matches_unrolled_graph(precision):
    net = jitter(make_network("c1", n_filaments=120, n_cyl_per_filament=20, box=2000.0, n_linkers=300), 0.5, seed=5)
    p = cg_params(energy_rel_tol=0.0)
    a = _run(precision, [net], "conditional", p)
    b = _run(precision, [net], "unrolled", p)
    c = _run(precision, [net], "unrolled_pdl", p)
    assert a[0][0]["status"] == 0 and a[0][0]["grad_inf_norm"] < 1.0
    _same(a, b)
    _same(b, c)


def test_conditional_graph_matches_unrolled_graph_batched():
    nets = make_ensemble(6, seed=3, fil_range=(20, 200), cyl_range=(10, 20))
    p = cg_params(energy_rel_tol=0.0)
    a = _run("mixed", nets, "conditional", p)
    b = _run("mixed", nets, "unrolled", p)
    c = _run("mixed", nets, "unrolled_pdl", p)
    assert all(r["status"] == 0 for r in a[0])
    _same(a, b)
    _same(b, c)


def test_cooperative_tail_matches_unrolled_graph():
    net = jitter(make_network("c1", n_filaments=120, n_cyl_per_filament=20, box=2000.0, n_linkers=300), 0.5, seed=5)
    p = cg_params(energy_rel_tol=0.0)
    a = _run("mixed", [net], "unrolled", p)
    b = _run("mixed", [net], "unrolled_coop", p)
    assert a[0][0]["status"] == 0 and a[0][0]["grad_inf_norm"] < 1.0
    _same(a, b)
    # relaxed to |F| <= 10 gradTol before the force-call limit: the direction
    # phase also copies the minimum-energy backup, and the limit ends the run
    small = make_network("c1", n_filaments=3, n_cyl_per_filament=5, box=1500.0, n_linkers=0, seed=11)
    small.coord = small.coord + np.random.default_rng(0).normal(0, 1e-2, small.coord.shape)
    q = cg_params(grad_tol=1e-3, energy_rel_tol=0.0, report_on_call_limit=1, energy_call_limit=0, force_call_limit=0)
    c = _run("mixed", [small], "unrolled", q)
    d = _run("mixed", [small], "unrolled_coop", q)
    _same(c, d)
    # FP64 and batched contexts keep the separate launches
    _same(_run("fp64", [net], "unrolled", p), _run("fp64", [net], "unrolled_coop", p))
    nets = make_ensemble(3, seed=3, fil_range=(20, 60), cyl_range=(10, 20))
    _same(_run("mixed", nets, "unrolled", p), _run("mixed", nets, "unrolled_coop", p))
