"""Failure branches of the minimizer and the force-field manager, GPU against the oracle.

* A line search that cannot succeed (lambdaMax = 1e-9 puts the first trial
  below the 1e-8 step tolerance, CGMethod.hpp:238-373): with recovery disabled
  the minimization stops after one iteration with errorLineSearch
  (MECH_ERR_LINESEARCH); with recovery enabled it alternates safe mode and
  MController's recovery move (CGMethod.hpp:1600-1743, MController.h:273-339),
  call for call like the oracle.
* The minimum-energy backup (CGMethod.hpp:1540-1580, 1722-1724): a network
  relaxing slowly near equilibrium reaches the force-call limit with
  reportOnCallLimit set and returns its lowest-energy relaxed coordinates.
* A force field that fails: coincident cylinders of two filaments make both
  the analytic and the numeric excluded-volume energy fail (-1), and the
  manager's total becomes +inf (ForceFieldManager.cpp:96-207).
"""
import numpy as np
import pytest

import oracle
from picgo_gb300 import Engine, cg_params, jitter, make_network

pytestmark = pytest.mark.gpu


def _net():
    return jitter(make_network("c1", n_filaments=60, n_cyl_per_filament=12, box=1500.0, n_linkers=80, n_motors=40,
                               seed=3), 0.3, seed=7)


def _counters(r):
    return (r["num_iter"], r["num_energy_call"], r["num_force_call"], r["num_safe_mode"], r["num_recover"])


def _o_counters(r):
    return (r.numIter, r.numEnergyCall, r.numForceCall, r.numSafeMode, r.numRecover)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_line_search_failure_without_recovery(precision):
    net = _net()
    vec = oracle.vectorize(net)
    x_o, _, r_o = oracle.minimize(vec, net.coord, oracle.cg_params(lambdaMax=1e-9, energyCallLimit=40, tryToRecover=0))
    assert r_o.errorFlags & 1
    with Engine(precision) as eng:
        eng.set_network(net)
        r = eng.minimize(cg_params(lambda_max=1e-9, energy_call_limit=40, try_to_recover=0))[0]
        x = eng.coords()
    assert r["status"] == -5 and r["error_flags"] & 1, r
    assert _counters(r) == _o_counters(r_o)
    assert np.abs(x - net.coord).max() <= 1e-9 * np.abs(net.coord).max()


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("mixed", 1e-5)])
def test_safe_mode_and_recovery_moves_track_oracle(precision, tol):
    net = _net()
    vec = oracle.vectorize(net)
    x_o, _, r_o = oracle.minimize(vec, net.coord, oracle.cg_params(lambdaMax=1e-9, energyCallLimit=40, tryToRecover=1))
    assert r_o.numSafeMode >= 5 and r_o.numRecover >= 5
    with Engine(precision) as eng:
        eng.set_network(net)
        r = eng.minimize(cg_params(lambda_max=1e-9, energy_call_limit=40, try_to_recover=1))[0]
        x = eng.coords()
    assert r["status"] == 0 and r["error_flags"] == 0, r
    assert _counters(r) == _o_counters(r_o)
    # each recovery moves the largest direction component by maxDist = 1 nm
    assert np.abs(x_o - net.coord).max() > 1.0
    assert np.abs(x - x_o).max() <= tol * np.abs(x_o).max(), np.abs(x - x_o).max()


def test_minimum_energy_backup_on_call_limit():
    """18 beads (force-call limit 3 x 18 = 54) relaxing from a 0.01 nm perturbation with
    gradTol 1e-3 pN: relaxed (|F| <= 10 gradTol) after iteration 27 but not converged when
    the limit hits, so the lowest-energy relaxed coordinates are returned."""
    net = make_network("c1", n_filaments=3, n_cyl_per_filament=5, box=1500.0, n_linkers=0, seed=11)
    x0 = net.coord + np.random.default_rng(0).normal(0, 1e-2, net.coord.shape)
    vec = oracle.vectorize(net)
    prm_o = oracle.cg_params(gradTol=1e-3, energyRelTol=0.0, reportOnCallLimit=1, energyCallLimit=0,
                             forceCallLimit=0)
    x_o, _, r_o = oracle.minimize(vec, x0, prm_o)
    assert r_o.usedBackup == 1
    with Engine("fp64") as eng:
        eng.set_network(net)
        eng.set_coords(x0)
        r = eng.minimize(cg_params(grad_tol=1e-3, energy_rel_tol=0.0, report_on_call_limit=1, energy_call_limit=0,
                                   force_call_limit=0))[0]
        x = eng.coords()
    assert r["used_backup"] == 1, r
    assert _counters(r) == _o_counters(r_o)
    assert np.abs(x - x_o).max() <= 1e-9 * np.abs(x_o).max()
    # a relaxed 18-bead network: its energy (4e-5 pN nm) is round-off of terms of ~1 pN nm
    assert abs(r["energies_after"][6] - r_o.energiesAfter[6]) <= 1e-6 * abs(r_o.energiesAfter[6]) + 1e-9


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_failing_force_field_makes_energy_infinite(precision):
    net = make_network("c1", n_filaments=4, n_cyl_per_filament=3, box=1500.0, n_linkers=0, seed=11)
    x = net.coord.copy()
    c0 = np.array([700.0, 700.0, 700.0])
    for i in range(4):   # filaments 0 and 1 on top of each other
        x[i] = c0 + np.array([(i - 1.5) * 108.0, 0, 0])
        x[4 + i] = x[i]
    net.coord = x
    vec = oracle.vectorize(net)
    o_tot, o_per = oracle.energies(vec, x)
    assert o_per[4] == -1.0 and oracle.energy(vec, x) == np.inf
    with Engine(precision) as eng:
        eng.set_network(net)
        per, tot, en = eng.energies()
    assert per[4] == -1.0, per
    assert en == np.inf
    # the plain total: -1 plus the other force fields (single-precision terms in mixed)
    assert abs(tot - o_tot) <= (1e-9 if precision == "fp64" else 1e-6) * (abs(o_tot) + 1.0)
