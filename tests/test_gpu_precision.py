"""Mixed precision against FP64 at the end of a minimization (the 200 x 20
network: 4,000 cylinders, 500 linkers, seed 20261204), and the mixed engine's
accumulation error separated from the error of its single-precision terms.

End state: the mixed engine minimizes to max|F| < 1 pN.  At its end
coordinates:
* the FP64 oracle's energy agrees with the mixed energy to 1e-6 relative;
* FP64 CG continued from there to the same 1 pN tolerance (the "FP64 polish")
  changes the energy by at most 1e-6 relative and moves no bead by more than
  1 nm: the mixed end state is an FP64 equilibrium of the same tolerance, not
  merely a nearby configuration.  (Minimizing both precisions from the seeded
  start is no error measure: on this frustrated network the two line searches
  branch differently after a few iterations and end in different local minima.)

Accumulation: the mixed engine sums single-precision terms in compensated
float pairs.  Summing the same per-cylinder FP32 terms exactly on the host
(math.fsum) must reproduce the engine's filament energies to 1e-10 relative
(the compensated pairs carry ~48 bits; a million terms),
while the FP32 terms themselves differ from FP64 by ~1e-7.
"""
import math

import numpy as np
import pytest

import oracle
from picgo_gb300 import Engine, cg_params, jitter, make_network

pytestmark = pytest.mark.gpu


def test_mixed_end_state_is_an_fp64_equilibrium():
    net = make_network("c1", seed=20261204)
    vec = oracle.vectorize(net)
    prm = cg_params(energy_rel_tol=0.0, force_call_limit=200000)
    with Engine("mixed") as eng:
        eng.set_network(net)
        r = eng.minimize(prm)[0]
        x_m = eng.coords()
        _, e_m, _ = eng.energies()
    assert r["status"] == 0 and r["grad_inf_norm"] < 1.0
    e_o, _ = oracle.energies(vec, x_m)
    assert abs(e_m - e_o) <= 1e-6 * abs(e_o), (e_m, e_o)
    with Engine("fp64") as eng:
        eng.set_network(net)
        eng.set_coords(x_m)
        r64 = eng.minimize(prm)[0]
        x_p = eng.coords()
    assert r64["status"] == 0 and r64["grad_inf_norm"] < 1.0
    e_p = r64["energies_after"][6]
    assert abs(e_p - e_o) <= 1e-6 * abs(e_o), (e_p, e_o, r64["num_iter"])
    assert np.linalg.norm(x_p - x_m, axis=1).max() <= 1.0


@pytest.mark.parametrize("name", ["c1", "c2"])
def test_mixed_accumulation_is_exact_to_double(name):
    net = jitter(make_network(name), 0.7, seed=3)   # bent filaments: bending energy well above round-off
    vec = oracle.vectorize(net)
    _, o_per = oracle.energies(vec, net.coord)
    with Engine("mixed") as eng:
        eng.set_network(net)
        per, _, _ = eng.energies()
        st, bd = eng.energy_terms()
    for k, terms in ((0, st), (1, bd)):
        exact = math.fsum(terms.tolist())
        # the engine's sum of its own FP32 terms: accumulation error only
        assert abs(per[k] - exact) <= 1e-10 * abs(exact), (k, per[k], exact)
        # the FP32 terms against FP64: the term error, orders of magnitude larger
        assert abs(exact - o_per[k]) <= 1e-6 * abs(o_per[k])
    with Engine("fp64") as eng:
        eng.set_network(net)
        per64, _, _ = eng.energies()
        st64, bd64 = eng.energy_terms()
    assert abs(math.fsum(st64.tolist()) - per64[0]) <= 1e-13 * abs(per64[0])
