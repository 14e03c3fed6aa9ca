"""Mixed precision against the FP64 oracle at the end of a minimization (the
200 x 20 network: 4,000 cylinders, 500 linkers).

The mixed engine minimizes to max|F| < 1 pN; at its end state the oracle's
FP64 energy must agree with the mixed engine's to 1e-6 relative, and the
oracle's own max|F| there must stay near the 1 pN tolerance (the mixed
forces carry single-precision error, bounded per component as in
test_gpu_parity's mixed checks).
"""
import numpy as np
import pytest

import oracle
from picgo_gb300 import Engine, cg_params, make_network

pytestmark = pytest.mark.gpu


def test_mixed_end_state_against_oracle():
    net = make_network("c1", seed=20261204)
    vec = oracle.vectorize(net)
    with Engine("mixed") as eng:
        eng.set_network(net)
        r = eng.minimize(cg_params(energy_rel_tol=0.0, force_call_limit=200000))[0]
        x = eng.coords()
        per, tot, _ = eng.energies()
    assert r["status"] == 0 and r["grad_inf_norm"] < 1.0
    e_o, per_o = oracle.energies(vec, x)
    assert abs(tot - e_o) <= 1e-6 * abs(e_o), (tot, e_o)
    f_o = oracle.forces(vec, x)
    assert np.abs(f_o).max() < 2.0, np.abs(f_o).max()
    # the FP64 oracle minimizing from the same start also reaches 1 pN; the two
    # line searches branch differently after a few iterations and this
    # frustrated network has many minima, so the end states are different
    # local minima (energies within ~10 % here): only a sanity band is asserted
    x_o, _, r_o = oracle.minimize(vec, net.coord, oracle.cg_params(energyRelTol=0.0, forceCallLimit=200000))
    assert r_o.gradInfNorm < 1.0
    assert abs(r_o.energiesAfter[6] - e_o) <= 0.25 * abs(r_o.energiesAfter[6])
