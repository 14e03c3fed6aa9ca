"""The autotuner picks valid launch geometries and bin edges without changing results."""
import numpy as np
import pytest

from picgo_gb300 import Engine, jitter, make_network

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_autotune_keeps_results(precision):
    net = jitter(make_network("c1", seed=31), 0.5, seed=4)
    with Engine(precision) as eng:
        eng.set_network(net)
        pairs0 = eng.pairs()
        per0, tot0, _ = eng.energies()
        f0 = eng.forces()
        t = eng.autotune(force=True)
        assert 1 <= t["energy_tiles_per_block"] <= 64 and 1 <= t["force_tiles_per_block"] <= 64
        assert t["cell_scale"] > 0
        assert np.array_equal(eng.pairs(), pairs0)
        per1, tot1, _ = eng.energies()
        f1 = eng.forces()
        # tiles per block only regroup the partial sums
        assert abs(tot1 - tot0) <= 1e-12 * abs(tot0)
        assert np.allclose(f1, f0, rtol=0, atol=1e-9 * (1 + np.abs(f0).max()))
        again = eng.autotune()          # cached for this shape
        assert again == t
