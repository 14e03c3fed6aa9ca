"""The seeded network generator (picgo_gb300/network.py), on CPU.

Every benchmark and parity case starts from these networks, so their topology
invariants, placement bounds and seeding are checked here.
"""
import numpy as np
import pytest

from picgo_gb300 import jitter, make_network
from picgo_gb300.network import make_ensemble


def _check_topology(net):
    nf, nc = net.n_filaments, net.n_cyl
    fcs = np.asarray(net.fil_cyl_start)
    assert fcs[0] == 0 and fcs[-1] == nc and np.all(np.diff(fcs) > 0)
    # cylinders filament by filament, minus end first, consecutive beads
    fil_of = np.repeat(np.arange(nf), np.diff(fcs))
    assert np.array_equal(net.cyl_fil, fil_of)
    assert np.array_equal(net.cyl_pos, np.concatenate([np.arange(k) for k in np.diff(fcs)]))
    b1, b2 = np.asarray(net.cyl_b1), np.asarray(net.cyl_b2)
    assert np.all((b1 >= 0) & (b1 < net.n_beads) & (b2 >= 0) & (b2 < net.n_beads))
    same = np.diff(fil_of) == 0
    assert np.array_equal(b2[:-1][same], b1[1:][same])      # a filament's cylinders share beads
    assert len(np.unique(net.cyl_id)) == nc
    for cyl, pos in ((net.lk_cyl, net.lk_pos), (net.mt_cyl, net.mt_pos)):
        cyl = np.asarray(cyl)
        if len(cyl):
            assert cyl.min() >= 0 and cyl.max() < nc
            assert np.all(net.cyl_fil[cyl[:, 0]] != net.cyl_fil[cyl[:, 1]])   # bonds join two filaments
            assert np.all((pos >= 0) & (pos <= 1))
    assert np.all(np.asarray(net.lk_k) > 0) and np.all(np.asarray(net.lk_l0) > 0)


@pytest.mark.parametrize("shape", [dict(n_filaments=60, n_cyl_per_filament=12, box=1500.0, n_linkers=80, n_motors=10),
                                   dict(n_filaments=20, n_cyl_per_filament=30, box=3000.0, n_linkers=15)])
def test_generated_network_topology_and_bounds(shape):
    net = make_network("c1", seed=3, **shape)
    _check_topology(net)
    assert net.n_filaments == shape["n_filaments"] and net.n_cyl == shape["n_filaments"] * shape["n_cyl_per_filament"]
    # every bead inside the box, cylinders at their rest length
    assert np.all((net.coord > 0) & (net.coord < net.box))
    lens = np.linalg.norm(net.coord[net.cyl_b2] - net.coord[net.cyl_b1], axis=1)
    assert np.allclose(lens, net.cyl_l0, rtol=1e-9)
    # one repulsive plane per cube face, normals unit length
    assert net.planes.shape == (6, 4)
    assert np.allclose(np.linalg.norm(net.planes[:, :3], axis=1), 1.0)


def test_generator_is_seeded():
    a = make_network("c1", seed=11, n_filaments=30, n_cyl_per_filament=8, box=1500.0, n_linkers=20)
    b = make_network("c1", seed=11, n_filaments=30, n_cyl_per_filament=8, box=1500.0, n_linkers=20)
    c = make_network("c1", seed=12, n_filaments=30, n_cyl_per_filament=8, box=1500.0, n_linkers=20)
    assert np.array_equal(a.coord, b.coord) and np.array_equal(a.lk_cyl, b.lk_cyl)
    assert not np.array_equal(a.coord, c.coord)
    j1, j2 = jitter(a, 0.5, seed=2), jitter(a, 0.5, seed=2)
    assert np.array_equal(j1.coord, j2.coord) and not np.array_equal(j1.coord, a.coord)
    assert np.array_equal(a.coord, b.coord)        # jitter copies; the original is untouched


def test_shuffled_storage_keeps_the_same_geometry():
    kw = dict(seed=5, n_filaments=25, n_cyl_per_filament=10, box=1500.0, n_linkers=30)
    plain = make_network("c1", **kw)
    shuf = make_network("c1", shuffle_beads=True, shuffle_ids=True, **kw)
    _check_topology(shuf)
    # the same cylinder end points, stored in another bead order
    assert np.allclose(plain.coord[plain.cyl_b1], shuf.coord[shuf.cyl_b1])
    assert np.allclose(plain.coord[plain.cyl_b2], shuf.coord[shuf.cyl_b2])
    assert not np.array_equal(plain.cyl_id, shuf.cyl_id)


def test_ensemble_sizes_stay_in_their_ranges():
    nets = make_ensemble(5, seed=9, fil_range=(10, 60), cyl_range=(5, 9))
    assert len(nets) == 5
    for net in nets:
        _check_topology(net)
        counts = np.diff(net.fil_cyl_start)
        assert 10 <= net.n_filaments <= 60
        assert np.all((counts >= 5) & (counts <= 9))
        assert np.all((net.coord > 0) & (net.coord < net.box))


def test_c5_linkers_start_stretched_with_rest_lengths_in_range():
    """The adjoint workload's linkers: k ~ U(4, 12), rest length ~ U(20, 40) nm,
    attached where the attachment points are at least the rest length apart."""
    net = make_network("c5", seed=20261208)
    x = net.coord
    p1 = x[net.cyl_b1[net.lk_cyl[:, 0]]] * (1 - net.lk_pos[:, :1]) + net.lk_pos[:, :1] * x[net.cyl_b2[net.lk_cyl[:, 0]]]
    p2 = x[net.cyl_b1[net.lk_cyl[:, 1]]] * (1 - net.lk_pos[:, 1:]) + net.lk_pos[:, 1:] * x[net.cyl_b2[net.lk_cyl[:, 1]]]
    d = np.sqrt(((p2 - p1) ** 2).sum(1))
    assert len(d) == 5000
    assert np.all(d >= net.lk_l0 - 1e-9)
    assert net.lk_l0.min() >= 0.0 and net.lk_l0.max() <= 40.0
    assert np.mean((net.lk_l0 >= 20.0) & (net.lk_l0 <= 40.0)) > 0.99
    assert net.lk_k.min() >= 4.0 and net.lk_k.max() <= 12.0
