"""mech_filament_energy_device (fixed device scratch, no allocation) against mech_energy.

Kept in its own file, collected last, so that it runs both alone and after
every other GPU test in one process.
"""
import ctypes as C

import numpy as np
import pytest

from picgo_gb300 import Engine, _lib, make_network, jitter

pytestmark = pytest.mark.gpu


def _device_arrays(torch, net):
    """The network's filament arrays on cuda:0, in the layout the entry point takes."""
    nfil = net.n_filaments
    fcs = np.asarray(net.fil_cyl_start, dtype=np.int32)
    # filament-contiguous beads: cylinder c of filament f joins beads c + f and c + f + 1
    fil_of = np.repeat(np.arange(nfil), np.diff(fcs))
    assert np.array_equal(net.cyl_b1, np.arange(net.n_cyl) + fil_of)
    assert np.array_equal(net.cyl_b2, net.cyl_b1 + 1)
    dev = torch.device("cuda", 0)
    t = {
        "fcs": torch.from_numpy(fcs).to(dev),
        "x": torch.from_numpy(np.ascontiguousarray(net.coord, dtype=np.float64)).to(dev),
        "ks": torch.from_numpy(np.asarray(net.cyl_kstr, np.float64)).to(dev),
        "l0": torch.from_numpy(np.asarray(net.cyl_l0, np.float64)).to(dev),
        "kb": torch.from_numpy(np.asarray(net.cyl_kbend, np.float64)).to(dev),
        "t0": torch.from_numpy(np.asarray(net.cyl_theta0, np.float64)).to(dev),
        "out": torch.full((2,), float("nan"), dtype=torch.float64, device=dev),
    }
    return t


def _call(L, torch, net, t):
    stream = torch.cuda.current_stream(0).cuda_stream
    p = lambda a: C.c_void_p(a.data_ptr())
    rc = L.mech_filament_energy_device(net.n_filaments, net.n_cyl, p(t["fcs"]), p(t["x"]), p(t["ks"]), p(t["l0"]),
                                       p(t["kb"]), p(t["t0"]), p(t["out"]), C.c_void_p(stream))
    _lib.check(rc)
    torch.cuda.synchronize()
    return t["out"].cpu().numpy().copy()


@pytest.mark.parametrize("shape", [(24, 10, 1400.0, 40), (200, 20, 2000.0, 500)])
def test_no_alloc_energy_matches_context_energy_twice(shape):
    torch = pytest.importorskip("torch")
    nf, nc, box, nl = shape
    net = jitter(make_network("c1", n_filaments=nf, n_cyl_per_filament=nc, box=box, n_linkers=nl), 0.5, seed=11)
    L = _lib.load()
    with Engine("fp64") as eng:
        eng.set_network(net)
        per, _, _ = eng.energies()
    t = _device_arrays(torch, net)
    first = _call(L, torch, net, t)
    second = _call(L, torch, net, t)
    ref = np.array([per[_lib.FF_NAMES.index("FilamentStretching")], per[_lib.FF_NAMES.index("FilamentBending")]])
    for got in (first, second):
        assert np.all(np.isfinite(got)), got
        assert np.all(np.abs(got - ref) <= 1e-12 * np.abs(ref) + 1e-12), (got, ref)
    # fixed summation order: the two calls agree bit for bit
    assert np.array_equal(first, second)


def test_no_alloc_rejects_sizes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    L = _lib.load()
    dummy = torch.zeros(8, dtype=torch.float64, device="cuda:0")
    p = C.c_void_p(dummy.data_ptr())
    rc = L.mech_filament_energy_device(1, 2_097_153, p, p, p, p, p, p, p, None)
    assert rc == -7, rc
    assert b"scratch" in L.mech_last_error()
    assert L.mech_filament_energy_device(1, 10, None, p, p, p, p, p, p, None) == -1
