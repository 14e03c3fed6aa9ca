"""Hessian-vector products and the implicit adjoint (FP64 engine).

* the force Jacobian mode against central differences of the oracle's forces
  (h = 1e-5 nm along v), the energy Hessian mode against second differences
  of the oracle's energy, and the energy Hessian's symmetry u . (H v) = v . (H u)
  (the force routine moves nearly coplanar excluded-volume pairs, so only the
  energy Hessian is exactly symmetric);
* damped Newton refinement lowers max |F| by orders of magnitude;
* the adjoint gradient of L = E(x*) + mean over filaments |end - start|^2
  with respect to per-linker stiffness and rest length agrees with central
  finite differences (h = 1e-4 relative, each side re-equilibrated from x*)
  to 1e-4 relative.
"""
import numpy as np
import pytest

import oracle
from picgo_gb300 import Engine, cg_params, jitter, make_network

pytestmark = pytest.mark.gpu


def c5_like(n_filaments=40, n_cyl=10, n_linkers=120, seed=5, sigma=0.5):
    cfg = dict(n_filaments=n_filaments, n_cyl_per_filament=n_cyl, box=None, n_linkers=n_linkers,
               linker_k=(4.0, 12.0), linker_l0=(20.0, 40.0), n_motors=0, shape="chain")
    return jitter(make_network(cfg, seed=seed), sigma, seed=2)


def test_force_jacobian_matches_finite_differences_of_oracle_forces():
    net = c5_like()
    vec = oracle.vectorize(net)
    rng = np.random.default_rng(0)
    v = rng.normal(size=net.coord.shape)
    with Engine("fp64") as eng:
        eng.set_network(net)
        hv = eng.hvp(v, jacobian=True)
    h = 1e-5
    fd = -(oracle.forces(vec, net.coord + h * v) - oracle.forces(vec, net.coord - h * v)) / (2 * h)
    scale = np.abs(fd).max()
    assert np.abs(hv - fd).max() <= 1e-7 * scale + 1e-6, (np.abs(hv - fd).max(), scale)


def test_energy_hessian_matches_second_differences_of_oracle_energy():
    net = c5_like(seed=7)
    vec = oracle.vectorize(net)
    rng = np.random.default_rng(4)
    with Engine("fp64") as eng:
        eng.set_network(net)
        for _ in range(3):
            v = rng.normal(size=net.coord.shape)
            vhv = float((v * eng.hvp(v)).sum())
            h = 1e-4
            e0 = oracle.energy(vec, net.coord)
            fd = (oracle.energy(vec, net.coord + h * v) - 2 * e0 + oracle.energy(vec, net.coord - h * v)) / (h * h)
            # truncation ~1e-6 relative at this h, rounding ~1e-16 |E| / h^2
            assert abs(vhv - fd) <= 1e-5 * abs(fd) + 1e-14 * abs(e0) / (h * h), (vhv, fd)


def test_hvp_is_symmetric():
    net = c5_like(seed=9)
    rng = np.random.default_rng(1)
    u = rng.normal(size=net.coord.shape)
    v = rng.normal(size=net.coord.shape)
    with Engine("fp64") as eng:
        eng.set_network(net)
        hu, hv = eng.hvp(u), eng.hvp(v)
    a, b = float((u * hv).sum()), float((v * hu).sum())
    assert abs(a - b) <= 1e-10 * max(abs(a), abs(b)), (a, b)


def straight_net(seed=21):
    """C5's linker model on a small network of straight filaments: CG reaches
    1e-3 pN on it without safe mode, where Newton then converges."""
    cfg = dict(n_filaments=30, n_cyl_per_filament=8, box=1500.0, n_linkers=60, linker_k=(4.0, 12.0),
               linker_l0=(20.0, 40.0), n_motors=0)
    return make_network(cfg, seed=seed)


def end_to_end_loss(net, x):
    """mean over filaments of |last bead - first bead|^2, and its gradient."""
    fcs = np.asarray(net.fil_cyl_start)
    first = net.cyl_b1[fcs[:-1]]
    last = net.cyl_b2[fcs[1:] - 1]
    d = x[last] - x[first]
    nf = len(first)
    g = np.zeros_like(x)
    np.add.at(g, last, 2.0 * d / nf)
    np.add.at(g, first, -2.0 * d / nf)
    return float((d * d).sum(1).mean()), g


def test_newton_refine_tightens_the_equilibrium():
    """From a CG end state at 1e-3 pN, damped Newton lowers max |F| by orders of
    magnitude without raising the energy (the Hessian of these networks is very
    ill-conditioned, so the inner CG solves are inexact and the rate varies)."""
    net = straight_net(seed=21)
    with Engine("fp64") as eng:
        eng.set_network(net)
        r = eng.minimize(cg_params(grad_tol=1e-3, energy_rel_tol=0.0, force_call_limit=10000000))[0]
        assert r["grad_inf_norm"] < 1e-3
        e_cg = eng.energies()[1]
        info = eng.newton_refine(max_steps=30, force_tol=1e-9)
        assert info["max_force"] < 1e-6, info
        assert np.abs(eng.forces()).max() == pytest.approx(info["max_force"], rel=1e-9, abs=1e-12)
        assert eng.energies()[1] <= e_cg


def test_adjoint_matches_finite_differences():
    torch = pytest.importorskip("torch")
    from picgo_gb300.autograd import Equilibrium, EquilibriumOptions, equilibrate
    net = straight_net(seed=21)
    k0 = np.asarray(net.lk_k, dtype=np.float64)
    l00 = np.asarray(net.lk_l0, dtype=np.float64)
    opts = EquilibriumOptions()
    with Engine("fp64") as eng:
        eng.set_network(net)
        kt = torch.tensor(k0, requires_grad=True)
        lt = torch.tensor(l00, requires_grad=True)
        x, e = Equilibrium.apply(kt, lt, eng, net.coord, opts)
        xs = x.detach().numpy().copy()
        fcs = np.asarray(net.fil_cyl_start)
        first = torch.as_tensor(net.cyl_b1[fcs[:-1]], dtype=torch.long)
        last = torch.as_tensor(net.cyl_b2[fcs[1:] - 1], dtype=torch.long)
        loss = e + ((x[last] - x[first]) ** 2).sum(1).mean()
        loss.backward()
        gk, gl = kt.grad.numpy().copy(), lt.grad.numpy().copy()
        fd_opts = EquilibriumOptions(rebuild_at_minimum=False)
        rng = np.random.default_rng(3)
        picks = rng.choice(len(k0), size=4, replace=False)

        def L(k, l0):
            xe, ee, info = equilibrate(eng, xs, k, l0, fd_opts)
            assert info["max_force"] < 1e-8, info
            return ee + end_to_end_loss(net, xe)[0]

        for j in picks:
            for which, g in (("k", gk), ("l0", gl)):
                base = k0 if which == "k" else l00
                h = 1e-4 * base[j]
                p, m = base.copy(), base.copy()
                p[j] += h
                m[j] -= h
                if which == "k":
                    fd = (L(p, l00) - L(m, l00)) / (2 * h)
                else:
                    fd = (L(k0, p) - L(k0, m)) / (2 * h)
                assert abs(g[j] - fd) <= 1e-4 * abs(fd) + 1e-7 * (1 + abs(fd)), (which, j, g[j], fd)
