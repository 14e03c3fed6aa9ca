"""torch.autograd.Function over the equilibrium map theta -> x*(theta), E(x*, theta).

theta are the per-linker stiffness k and rest length l0 of one replica.  The
forward pass minimizes the network (Polak-Ribiere CG, then Newton refinement
with exact Hessian-vector products) from a given start; the backward pass is
the implicit adjoint (mech_adjoint): one CG solve with the Hessian, then the
per-linker terms.  It exists for gradient checks against finite differences,
so it runs on CPU tensors and converts through numpy.
"""
from __future__ import annotations

import numpy as np
import torch

from .engine import Engine, cg_params


class EquilibriumOptions:
    def __init__(self, grad_tol: float = 1e-3, newton_steps: int = 30, newton_force_tol: float = 1e-9,
                 cg_rel_tol: float = 1e-10, cg_max_iter: int = 50000, rebuild_at_minimum: bool = True):
        self.grad_tol = grad_tol
        self.newton_steps = newton_steps
        self.newton_force_tol = newton_force_tol
        self.cg_rel_tol = cg_rel_tol
        self.cg_max_iter = cg_max_iter
        self.rebuild_at_minimum = rebuild_at_minimum


def equilibrate(engine: Engine, x0: np.ndarray, k: np.ndarray, l0: np.ndarray, opts: EquilibriumOptions,
                replica: int = 0):
    """Minimize replica 0 from x0 with linker parameters (k, l0); returns (x*, E*, info)."""
    engine.set_coords(x0, replica)
    engine.set_linker_params(k, l0, replica)
    prm = cg_params(grad_tol=opts.grad_tol, energy_rel_tol=0.0, force_call_limit=10_000_000)
    r = engine.minimize(prm)[replica]
    if opts.rebuild_at_minimum:
        engine.rebuild()
        r = engine.minimize(prm)[replica]
    info = engine.newton_refine(opts.newton_steps, opts.newton_force_tol, 1e-8, opts.cg_max_iter)
    info["cg_status"] = r["status"]
    x = engine.coords(replica)
    e = engine.energies(replica=replica)[1]
    return x, e, info


class Equilibrium(torch.autograd.Function):
    """(k, l0) -> (x* [n_beads, 3], E*): forward = minimization, backward = implicit adjoint."""

    @staticmethod
    def forward(ctx, k: torch.Tensor, l0: torch.Tensor, engine: Engine, x0: np.ndarray,
                opts: EquilibriumOptions):
        x, e, info = equilibrate(engine, x0, k.detach().double().numpy(), l0.detach().double().numpy(), opts)
        ctx.engine = engine
        ctx.x = x
        ctx.k = k.detach().double().numpy().copy()
        ctx.l0 = l0.detach().double().numpy().copy()
        ctx.opts = opts
        ctx.info = info
        return torch.from_numpy(x), torch.tensor(e, dtype=torch.float64)

    @staticmethod
    def backward(ctx, gx: torch.Tensor, gE: torch.Tensor):
        eng: Engine = ctx.engine
        # the adjoint runs at this forward pass's equilibrium and parameters
        eng.set_coords(ctx.x)
        eng.set_linker_params(ctx.k, ctx.l0)
        g = np.zeros(ctx.x.shape) if gx is None else gx.detach().double().numpy()
        wE = 0.0 if gE is None else float(gE)
        dk, dl, info = eng.adjoint(g, wE, rel_tol=ctx.opts.cg_rel_tol, max_iter=ctx.opts.cg_max_iter)
        ctx.adjoint_info = info
        return torch.from_numpy(dk), torch.from_numpy(dl), None, None, None
