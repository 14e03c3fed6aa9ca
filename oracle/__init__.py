"""CPU FP64 oracle of MEDYAN's mechanical-equilibration path.

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by ``bench.py``'s CPU-baseline leg, as the checker.  The product library
(``picgo_gb300``) never imports it.
"""
from .oracle import (  # noqa: F401
    FF_NAMES, CGParams, CGResult, System, Vectorized, build, lib, vectorize, energy, energies, forces,
    cyl_pairs, cyl_pairs_fast, boundary_list, minimize, minimize_quadratic, cg_params, force_scale,
    series_atan_mode, threads, stretch_forces, load_forces,
)
