"""GB300-native engine for MEDYAN's mechanical-equilibration path.

Force fields (filament stretching and bending, linker and motor stretching,
cylinder excluded volume, boundary repulsion), the neighbor-list rebuild and
the Polak-Ribiere CG minimizer run as sm_103a CUDA kernels behind the C ABI
of include/medyan_mech.h; this package builds that library and drives it.
"""
from .network import CONFIGS, Network, jitter, make_network  # noqa: F401
from .engine import Engine, cg_params  # noqa: F401
