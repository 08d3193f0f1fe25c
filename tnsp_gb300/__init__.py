"""GB300-native sampling-lattice Monte Carlo over PEPS (sweep sampling, E_loc, gradient)."""
from .lattice import SamplingLattice, random_heisenberg, neel  # noqa: F401


def __getattr__(name):
    # the GPU classes load the CUDA library on first use
    if name in ("SweepSampling", "Observer", "Configuration"):
        from . import sampling
        return getattr(sampling, name)
    raise AttributeError(name)
