"""GB300-native sampling-lattice Monte Carlo over PEPS (sweep sampling, E_loc, gradient)."""
from .lattice import SamplingLattice, random_heisenberg, neel  # noqa: F401
