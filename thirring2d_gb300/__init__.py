"""GB300-native (sm_103a) hybrid Monte Carlo hot path of the 2D staggered Thirring model.

The compute lives in libthirring_gpu.so (CUDA C ABI, include/thirring_gpu.h);
this package is its numpy front end.  Importing it does not load the library;
`Lattice(...)` does, and raises if it is missing.
"""
from .lattice import Batch, Lattice, batch_params, cg_params, hmc_params  # noqa: F401
from . import native  # noqa: F401
