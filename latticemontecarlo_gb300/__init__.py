"""GB300-native lattice Monte Carlo hot path (cluster-expansion barriers,
energy changes, KMC and CMC drivers) behind a C ABI; see include/lmc_gb300.h."""
from . import _native
from ._native import LmcError
from .api import Context, Model, load_coefficients, write_coefficients

__all__ = ["Context", "Model", "LmcError", "load_coefficients", "write_coefficients", "_native"]
