"""GB300-native photon-transport engine (mcsub / mcxyz hop-drop-spin-roulette).

The engine is the CUDA shared library nmc_gb300/_build/libnmc_gb300.so behind
the C ABI of include/nmc_abi.h.  Importing this package does not load it;
the first engine call does, and raises if it has not been built.
"""
from . import abi  # noqa: F401

__all__ = ["abi"]
