"""GB300-native exact-diagonalisation engine with PyHub's Python API.

The hot path -- the on-the-fly H*v product of a fixed (N_up, N_down)
Fermi-Hubbard sector or fixed-Sz Heisenberg sector, and the Lanczos, RDM and
Green's-function loops built on it -- runs as hand-written sm_103a CUDA behind
the C ABI of include/pyhub_ed.h (``libpyhub_ed.so``).  The Python classes
mirror pyhub.solver / pyhub.core / pyhub.tools.
"""
__version__ = "1.0.0"
