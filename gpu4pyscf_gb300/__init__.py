"""GB300-native direct-SCF Coulomb/exchange (J/K) engine.

The public entry points mirror gpu4pyscf: ``scf.jk.get_jk``, ``scf.jk.get_j``,
``scf.jk.get_k``, ``scf.jk._VHFOpt`` and ``scf.hf.RHF``.  Integrals run in
hand-written sm_103a CUDA kernels reached through the C ABI declared in
include/gb300jk.h.
"""
__version__ = '0.1.0'
from . import gto
