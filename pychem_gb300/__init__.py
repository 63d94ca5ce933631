"""pychem_gb300: GB300-native (sm_103a) Hartree-Fock + MP2 hot path of pychem.

Layers:
  include/pychem_gb300.h + csrc/   C ABI and CUDA kernels (libpychem_gb300.so)
  _lib                               ctypes binding (fails loudly without the library)
  _c_ints                            drop-in module for the upstream `_c_ints` extension
  molecule, engine, scf              whole-molecule GPU integrals, RHF and MP2
"""
__version__ = "0.1.0"
