"""ocean_gb300: GB300-native (sm_103a) BSE Hamiltonian action and Haydock/GMRES
solvers for OCEAN's core-level spectroscopy path.

The product is the C-ABI library libocean_gpu.so (include/ocean_gpu.h); this
package holds its sources (csrc/), the in-tree build (build.py), ctypes bindings
(capi.py) and the seeded synthetic workloads (workloads.py).
"""
from . import workloads  # noqa: F401

__all__ = ["workloads", "capi", "build"]
