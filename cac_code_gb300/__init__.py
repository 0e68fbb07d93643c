"""GB300-native CAC per-step force path (sm_103a CUDA behind a C ABI).

* ``cac_code_gb300.cacg``    -- ctypes binding of libcacg.so and ``System``
* ``cac_code_gb300.lattice`` -- seeded FCC/element models, data and EAM files
* ``cac_code_gb300.build``   -- in-tree nvcc build of libcacg.so
"""
from . import build, lattice  # noqa: F401

__all__ = ["build", "lattice", "cacg"]
