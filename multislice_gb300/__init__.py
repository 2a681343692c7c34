"""GB300 multislice TEM/STEM simulator: C++/CUDA (sm_103a) library behind a C ABI.

The compute path is libmsl.so (include/msl.h); this package only binds it
(ctypes) and supplies host logic: specimen generators and scan geometry.
"""
from . import specimen  # noqa: F401
from ._abi import MslError  # noqa: F401
from .api import Context, fparams_table, phonon_displacements, sigma, wavelength  # noqa: F401

__all__ = ["Context", "MslError", "fparams_table", "phonon_displacements", "sigma", "wavelength",
           "specimen"]
