"""GB300-native (sm_103a) XPFC semi-implicit spectral step behind a C ABI.

The product is libxpfc.so (include/xpfc.h); this package builds it in-tree
(build.py), binds it (_lib.py) and mirrors LC2500/XPFC_CUDA's interface
(api.py).
"""
from .api import (Batch, Server, Xpfc, XpfcError, build_initial_field, build_initial_field_device,  # noqa: F401
                  default_params, read_density_field, read_input, run_reference_loop, set_params, writeVTKFile)
from ._lib import load  # noqa: F401
