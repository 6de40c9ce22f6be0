"""Host-side Python layer over libmflbm (the sm_103a MF-LBM hot path).

The compute path is the C ABI declared in include/mflbm.h; this package
only binds it (``mflbm.lib``), describes cases (``mflbm.cases``) and
generates synthetic porous media (``mflbm.geometry``).
"""
from . import abi, cases, geometry  # noqa: F401
