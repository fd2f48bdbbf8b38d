"""GB300-native drop-in for subsweep's radiative-transfer sweep + hydrogen chemistry.

The product is the CUDA library behind include/subsweep_gpu.h (built in-tree by
:func:`subsweep_gb300.build.build`); this package holds its Python bindings, a
mirror of the reference's sweep-plugin interface, and host-side grid/workload
producers.
"""
from .sweep import Sweep, SweepError, SweepParameters, directions_from_num  # noqa: F401

__all__ = ["Sweep", "SweepError", "SweepParameters", "directions_from_num"]
