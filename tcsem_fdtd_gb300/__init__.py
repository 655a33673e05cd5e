"""GB300-native (sm_103a) implementation of the TCSEM_FDTD time-stepping path.

The compute path is the CUDA library ``libtcsem.so`` behind the C ABI of
``include/tcsem.h``; :class:`Simulation` (one survey) and :class:`Batch`
(many surveys advanced together) are its Python mirror, and
:mod:`tcsem_fdtd_gb300.inputs` writes seeded synthetic surveys in the
reference's file formats.
"""
from .api import COMP, Batch, Simulation, TcsemError, declared_functions, library  # noqa: F401

__all__ = ["Simulation", "Batch", "TcsemError", "library", "declared_functions", "COMP"]
