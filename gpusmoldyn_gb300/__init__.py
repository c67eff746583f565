"""gpusmoldyn_gb300: GB300-native (sm_103a) Smoldyn Brownian-dynamics step.

The compute path is libgpusmoldyn.so (hand-written CUDA kernels behind the C
ABI in include/gpusmoldyn.h).  This package is the host-side mirror of the
reference's ParticleSystem interface plus a thin ctypes binding; it has no
CPU fallback.
"""
from . import _lib
from ._lib import BDError, load
from .system import System, actrxnrate, bindingradius, gauss_table, numrxnrate, unbindingradius
from .particle_system import ParticleSystem

__all__ = ["System", "ParticleSystem", "BDError", "load", "numrxnrate", "actrxnrate", "bindingradius",
           "unbindingradius", "gauss_table", "_lib"]
