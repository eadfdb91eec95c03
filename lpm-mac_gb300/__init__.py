"""GB300-native LPM quasi-static Newton load step.

Host-side Python mirror over liblpmgpu (hand-written CUDA for sm_103a behind
the C ABI in include/lpm_gpu.h):

  lattice   unit cells, lattice generators and the createBonds bond rule
  capi      ctypes binding of the C ABI (Lattice = one device lattice)
  adjoint   adjoint over a load history with checkpoints (lpm_backward_step)
  build     nvcc build of liblpmgpu.so
  fatigue   cyclic loading over lpm_fatigue_cycle (solveProblemCyclic)

The directory name is not a Python identifier; load it with
``__graft_entry__.load_package()``, which registers it as ``lpm_mac_gb300``.
"""
from . import adjoint, build, capi, fatigue, lattice  # noqa: F401
