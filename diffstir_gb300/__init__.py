"""diffstir_gb300: differentiable 3D MLS-MPM stirring simulator on GB300 (sm_103a).

A GB300-native rebuild of the simulation path of DiffStir (a rod stirring a
non-Newtonian fluid; the rod's reaction force identifies Carreau, Cross and
Herschel-Bulkley viscosity parameters).  Hand-written CUDA kernels behind the C
ABI of include/diffstir.h; Python/PyTorch on the host.

* :mod:`diffstir_gb300.scene`      reference scene and synthetic benchmark scenes
* :mod:`diffstir_gb300.simulator`  Simulator (batched handle), RolloutFunction (autograd)
* :mod:`diffstir_gb300.compat`     the reference's simulation_functions module API
* :mod:`diffstir_gb300.ops`        batched 3x3 SVD / SVD backward kernels
"""

from . import scene  # noqa: F401
from .scene import Scene, reference_scene, synthetic_scene  # noqa: F401

__all__ = ['scene', 'Scene', 'reference_scene', 'synthetic_scene', 'Simulator', 'RolloutFunction']


def __getattr__(name):
    if name in ('Simulator', 'RolloutFunction'):
        from . import simulator
        return getattr(simulator, name)
    raise AttributeError(name)
