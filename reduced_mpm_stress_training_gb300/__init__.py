"""GB300-native (sm_103a) MPM substep, a drop-in for MPM_Simulator_WARP.p2g2p
of zeshunzong/reduced_mpm_stress_training (engine_stress/mpm_solver_warp.py).

Importing the package does not touch the GPU; the CUDA library
(libmpm_gb300.so, built by ``build.build()``) is loaded on first use and its
absence is an error -- there is no CPU fallback.
"""
from .engine import Collider, MPMEngine, MPMStatusError, SceneParams  # noqa: F401
from .solver import MPM_Simulator_WARP, MPMSimulator  # noqa: F401

__version__ = "0.1.0"
