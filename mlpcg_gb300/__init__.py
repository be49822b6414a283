"""mlpcg_gb300 -- neural-preconditioned CG Poisson solve on voxel grids, native to GB300 (sm_103a).

Host code (this package) mirrors the reference's interface:

* ``sm_model_3d``  -- SMBlockFunction3D, SmallSMModelDn3D, ... and the
  extension-module stand-ins smblock3d / smblocktrans3d / smlinear3d;
* ``cg``           -- npcg, npcg_flex, npsd, model_predict;
* ``laplacian``    -- matrix-free FluidLaplacian and an FP64 CSR builder;
* ``precond``      -- PrecondPlan: coefficients precomputed once, fused levels;
* ``solver``       -- FusedSolver: the whole iteration on the GPU in one CUDA graph;
* ``scenes``       -- seeded synthetic scenes.

All arithmetic runs in ``lib/libmlpcg_gb300.so`` (C ABI: include/mlpcg_gb300.h).
"""
from . import _lib  # noqa: F401

__all__ = ["ops", "sm_model_3d", "cg", "laplacian", "scenes", "model", "clock"]
