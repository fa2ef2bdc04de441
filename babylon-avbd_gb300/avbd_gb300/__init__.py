"""avbd_gb300: the reference's per-step 3D AVBD rigid-body pipeline on one GB300 (sm_103a).

Host side of the engine: the scene builder (``AvbdScene3D``), ``createSolverPipeline`` with
its worlds, batches and world servers over the C ABI of ``libavbd_gb300.so``, and the synthetic benchmark
scenes. The compute path is CUDA only; there is no CPU fallback.
"""
from .scene import AvbdScene3D, Hinge, SceneArrays, SceneBuilder, SolverParams  # noqa: F401
from .pipeline import Batch, Server, SolverPipeline, World, createSolverPipeline  # noqa: F401

__all__ = ["AvbdScene3D", "Hinge", "SceneArrays", "SceneBuilder", "SolverParams", "createSolverPipeline",
           "SolverPipeline", "World", "Batch", "Server"]
