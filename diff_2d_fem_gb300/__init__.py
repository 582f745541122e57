"""diff_2d_fem_gb300 — the implicit step of Diff_2D_FEM, GB300-native.

    import numpy as np, diff_2d_fem_gb300 as D
    model = D.Model()
    model.add_ground(0.0, mu=0.8)
    model.add_soft_body(np.ones((6, 72)), physical_size=(0.054, 0.0045), center=(0.0, 0.003),
                        E=0.5e6, nu=0.40, density=1100.0)
    model.finalize(); model.gravity = (0.0, -9.81)
    integ = D.ImplicitIntegrator()
    integ.simulate(model, 2e-3)

The step is hand-written CUDA for sm_103a (csrc/, bound through the C ABI of
include/d2f.h); PyTorch holds the device buffers.
"""
from .model import Model, SimConfig, Collider, NONE, DISC, ELLIPSE, BOX, TRIANGLE, HALFSPACE
from .integrator import ImplicitIntegrator
from .adjoint import AdjointPNCG2D
from .mesh import Mesh, build_scene, check_mesh, lame, mask_to_mesh

__version__ = "0.1.0"
__all__ = ["Model", "SimConfig", "Collider", "ImplicitIntegrator", "AdjointPNCG2D", "Mesh", "build_scene", "check_mesh", "lame", "mask_to_mesh",
           "NONE", "DISC", "ELLIPSE", "BOX", "TRIANGLE", "HALFSPACE"]
