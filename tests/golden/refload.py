"""Import the reference package (Diff_2D_FEM) on top of the serial Warp stand-in.

TEST INFRASTRUCTURE ONLY: used by make_golden.py in a checkout that has the reference
source next to it. The package's own __init__ is skipped (it pulls in the matplotlib and
OpenGL viewers, which are not part of the simulation); its modules are imported one by one
under their real package names so that their relative imports resolve.
"""
from __future__ import annotations

import importlib
import os
import sys
import types

HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)

import warp_shim  # noqa: E402


def load(ref_root):
    """Returns a namespace with Model, ImplicitIntegrator and the reference modules."""
    os.environ.setdefault("DIFF2DFEM_PRECISION", "double")
    warp_shim.install()
    if "Diff_2D_FEM" not in sys.modules:
        pkg = types.ModuleType("Diff_2D_FEM")
        pkg.__path__ = [ref_root]
        sys.modules["Diff_2D_FEM"] = pkg
    ns = types.SimpleNamespace()
    ns.mesh = importlib.import_module("Diff_2D_FEM.core.mesh")
    ns.sim_model = importlib.import_module("Diff_2D_FEM.sim_model")
    ns.integrator = importlib.import_module("Diff_2D_FEM.implicit.integrator")
    ns.solver = importlib.import_module("Diff_2D_FEM.implicit.solver")
    ns.kernels = importlib.import_module("Diff_2D_FEM.implicit.kernels")
    ns.affine = importlib.import_module("Diff_2D_FEM.implicit.affine")
    ns.actuation = importlib.import_module("Diff_2D_FEM.implicit.actuation")
    ns.ipc = importlib.import_module("Diff_2D_FEM.implicit.ipc_contact")
    ns.adjoint = importlib.import_module("Diff_2D_FEM.implicit.adjoint")
    ns.Model = ns.sim_model.Model
    ns.ImplicitIntegrator = ns.integrator.ImplicitIntegrator
    ns.wp = warp_shim
    return ns
