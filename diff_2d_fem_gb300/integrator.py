"""ImplicitIntegrator — the implicit backward-Euler PNCG-IPC step, on the GPU.

Same constructor arguments and methods as the reference's ImplicitIntegrator
(implicit/integrator.py:34-358): `simulate(model, dt)`, `stats(model)`, `cfl_number`,
`attach`. The first simulate() builds the solver problem on the host (scene.py) and binds
it to device memory (device.py); every step after that is one kernel launch covering every
environment, with convergence tested per environment on the device.

New keyword-only options, all off by default:
  precision   "fp64" (the reference's arithmetic; default, or DIFF2DFEM_PRECISION=double)
              or "mixed": element, barrier and preconditioner arithmetic in FP32 with FP64
              positions, dot products, energies and step lengths.
  gtol        stop an environment once its gradient norm falls below gtol x the norm at
              the step's first iteration (in addition to the reference's tests).
  threads, blocks_per_sm   launch shape of the per-scene kernel (0 = tuned default).
  blocks_per_scene         mixed precision: a cluster of 8, 12 or 16 blocks per scene for large
                           scenes (0 = library default, 1 = a block per scene).
"""
from __future__ import annotations

import os
import warnings

import numpy as np

from . import scene as _scene


def _default_precision():
    p = os.environ.get("DIFF2DFEM_PRECISION", "double").strip().lower()
    if p in ("double", "float64", "64", "d", "fp64"):
        return "fp64"
    if p in ("mixed", "fp32", "single", "float32", "32", "f"):
        return "mixed"
    raise ValueError(f"DIFF2DFEM_PRECISION must be 'double' or 'mixed', not {p!r}")


class ImplicitIntegrator:
    def __init__(self, max_iter=None, eps=None, self_collision=True, friction=True,
                 near_factor=4.0, alpha_max=3.0, area_shrink=0.1, ccd_eta=0.9,
                 self_radius=None, tol_x=0.0, conv_check=8,
                 line_search=False, n_backtrack=4, ls_tol=1e-7, rigid_modes=True,
                 iters_per_cfl=2.0, max_iter_cap=2000, cg_restart=None, *,
                 precision=None, gtol=0.0, threads=0, blocks_per_sm=0, blocks_per_scene=0):
        self.precision = _default_precision() if precision is None else str(precision)
        if self.precision not in ("fp64", "mixed"):
            raise ValueError("precision must be 'fp64' or 'mixed'")
        self.max_iter = None if max_iter is None else int(max_iter)
        self.iters_per_cfl = float(iters_per_cfl)
        self.max_iter_cap = int(max_iter_cap)
        self.eps = float(1e-10 if eps is None else eps)
        self.tol_x = float(tol_x)
        self.conv_check = int(conv_check)
        self.line_search = bool(line_search)
        self.n_backtrack = int(n_backtrack)
        self.ls_tol = float(ls_tol)
        self.self_collision = bool(self_collision)
        self.friction = bool(friction)
        self.near_factor = float(near_factor)
        self.alpha_max = float(alpha_max)
        self.area_shrink = float(area_shrink)
        self.ccd_eta = float(ccd_eta)
        self.self_radius = self_radius
        self.rigid_modes = bool(rigid_modes)
        self.cg_restart = cg_restart
        self.gtol = float(gtol)
        self.threads = int(threads)
        self.blocks_per_sm = int(blocks_per_sm)
        self.blocks_per_scene = int(blocks_per_scene)

    # ---- the step (implicit/integrator.py:81-86)
    def simulate(self, model, dt, control=None):
        s = self.attach(model, dt)
        s.set_targets(model._targets)
        s.step()
        model.time += dt

    def cfl_number(self, model, dt):
        return _scene.cfl_number(model, dt)

    def stats(self, model):
        s = model._solver
        it, ac, st = s.stats()
        out = dict(iters=it, converged=(ac == 0), max_iter=s.iter_max, status=st)
        if s.prob.get("ipc") is not None and len(s.bc_sorted):
            x = s.get_x()
            tg = s.tensor("bc_target").cpu().numpy()
            out["bc_lag"] = float(np.linalg.norm(tg - x[s.bc_sorted], axis=1).max())
        return out

    def attach(self, model, dt):
        if model._solver is None:
            self._build(model, dt)
        s = model._solver
        if abs(s.dt - dt) > 1e-12 * dt:
            s.dt = float(dt)
            s.iter_max = _scene.iters_for(model, self, dt)
            s.set_dt(dt, s.iter_max)
        self._sync_actuation(model)
        return model._solver        # rebuilt by the sync when a term was added

    def _sync_actuation(self, model):
        """Rebuild the solver when an actuator was added (from the current state), and push
        the commands that changed since the last step: force field (gravity folded in),
        chamber pressures, tendon tensions and lengths, active-region rest shapes, spring
        anchors and lengths (implicit/integrator.py:151-229)."""
        s = model._solver
        f = _scene.external_force(model) if s._ctrl_version != model._ctrl_version else None
        # a term the solver was built without (an actuator, or a first force field): rebuild
        if s._act_version != model._act_version or (f is not None and "fext" not in s._t):
            model._x_host, model._v0 = s.get_x(), s.get_v()
            dt = s.dt
            s.close()
            model._solver = None
            self._build(model, dt)
            s = model._solver
        if s._ctrl_version != model._ctrl_version:
            if f is not None:
                s.set_fext(f)
            if model._chambers:
                s.set_pressures([c.pressure for c in model._chambers])
            if model._tendons:
                s.set_tendons([t.tension for t in model._tendons], [t.length for t in model._tendons])
            if model._regions:
                s.set_rest_shape(*_scene.rest_shape(model))
            if model._springs:
                s.set_springs([k.anchor for k in model._springs], [k.length for k in model._springs])
            s._ctrl_version = model._ctrl_version

    # ---- contact read-outs (implicit/integrator.py:340-358), computed on the device
    def collider_force(self, model, index=None, friction=True):
        """Reaction on the colliders (barrier, + friction unless friction=False) per
        environment, (B, 2): on collider `index`, or on all of them when index is None."""
        return model._solver.collider_force(index, include_friction=friction)

    def contact_force(self, model, handle=None, friction=True, colliders=True, bodies=True):
        """Force contact exerts on each node of a body [N/m], (n_body_nodes, 2), or (N, 2)
        for every node when handle is None; kinematic nodes included."""
        f = model._solver.contact_force(friction=friction, colliders=colliders, bodies=bodies)
        return f if handle is None else f[model.body_nodes(handle)]

    def body_contact_force(self, model, handle, friction=True, colliders=True, bodies=True):
        """Resultant of contact_force over a body: (fx, fy) [N/m]."""
        return self.contact_force(model, handle, friction, colliders, bodies).sum(0)

    def adjoint(self, model, dt, Emin=1e-3):
        """Adjoint of the implicit solve on this model (implicit/integrator.py:231-250): an
        AdjointPNCG2D over its FP64 solver. Density scales each element's stiffness,
        E(rho) = Emin + rho (1 - Emin); transient_adjoint refuses to run while the model has
        actuators the adjoint operator has no tangent for (pressure, springs, active
        material) or IPC contact between bodies."""
        from .adjoint import AdjointPNCG2D
        return AdjointPNCG2D(self.attach(model, dt), Emin=Emin, model=model)

    def _build(self, model, dt):
        from .device import DeviceSolver
        prob = _scene.solver_problem(model, self, dt)
        prob["rest"] = np.asarray(model.me.rest_pos, np.float64)
        if prob.get("ipc") is not None:
            gap = _scene.min_distance(prob)
            if not gap.min() > 0.0:
                raise ValueError(
                    f"two surfaces touch in environment {int(gap.argmin())} before the first "
                    f"step. IPC contact needs the bodies to start apart: leave a gap between "
                    f"them (anything from model.dhat = {model.dhat:.3g} m up is out of the "
                    f"barrier's reach).")
            if any(b.is_mesh for b in model._bodies) and gap.min() < model.dhat:
                warnings.warn(
                    f"two boundaries are {gap.min():.3g} m apart at rest in environment "
                    f"{int(gap.argmin())}, inside the barrier's reach (model.dhat = "
                    f"{model.dhat:.3g} m): they push each other apart from the first step. A slit "
                    f"in a mesh narrower than dhat does this; widen it or lower model.dhat.",
                    stacklevel=4)
        if model._gravity != (0.0, 0.0) or model._fext is not None:
            loose = [h for h in range(model.n_bodies)
                     if h not in model._constrained or len(model._constrained[h]) == 0]
            if loose and self.alpha_max < 1e3 and not self.rigid_modes:
                warnings.warn(f"a force acts on unanchored body {loose}, but alpha_max = "
                              f"{self.alpha_max:g} caps each iteration's step: its rigid motion "
                              f"will converge very slowly or not at all. Leave rigid_modes on.",
                              stacklevel=3)
        s = DeviceSolver(prob, precision=self.precision, threads=self.threads,
                         blocks_per_sm=self.blocks_per_sm, device=model.device,
                         blocks_per_scene=self.blocks_per_scene)
        s.dt = float(dt)
        s.iter_max = int(prob["iter_max"])
        s._act_version = model._act_version
        s._ctrl_version = model._ctrl_version
        model._solver = s
