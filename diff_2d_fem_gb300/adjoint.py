"""Adjoint of the implicit step: gradients of a rollout with respect to per-element stiffness,
tendon tensions and the initial state, on the GPU.

Two layers:

* `AdjointPNCG2D` mirrors the reference's class of the same name (implicit/adjoint.py:186-399):
  `set_density`, `adjoint_solve`, `drho`, `transient_adjoint`, with the same meaning. Where
  the reference runs host MINRES whose every matrix-vector product is two host-device copies,
  here each `adjoint_solve` is one kernel launch solving every scene's system on the device
  (d2f_adjoint_solve: Jacobi-preconditioned CG, one block per scene) and `drho` one launch
  (d2f_adjoint_vjp).

* `Rollout` is a differentiable T-step rollout of every scene: a `torch.autograd.Function`
  taking per-element stiffness multipliers E, a tension schedule, x0 and v0 and returning
  the positions at the recorded steps. The forward pass keeps the state every
  `checkpoint_every` steps only; the backward pass replays each segment from its checkpoint
  (the FP64 step is deterministic, so the replayed states are bit-identical) and runs the
  damped backward-Euler adjoint recursion of implicit/adjoint.py:386-398,

      H_k lam_k = dL/dx_k + (1 + drag) M lam_{k+1} - drag M lam_{k+2}
      dL/dE_e  += -h^2 lam_k . f_e(x_k) / E_e          (f_e: element force at modulus E_e)
      dL/dT_k   = -h^2 lam_k . dlen/dx(x_k)             (tension-controlled tendons, T_k > 0)
      dL/dx_0   = M lam_1 - drag M lam_2,   dL/dv_0 = h drag M lam_1   (free DOFs)

  which follows from the predictor xhat_{k+1} = x_k + h drag v_k, v_k = (x_k - x_{k-1}) / h.

The operator H_k = M + h^2 (K_elastic + K_collider + K_tendon + K_spring + K_pressure + K_ipc)
has the collider contact gate frozen at x_k, as the reference's; like the reference it leaves
out friction. Beyond the reference, which refuses them (implicit/adjoint.py:372-385): the
tangent of IPC contact between bodies (the barrier terms active at x_k, frozen, each
distance's exact Hessian), affine bodies in their reduced coordinates (x = J q on a body's
nodes, the body's exact elastic block; the solution on its nodes is J lam_q), and tendons
(tension-controlled cables).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib

try:
    import torch
except ImportError:  # pragma: no cover
    torch = None


def _solver_of(obj):
    s = getattr(obj, "_solver", None) if not hasattr(obj, "h") else obj
    if s is None:
        raise RuntimeError("the model has no solver yet: run simulate() once first")
    if s.mixed:
        raise ValueError("the adjoint needs an FP64 solver (ImplicitIntegrator(precision='fp64'))")
    _refuse_actuators(False, False, bool(s.prob.get("active_regions", 0)))
    return s


def _refuse_actuators(pressure, springs, active):
    """The reference's refusal (implicit/adjoint.py:376-385): no gradient of a different
    system for terms the adjoint operator has no tangent for."""
    missing = [nm for nm, on in (("ActiveStrain", active), ("Pressure", pressure), ("Springs", springs)) if on]
    if missing:
        raise NotImplementedError(
            f"the adjoint operator has no tangent for {', '.join(missing)}: the gradient would be "
            f"of a different system. Differentiate without these actuators.")


class AdjointPNCG2D:
    """Adjoint of the FP64 step of a DeviceSolver (or of a Model's solver).

    Density enters as in the reference (implicit/adjoint.py:1-12): per element
    mu_e = E(rho_e) mu0_e, lam_e = E(rho_e) lam0_e with E(rho) = Emin + rho (1 - Emin), mu0 and
    lam0 the moduli the solver was built with."""

    def __init__(self, solver, Emin=1e-3, model=None):
        s = _solver_of(solver)
        self._s = s
        self.model = model          # its current solver is followed: one rebuilt for a new term
        self.Emin = float(Emin)
        self.dev = s.dev
        self.N, self.n_tri, self.B = s.N, int(s.desc.T), s.B
        self.mu0 = s.tensor("mu").clone()
        self.lam0 = s.tensor("lam").clone()
        self.E = torch.ones(self.n_tri, dtype=torch.float64, device=self.dev)
        fm = s.tensor("free_mask").to(torch.int32)
        self.free = torch.stack([(fm & 1) > 0, (fm & 2) > 0], 1).to(torch.float64)
        self.mass = s.tensor("mass")
        self._work = torch.empty(int(s.L.d2f_adjoint_work_doubles(s.h)), dtype=torch.float64, device=self.dev)
        self.iters = torch.zeros(self.B, dtype=torch.int32, device=self.dev)
        self.status = torch.zeros(self.B, dtype=torch.int32, device=self.dev)
        self.worst_status = torch.zeros(self.B, dtype=torch.int32, device=self.dev)
        self.max_iters = torch.zeros(self.B, dtype=torch.int32, device=self.dev)
        self.total_iters = torch.zeros(self.B, dtype=torch.int64, device=self.dev)
        self.solves = 0

    @property
    def s(self):
        """The solver: the model's current one when built from a model (the integrator
        rebuilds it when a term is added), with this adjoint's modulus multipliers applied."""
        m = self.model
        if m is not None and m._solver is not None and m._solver is not self._s:
            self._s = _solver_of(m._solver)
            self._s.tensor("mu").copy_(self.mu0 * self.E)
            self._s.tensor("lam").copy_(self.lam0 * self.E)
        return self._s

    @property
    def h2(self):
        return float(self.s.desc.dt) ** 2

    @property
    def drag(self):
        return float(self.s.desc.drag)

    # ---- stiffness
    def set_modulus(self, E):
        """Per-element multiplier of the solver's moduli (a tensor or array of n_tri)."""
        E = torch.as_tensor(E, dtype=torch.float64, device=self.dev).reshape(self.n_tri)
        if not bool((E > 0).all()):
            raise ValueError("every element's modulus multiplier must be positive")
        self.E.copy_(E)
        self.s.tensor("mu").copy_(self.mu0 * self.E)
        self.s.tensor("lam").copy_(self.lam0 * self.E)

    def set_density(self, rho_e):
        """implicit/adjoint.py:212-215: E = Emin + rho (1 - Emin)."""
        rho = torch.as_tensor(rho_e, dtype=torch.float64, device=self.dev)
        self.set_modulus(self.Emin + rho * (1.0 - self.Emin))

    # ---- the device calls
    def _x(self, x):
        return torch.as_tensor(x, dtype=torch.float64, device=self.dev).reshape(self.N, 2).contiguous()

    def adjoint_solve(self, xk, rhs, rtol=1e-12, maxiter=20000, tension=None, guess=None):
        """Solve H(x_k) lam = rhs on the free DOFs for every scene (one launch), from `guess`
        (N, 2) if given, else from zero. Returns lam (N, 2), a device tensor; per-scene
        iterations and status in self.iters / self.status (0 converged, 1 maxiter reached,
        -4 operator not positive along a direction), the worst over all solves so far in
        self.worst_status / self.max_iters, the sum of iterations in self.total_iters."""
        xk, rhs = self._x(xk), self._x(rhs)
        if guess is not None:
            lam = self._x(guess).clone()
        else:
            lam = torch.empty((self.N, 2), dtype=torch.float64, device=self.dev)
        tp = None
        if tension is not None:
            tp = C.c_void_p(tension.data_ptr())
        _lib.check(self.s.L.d2f_adjoint_solve(self.s.h, C.c_void_p(xk.data_ptr()), C.c_void_p(rhs.data_ptr()),
                                              C.c_void_p(lam.data_ptr()), C.c_void_p(self._work.data_ptr()), tp,
                                              float(rtol), int(maxiter), int(guess is not None),
                                              C.c_void_p(self.iters.data_ptr()),
                                              C.c_void_p(self.status.data_ptr()), self.s._stream_ptr()),
                   "d2f_adjoint_solve")
        worse = (self.status.abs() > self.worst_status.abs())
        self.worst_status.copy_(torch.where(worse, self.status, self.worst_status))
        torch.maximum(self.max_iters, self.iters, out=self.max_iters)
        self.total_iters += self.iters.to(torch.int64)
        self.solves += 1
        return lam

    def vjp(self, xk, lam, dscale, dtension=None):
        """dscale += -h^2 lam . f_e(x_k) at the current moduli; dtension (n_ten, device order)
        = -h^2 lam . dlen/dx."""
        xk, lam = self._x(xk), self._x(lam)
        dt_ = C.c_void_p(dtension.data_ptr()) if dtension is not None else None
        _lib.check(self.s.L.d2f_adjoint_vjp(self.s.h, C.c_void_p(xk.data_ptr()), C.c_void_p(lam.data_ptr()),
                                            C.c_void_p(dscale.data_ptr()), dt_, self.s._stream_ptr()),
                   "d2f_adjoint_vjp")

    def dpressure(self, xk, lam, out=None):
        """dL/dp of every chamber (model order) for one step: the product of lam (from
        adjoint_solve at x_k) with the step residual's derivative in each chamber's pressure.
        Added into `out` (n_ch, device) if given; returned."""
        n_ch = int(self.s.desc.n_ch)
        if out is None:
            out = torch.zeros(n_ch, dtype=torch.float64, device=self.dev)
        if n_ch:
            xk, lam = self._x(xk), self._x(lam)
            _lib.check(self.s.L.d2f_adjoint_vjp_pressure(self.s.h, C.c_void_p(xk.data_ptr()), C.c_void_p(lam.data_ptr()),
                                                         C.c_void_p(out.data_ptr()), self.s._stream_ptr()),
                       "d2f_adjoint_vjp_pressure")
        return out

    def drho(self, xk, lam):
        """implicit/adjoint.py:277-283: -(1 - Emin) lam . [h^2 f_e(x_k)] at full density."""
        d = torch.zeros(self.n_tri, dtype=torch.float64, device=self.dev)
        self.vjp(xk, lam, d)
        return d / self.E * (1.0 - self.Emin)

    def transient_adjoint(self, xs, seed, drag=None, rtol=1e-12, maxiter=20000, warm_start=True):
        """implicit/adjoint.py:371-399. xs = [x_0 .. x_T] (the forward states, arrays or
        tensors (N, 2)), seed = {k: dJ/dx_k (N, 2)}. Returns dJ/drho (n_tri,) as a device
        tensor, accumulated over the trajectory."""
        # the operator has the springs' and chambers' tangents at their current commands, but a
        # trajectory may have changed those commands step by step: refused as the reference does
        m = self.model
        if m is not None:
            _refuse_actuators(bool(m._chambers), bool(m._springs), bool(m._regions))
            self.s                  # the model's current solver
        _refuse_actuators(self.s.desc.n_pe > 0, self.s.desc.n_sp > 0, False)
        T = len(xs) - 1
        dr = self.drag if drag is None else float(drag)
        m2 = self.mass[:, None]
        lam1 = torch.zeros((self.N, 2), dtype=torch.float64, device=self.dev)
        lam2 = torch.zeros_like(lam1)
        g = torch.zeros(self.n_tri, dtype=torch.float64, device=self.dev)
        for k in range(T, 0, -1):
            rhs = (1.0 + dr) * m2 * lam1 - dr * m2 * lam2
            if k in seed:
                rhs = rhs + self._x(seed[k])
            lam = self.adjoint_solve(xs[k], rhs, rtol=rtol, maxiter=maxiter,
                                     guess=lam1 if (warm_start and k < T) else None)
            self.vjp(xs[k], lam, g)
            lam2, lam1 = lam1, lam
        return g / self.E * (1.0 - self.Emin)


class _RolloutFn(torch.autograd.Function if torch is not None else object):
    @staticmethod
    def forward(ctx, E, tension, x0, v0, ro):
        ro._forward(E, tension, x0, v0)
        ctx.ro = ro
        return ro._out.clone()

    @staticmethod
    def backward(ctx, g_out):
        dE, dT, dx0, dv0 = ctx.ro._backward(g_out)
        return dE, dT, dx0, dv0, None


class Rollout:
    """A differentiable rollout of `steps` implicit steps of every scene of an FP64 solver.

        ro = Rollout(model, steps=20, record=[20], checkpoint_every=5)
        x = ro(E, tension, x0, v0)          # (len(record), N, 2), differentiable
        loss(x).backward()                  # gradients to E, tension, x0, v0

    E: (n_tri,) per-element multipliers of the solver's moduli. tension: (steps, n_tendons)
    tension commands per step, in the model's tendon order (tension-controlled tendons), or
    None when the model has no tendon. x0, v0: (N, 2) initial state. `targets`, if given, is
    (steps, N, 2) kinematic targets per step (not differentiated; held DOFs carry no
    gradient). After a call, `info` has the forward's per-step convergence and the adjoint
    solves' worst status.

    forward_precision="mixed" runs the forward steps and their replay with the mixed-precision
    step (a second solver on the same problem) and linearises the FP64 adjoint at those states;
    the replay then reproduces the forward to FP32 rounding of its tendon atomics instead of bit
    for bit."""

    def __init__(self, solver, steps, record=None, checkpoint_every=8, rtol=1e-12, max_iter=20000,
                 targets=None, Emin=1e-3, warm_start=True, forward_precision="fp64"):
        self.adj = AdjointPNCG2D(solver, Emin=Emin)
        self.s = self.adj.s
        if forward_precision not in ("fp64", "mixed"):
            raise ValueError("forward_precision must be 'fp64' or 'mixed'")
        if forward_precision == "mixed":
            from .device import DeviceSolver
            self.fs = DeviceSolver(self.s.prob, precision="mixed", threads=self.s.desc.threads,
                                   blocks_per_sm=self.s.desc.blocks_per_sm, device=self.s.dev, stream=self.s.stream)
            self._fmu0 = self.fs.tensor("mu").clone()
            self._flam0 = self.fs.tensor("lam").clone()
        else:
            self.fs = self.s
        self.steps = int(steps)
        if self.steps < 1:
            raise ValueError("steps must be >= 1")
        self.record = sorted({int(k) for k in (record if record is not None else [self.steps])})
        if not all(1 <= k <= self.steps for k in self.record):
            raise ValueError("recorded steps must lie in 1..steps")
        self.K = max(1, int(checkpoint_every))
        self.rtol, self.max_iter = float(rtol), int(max_iter)
        self.warm_start = bool(warm_start)
        self.targets = targets
        td = self.s.td
        self.n_ten = 0 if td is None else len(td["t2env"])
        if td is not None and np.any(np.asarray(td["stiff"]) > 0):
            raise NotImplementedError("length-controlled tendons have no tension input to differentiate; "
                                      "use tension-controlled tendons (stiffness=None)")
        self.ten_order = None if td is None else torch.as_tensor(self.s.ten_order, device=self.s.dev)
        self.info = {}

    def __call__(self, E, tension, x0, v0):
        if tension is None:
            tension = torch.zeros((self.steps, self.n_ten), dtype=torch.float64, device=self.s.dev)
        return _RolloutFn.apply(E, tension, x0, v0, self)

    # ---- helpers
    def _set_step_commands(self, k, tension):
        """Commands of step k (0-based), on the forward solver."""
        if self.n_ten:
            self.fs.tensor("t_Tcmd").copy_(tension[k][self.ten_order])
        if self.targets is not None:
            self.fs.set_targets(np.asarray(self.targets[k]))

    def _load_state(self, x, v):
        self.fs.x.copy_(x)
        self.fs.v.copy_(v)

    def _set_modulus(self, E):
        self.adj.set_modulus(E)
        if self.fs is not self.s:
            self.fs.tensor("mu").copy_(self._fmu0 * E.to(self._fmu0.dtype))
            self.fs.tensor("lam").copy_(self._flam0 * E.to(self._flam0.dtype))

    def close(self):
        if self.fs is not self.s:
            self.fs.close()

    def _forward(self, E, tension, x0, v0):
        s, dev = self.fs, self.s.dev
        f64 = torch.float64
        self._E = E.detach().to(dev, f64).contiguous()
        self._tension = tension.detach().to(dev, f64).reshape(self.steps, self.n_ten).contiguous()
        self._set_modulus(self._E)
        x = x0.detach().to(dev, f64).reshape(s.N, 2)
        v = v0.detach().to(dev, f64).reshape(s.N, 2)
        self._ckpt = {0: (x.clone(), v.clone())}
        self._load_state(x, v)
        out = torch.empty((len(self.record), s.N, 2), dtype=f64, device=dev)
        rec = {k: i for i, k in enumerate(self.record)}
        unconv = torch.zeros(s.B, dtype=torch.int32, device=dev)
        bad = torch.zeros(s.B, dtype=torch.int32, device=dev)
        for k in range(1, self.steps + 1):
            self._set_step_commands(k - 1, self._tension)
            s.step()
            unconv += s.tensor("active")
            bad |= (s.tensor("status") != 0).to(torch.int32)
            if k in rec:
                out[rec[k]].copy_(s.x)
            if k % self.K == 0 and k < self.steps:
                self._ckpt[k] = (s.x.clone(), s.v.clone())
        self._final = (s.x.clone(), s.v.clone())
        self._out = out
        self.info = dict(forward_unconverged_steps=unconv.cpu().numpy(), forward_error=bad.cpu().numpy())

    def _backward(self, g_out):
        s, adj, dev = self.fs, self.adj, self.s.dev
        f64 = torch.float64
        N, K = s.N, self.K
        g = {k: g_out[i].to(dev, f64).contiguous() for i, k in enumerate(self.record)}
        dr = adj.drag
        h = float(s.desc.dt)
        m2 = adj.mass[:, None]
        lam1 = torch.zeros((N, 2), dtype=f64, device=dev)
        lam2 = torch.zeros_like(lam1)
        dscale = torch.zeros(adj.n_tri, dtype=f64, device=dev)
        dT_dev = torch.zeros((self.steps, max(self.n_ten, 1)), dtype=f64, device=dev)
        adj.worst_status.zero_()
        adj.max_iters.zero_()
        adj.total_iters.zero_()
        self._set_modulus(self._E)
        replay_mismatch = 0.0
        for c in reversed(range(0, self.steps, K)):
            e = min(c + K, self.steps)
            self._load_state(*self._ckpt[c])
            xs = []
            for k in range(c + 1, e + 1):
                self._set_step_commands(k - 1, self._tension)
                s.step()
                xs.append(s.x.clone())
            if e in self._ckpt:
                replay_mismatch = max(replay_mismatch, float((xs[-1] - self._ckpt[e][0]).abs().max()))
            for k in range(e, c, -1):
                xk = xs[k - c - 1]
                rhs = (1.0 + dr) * m2 * lam1 - dr * m2 * lam2
                if k in g:
                    rhs = rhs + g[k]
                tens = self._tension[k - 1][self.ten_order].contiguous() if self.n_ten else None
                warm = self.warm_start and k < self.steps
                lam = adj.adjoint_solve(xk, rhs, rtol=self.rtol, maxiter=self.max_iter, tension=tens,
                                        guess=lam1 if warm else None)
                adj.vjp(xk, lam, dscale, dT_dev[k - 1] if self.n_ten else None)
                lam2, lam1 = lam1, lam
        self._load_state(*self._final)
        dE = dscale / self._E
        dT = None
        if self.n_ten:
            dT = torch.zeros((self.steps, self.n_ten), dtype=f64, device=dev)
            dT[:, self.ten_order] = dT_dev
            dT = dT * (self._tension > 0)
        dx0 = (m2 * lam1 - dr * m2 * lam2) * adj.free
        dv0 = (h * dr) * m2 * lam1 * adj.free
        self.info.update(adjoint_worst_status=adj.worst_status.cpu().numpy(),
                         adjoint_max_iters=adj.max_iters.cpu().numpy(),
                         adjoint_total_iters=adj.total_iters.cpu().numpy(), replay_mismatch=replay_mismatch)
        return dE, dT, dx0, dv0
