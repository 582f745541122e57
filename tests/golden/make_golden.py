"""Golden vectors from the reference's own solver code — the script that made tests/golden/*.npz.

    python tests/golden/make_golden.py [/path/to/Diff_2D_FEM] [scene ...]

Each scene is built with the reference's own Model and ImplicitIntegrator, executed by the
serial Warp stand-in in warp_shim.py (the reference's kernel source runs unchanged, in
Python, with Warp's CPU semantics). Recorded per scene:

  * the solver problem exactly as the reference builds it (every array the reference's
    PNCG2DSolver holds after ImplicitIntegrator.attach, plus its terms and modes), in the
    problem-dict layout the oracle and the CUDA path consume;
  * per step, the commands issued (kinematic targets, tendon tension) and the results
    (node positions and velocities, iterations, convergence flags, affine q).

The scenes are small (a few hundred nodes, a few steps): pure Python is slow.
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import fixture_io  # noqa: E402
import refload  # noqa: E402


# ----------------------------------------------------------------------------- extraction
def _np(a):
    return np.asarray(a.numpy())


def extract_problem(R, model, s):
    """The reference solver `s` (after attach) as a problem dict."""
    A = R.actuation
    prob = dict(
        B=int(s.B), x=_np(s.x), v=_np(s.v), mass=_np(s.mass), free=_np(s.free),
        node2env=_np(s.node2env).astype(np.int32), tri=_np(s.tri).astype(np.int32),
        Bm=_np(s.Bm), area=_np(s.area), mu=_np(s.mu), lam=_np(s.lam),
        tri2env=_np(s.tri2env).astype(np.int32), bnd=_np(s.bnd).astype(np.int32),
        b2e=_np(s.b2e).astype(np.int32), bc_idx=_np(s.bc_idx).astype(np.int32),
        colliders=np.array([[c["kind"], c["cx"], c["cy"], c["rx"], c["ry"], c["rref"],
                             c.get("r", c["rx"]), c["mu"]] for c in s.colliders],
                           np.float64).reshape(-1, 8),
        dt=s.dt, drag=s.drag, dhat=s.dhat, kappa=s.kappa, epsv=s.epsv, eps=s.eps,
        tol_x=s.tol_x, near_factor=s.near_factor, alpha_max=s.alpha_max,
        area_shrink=s.area_shrink, ccd_eta=s.ccd_eta, cg_guard=s.cg_guard, ls_tol=s.ls_tol,
        gtol=0.0, iter_max=s.iter_max, conv_check=s.conv_check, friction=int(s.friction),
        line_search=int(s.line_search), n_bt=s.n_bt)
    assert s.self_stiffness == 0.0, "the 'node' contact is out of scope"
    # terms, in the reference's order
    kinds = [type(t).__name__ for t in s.terms]
    order = [k for k in ("ExternalForce", "AffineBodies", "IPCContact", "Tendon") if k in kinds]
    assert kinds == order, f"unexpected term order {kinds}"
    for t in s.terms:
        if isinstance(t, A.ExternalForce):
            prob["fext"] = _np(t.f)
        elif isinstance(t, A.Tendon):
            prob["tendon"] = dict(node=_np(t.node), prv=_np(t.prv), nxt=_np(t.nxt), tid=_np(t.tid),
                                  t2env=_np(t.t2env), stiff=_np(t.stiff), L0=_np(t.L0),
                                  Tcmd=_np(t.Tcmd))
    if s.ipc is not None:
        ip = s.ipc
        excl = _np(ip.excl).astype(np.uint8)
        off = _np(ip.excl_off)
        bpe = _np(ip.bpe)
        ptr, idx = [0], []
        for e in range(s.B):
            n = int(bpe[e])
            M = excl[int(off[e]):int(off[e]) + n * n].reshape(n, n)
            for r in range(n):
                nz = np.nonzero(M[r])[0]
                idx.extend(nz.tolist())
                ptr.append(ptr[-1] + len(nz))
        prob["ipc"] = dict(ea=_np(ip.ea), eb=_np(ip.eb), ela=_np(ip.ela), elb=_np(ip.elb),
                           e2env=_np(ip.e2env), ca=_np(ip.ca), cb=_np(ip.cb),
                           bstart=_np(ip.bstart), bpe=bpe,
                           excl_ptr=np.asarray(ptr, np.int32), excl_idx=np.asarray(idx, np.int32),
                           mu=ip.mu, per_body=ip.per_body,
                           mu_node=(_np(ip.mu_node) if ip.per_body else None),
                           dhat=ip.dhat, kappa=ip.kappa, reach=ip.reach, gap=ip.gap,
                           bc_floor=ip.bc_floor)
    modes = [type(m).__name__ for m in s.modes]
    assert modes in ([], ["AffineBodies"], ["RigidModes"], ["AffineBodies", "RigidModes"]), modes
    for m in s.modes:
        if type(m).__name__ == "AffineBodies":
            prob["affine"] = dict(node=_np(m.node), grp=_np(m.grp), env=_np(m.env), w=_np(m.w),
                                  Mu=_np(m.Mu), La=_np(m.La), q=_np(m.q))
        else:
            prob["rigid"] = dict(node=_np(m.node), grp=_np(m.grp), env=_np(m.env))
    return prob


def record(R, model, integ, dt, n_steps, command=None, name=""):
    s = integ.attach(model, dt)
    if command is not None:
        command(0)
        s = integ.attach(model, dt)
    prob = extract_problem(R, model, s)
    steps = []
    t0 = time.time()
    for k in range(n_steps):
        if command is not None and k > 0:
            command(k)
        s = integ.attach(model, dt)
        cmd = {}
        if len(prob["bc_idx"]):
            cmd["bc_target"] = np.asarray(model._targets, np.float64)[prob["bc_idx"]]
        if s._act.get("tendon") is not None:
            cmd["Tcmd"] = _np(s._act["tendon"].Tcmd)
        integ.simulate(model, dt)
        st = integ.stats(model)
        out = dict(cmd)
        out.update(x=_np(s.x), v=_np(s.v), iters=np.asarray(st["iters"]),
                   active=_np(s.active))
        if s.affine is not None:
            out["q"] = _np(s.affine.q)
        steps.append(out)
        print(f"  {name} step {k}: iters {st['iters'].tolist()}  ({time.time() - t0:.1f} s)", flush=True)
    return prob, steps


# ----------------------------------------------------------------------------- scenes
def scene_strip_small(R):
    m = R.Model(device="cpu")
    m.add_ground(0.0, mu=0.8)
    m.add_soft_body(np.ones((3, 12), np.uint8), physical_size=(0.009, 0.00225), center=(0.0, 0.0013),
                    E=0.5e6, nu=0.40, density=1100.0)
    m.finalize(); m.gravity = (0.0, -9.81)
    return record(R, m, R.ImplicitIntegrator(), 2e-3, 4, name="strip_small")


def scene_strip_cfg1(R):
    """The strip on the ground of the headline single-scene configuration, first steps."""
    m = R.Model(device="cpu")
    m.add_ground(0.0, mu=0.8)
    m.add_soft_body(np.ones((6, 72), np.uint8), physical_size=(0.054, 0.0045), center=(0.0, 0.0030),
                    E=0.5e6, nu=0.40, density=1100.0)
    m.finalize(); m.gravity = (0.0, -9.81)
    return record(R, m, R.ImplicitIntegrator(), 2e-3, 2, name="strip_cfg1")


def scene_batch_colliders(R):
    """Three environments with different designs pressed by kinematic top rows onto a disc,
    an ellipse, a rounded box and a rounded triangle; friction on; IPC self-contact sweeps
    the kinematic nodes."""
    rng = np.random.default_rng(3)
    d1 = np.ones((6, 4), np.uint8); d1[2:4, 1:3] = 0
    d2 = (rng.random((6, 4)) > 0.15).astype(np.uint8); d2[-1] = 1; d2[:, 0] = 1
    m = R.Model(device="cpu")
    m.add_disc(center=(0.0, 0.0), radius=0.004, mu=0.6)
    m.add_object("ellipse", (0.006, 0.001), 0.002, 0.001, mu=0.3)
    m.add_object("box", (-0.006, 0.001), 0.0015, 0.001, corner_radius=0.0004, mu=0.5)
    m.add_object("triangle", (0.0, -0.008), 0.002, corner_radius=0.0003, mu=0.4)
    hs = [m.add_soft_body(d, physical_size=(0.004, 0.006), center=(0.0, 0.0072), E=1.0e6, nu=0.40,
                          density=1100.0, env_id=i) for i, d in enumerate([d1, d2, d1])]
    m.finalize()
    x0 = [m.rest_x(h) for h in hs]
    tops = [np.where(x[:, 1] > x[:, 1].max() - 1e-9)[0] for x in x0]
    for h, t in zip(hs, tops):
        m.set_kinematic_constraint(h, t)
    integ = R.ImplicitIntegrator(max_iter=60)

    def command(k):
        for h, x, t in zip(hs, x0, tops):
            tgt = x.copy(); tgt[t, 1] -= 0.0012 * (k + 1) / 4
            m.set_kinematic_target(h, tgt)
    return record(R, m, integ, 1e-3, 4, command, name="batch_colliders")


def scene_grip(R):
    """Two soft pads with kinematic backs close on a free rigid block above the ground:
    IPC contact between bodies with friction, an affine body, kinematic sweeps."""
    PX = 0.5e-3
    m = R.Model(device="cpu")
    m.body_friction = 0.8
    m.add_ground(0.0, mu=0.5)
    m.add_affine_body(np.ones((4, 4), np.uint8), physical_size=(4 * PX, 4 * PX),
                      center=(0.0, 2 * PX + 0.9 * PX / 8), density=600.0)
    pads = [m.add_soft_body(np.ones((4, 2), np.uint8), physical_size=(2 * PX, 4 * PX),
                            center=(s * 3.25 * PX, 2 * PX + 0.4e-3), E=1.0e6, nu=0.40, density=1100.0)
            for s in (-1, +1)]
    m.finalize(); m.gravity = (0.0, -9.81)
    rest = [m.rest_x(p) for p in pads]
    for s, p, X in zip((-1, +1), pads, rest):
        back = X[:, 0].min() if s < 0 else X[:, 0].max()
        m.set_kinematic_constraint(p, np.where(np.abs(X[:, 0] - back) < 1e-9)[0])

    def command(k):
        a = min((k + 1) / 4.0, 1.0)
        for s, p, X in zip((-1, +1), pads, rest):
            Y = X.copy(); Y[:, 0] -= s * 0.35 * PX * a
            m.set_kinematic_target(p, Y)
    return record(R, m, R.ImplicitIntegrator(max_iter=120), 1e-3, 5, command, name="grip")


def scene_tendon(R):
    """A cantilever clamped at its left end and bent by a tension-controlled tendon."""
    m = R.Model(device="cpu"); m.damping = 50.0
    h = m.add_soft_body(np.ones((3, 16), np.uint8), physical_size=(0.008, 0.0015), center=(0.0, 0.0),
                        E=1.0e6, nu=0.40, density=1100.0)
    m.finalize()
    X = m.rest_x(h)
    m.set_kinematic_constraint(h, np.where(X[:, 0] < X[:, 0].min() + 1e-9)[0])
    cable = m.add_tendon(h, through=[(x, 0.0005) for x in np.unique(np.round(X[:, 0], 9))])
    integ = R.ImplicitIntegrator(self_collision=False, friction=False, max_iter=80)

    def command(k):
        m.set_tendon_tension(cable, 5.0 + 5.0 * k)
    return record(R, m, integ, 1e-3, 4, command, name="tendon")


def scene_line_search(R):
    """The energy line search, on a soft block dropped on a disc collider, no rigid modes."""
    m = R.Model(device="cpu")
    m.add_disc(center=(0.0, -0.004), radius=0.004, mu=0.5)
    m.add_soft_body(np.ones((3, 4), np.uint8), physical_size=(0.002, 0.0015), center=(0.0002, 0.0008),
                    E=0.5e6, nu=0.40, density=1100.0)
    m.finalize(); m.gravity = (0.0, -9.81)
    integ = R.ImplicitIntegrator(line_search=True, rigid_modes=False, max_iter=50)
    return record(R, m, integ, 2e-3, 4, name="line_search")


SCENES = {
    "strip_small": scene_strip_small,
    "batch_colliders": scene_batch_colliders,
    "grip": scene_grip,
    "tendon": scene_tendon,
    "line_search": scene_line_search,
    "strip_cfg1": scene_strip_cfg1,
}


def main(argv):
    ref = "/root/reference"
    names = []
    for a in argv:
        if os.path.isdir(a):
            ref = a
        else:
            names.append(a)
    R = refload.load(ref)
    for name in (names or list(SCENES)):
        t0 = time.time()
        prob, steps = SCENES[name](R)
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **fixture_io.pack(prob, steps, dict(scene=name)))
        print(f"{name}: {os.path.getsize(path) / 1024:.0f} KB in {time.time() - t0:.0f} s", flush=True)


if __name__ == "__main__":
    main(sys.argv[1:])
