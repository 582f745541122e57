"""Golden vectors from the reference's own solver code — the script that made tests/golden/*.npz.

    python tests/golden/make_golden.py /path/to/Diff_2D_FEM [scene ...]

The reference checkout is the first argument that names a directory, or else the
DIFF2DFEM_REFERENCE environment variable; there is no default.

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
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import fixture_io  # noqa: E402
import refload  # noqa: E402
import scenes  # noqa: E402


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
    order = [k for k in ("ExternalForce", "AffineBodies", "IPCContact", "Springs", "Pressure", "Tendon")
             if k in kinds]
    assert kinds == order, f"unexpected term order {kinds}"
    for t in s.terms:
        if isinstance(t, A.ExternalForce):
            prob["fext"] = _np(t.f)
        elif isinstance(t, A.Springs):
            prob["springs"] = dict(a=_np(t.na), b=_np(t.nb), k=_np(t.k), L0=_np(t.L0), anchor=_np(t.anchor),
                                   env=_np(t.s2env))
        elif isinstance(t, A.Pressure):
            prob["pressure"] = dict(ea=_np(t.ea), eb=_np(t.eb), ch=_np(t.ech), ch2env=_np(t.ch2env),
                                    p=_np(t.p), ref=_np(t.cref))
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
def run_scene(R, name):
    ns = types.SimpleNamespace(Model=R.Model, ImplicitIntegrator=R.ImplicitIntegrator, device="cpu",
                               mask_to_mesh=R.mesh.mask_to_mesh)
    sc = scenes.SCENES[name](ns)
    return record(R, sc["model"], sc["integ"], sc["dt"], sc["steps"], sc["command"], name=name)


def main(argv):
    ref = os.environ.get("DIFF2DFEM_REFERENCE")
    names = []
    for a in argv:
        if os.path.isdir(a):
            ref = a
        else:
            names.append(a)
    if not ref:
        sys.exit("give the reference checkout as an argument or in DIFF2DFEM_REFERENCE")
    R = refload.load(ref)
    for name in (names or list(scenes.SCENES)):
        t0 = time.time()
        prob, steps = run_scene(R, name)
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **fixture_io.pack(prob, steps, dict(scene=name)))
        print(f"{name}: {os.path.getsize(path) / 1024:.0f} KB in {time.time() - t0:.0f} s", flush=True)


if __name__ == "__main__":
    main(sys.argv[1:])
