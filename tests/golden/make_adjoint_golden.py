"""Golden vectors of the reference's adjoint — the script that made tests/golden/adjoint_*.npz.

    python tests/golden/make_adjoint_golden.py /path/to/Diff_2D_FEM

(or the checkout in the DIFF2DFEM_REFERENCE environment variable; there is no default)

Runs the reference's own forward solve and its AdjointPNCG2D.transient_adjoint
(implicit/adjoint.py:371-399) on the serial Warp stand-in (warp_shim.py), on a scene the
reference's adjoint covers: a soft block, its top row held and swept down and sideways,
pressed onto a frictionless disc collider, with a non-uniform density field. The objective
is J = w . x_T for a fixed weight field w (the mean sideways position of the lower half).
Recorded: the solver problem at full density, the kinematic targets per step, the density
field, Emin, the forward states x_0..x_T, the seed dJ/dx_T and the reference's dJ/drho.

TEST INFRASTRUCTURE ONLY. Pure Python is slow: the scene is small.
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
from make_golden import extract_problem  # noqa: E402


def press_disc(R, steps=4, dt=2.0e-4, seed=0):
    m = R.Model(device="cpu")
    m.add_disc(center=(0.0, -0.0040), radius=0.004, mu=0.0)
    h = m.add_soft_body(np.ones((5, 4), np.uint8), physical_size=(0.004, 0.005), center=(0.0, 0.0027),
                        E=1.0e6, nu=0.40, density=1100.0)
    m.finalize()
    x0 = m.get_body_x(h)
    top = np.where(x0[:, 1] > x0[:, 1].max() - 1e-9)[0]
    m.set_kinematic_constraint(h, top)
    integ = R.ImplicitIntegrator(max_iter=3000, eps=1e-14, tol_x=0.0, conv_check=8,
                                 self_collision=False, friction=False)
    Emin = 1e-3
    adj = integ.adjoint(m, dt, Emin=Emin)
    s = integ.attach(m, dt)
    prob = extract_problem(R, m, s)            # full-density moduli (before set_density)
    rng = np.random.default_rng(seed)
    rho = 0.45 + 0.5 * rng.random(adj.n_tri)
    adj.set_density(rho)
    lower = np.where(x0[:, 1] < np.median(x0[:, 1]))[0]
    w = np.zeros((prob["x"].shape[0], 2))
    w[lower, 0] = 1.0 / len(lower)
    xs = [np.asarray(m.get_x(), np.float64)]
    targets = []
    t0 = time.time()
    for k in range(1, steps + 1):
        x = m.get_body_x(h)
        x[top, 1] = x0[top, 1] - 0.0012 * k / steps
        x[top, 0] = x0[top, 0] + 0.0006 * k / steps
        m.set_kinematic_target(h, x)
        targets.append(np.asarray(m._targets, np.float64)[prob["bc_idx"]])
        integ.simulate(m, dt)
        xs.append(np.asarray(m.get_x(), np.float64))
        print(f"  step {k}: iters {integ.stats(m)['iters'].tolist()}  ({time.time() - t0:.1f} s)", flush=True)
    g = adj.transient_adjoint(xs, seed={steps: w}, use_disc=True, rtol=1e-13, maxiter=20000)
    print(f"  adjoint: {adj.minres_calls} MINRES solves, {getattr(adj, 'minres_fail', 0)} not converged "
          f"({time.time() - t0:.1f} s)", flush=True)
    steps_rec = [dict(bc_target=targets[k], x=xs[k + 1]) for k in range(steps)]
    meta = dict(scene="press_disc", rho=rho, Emin=Emin, seed_w=w, x0=xs[0], dJdrho=np.asarray(g, np.float64),
                minres_fail=int(getattr(adj, "minres_fail", 0)))
    return prob, steps_rec, meta


def main(argv):
    ref = argv[0] if argv else os.environ.get("DIFF2DFEM_REFERENCE")
    if not ref:
        sys.exit("give the reference checkout as an argument or in DIFF2DFEM_REFERENCE")
    R = refload.load(ref)
    t0 = time.time()
    prob, steps, meta = press_disc(R)
    path = os.path.join(HERE, "adjoint_press_disc.npz")
    np.savez_compressed(path, **fixture_io.pack(prob, steps, meta))
    print(f"adjoint_press_disc: {os.path.getsize(path) / 1024:.0f} KB in {time.time() - t0:.0f} s", flush=True)


if __name__ == "__main__":
    main(sys.argv[1:])
