"""Batched implicit-step throughput: scene-steps/s of the PNCG step on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--scenes 4096] [--precision mixed|fp64]

Workload: the batching configuration — 4096 independent soft rectangles on the ground
(H ~ U{4..16}, W ~ U{32..128} pixels of 0.75 mm, per-pixel E log-uniform in [0.1, 2] MPa,
nu 0.40, density 1100, ground mu ~ U[0.3, 0.9] per scene, top-edge pressure ~ U[0, 5] kPa,
dt 2 ms, relative gradient-norm tolerance 1e-6), seeded synthetic inputs. One step = one
implicit step of every scene. The headline arm is the mixed-precision path; the plain FP64
path is timed on the same batch and reported beside it, with the position error between
the two after the timed steps.

`value` times K steps with the state resident in HBM (CUDA events on the launching
stream); `e2e` times the same steps through the public API (ImplicitIntegrator.simulate)
with the step's nodal loads uploaded from pinned host memory and the node positions read
back every step. `--impl reference` times the reference algorithm's CPU implementation:
the reference itself needs NVIDIA Warp, which is not installable here, so its serial FP64
restatement (oracle/) runs on the host cores, one thread per scene sample.
Multi-GPU (torchrun): replicas only — each rank advances its own batch, no exchange.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

HBM_FALLBACK_GBS = 6800.0


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": HBM_FALLBACK_GBS, "sm_max_mhz": 2070.0}, "fallback"


class Clocks:
    """nvidia-smi sampled every 200 ms while the timed region runs."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu=0):
        self.gpu, self.rows, self.stop = gpu, [], threading.Event()

    def _run(self):
        while not self.stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                     timeout=5).stdout.strip()
                if out:
                    self.rows.append([c.strip() for c in out.split(",")])
            except Exception:
                pass
            self.stop.wait(0.2)

    def __enter__(self):
        self.t = threading.Thread(target=self._run, daemon=True)
        self.t.start()
        return self

    def __exit__(self, *a):
        self.stop.set()
        self.t.join(timeout=10)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in self.rows for n, v in zip(names, r[5:9]) if v.strip().lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def algorithmic_bytes(prob, iters, mixed):
    """Compulsory bytes of one step at the iteration counts run: per iteration,
    136 T + 216 N + 88 Nb bytes (FP64) or 80 T + 144 N + 72 Nb (mixed) per scene."""
    B = int(prob["B"])
    n = np.bincount(np.asarray(prob["node2env"]), minlength=B)
    t = np.bincount(np.asarray(prob["tri2env"]), minlength=B)
    b = np.bincount(np.asarray(prob["b2e"]), minlength=B)
    per = (80 * t + 144 * n + 72 * b) if mixed else (136 * t + 216 * n + 88 * b)
    return float((np.asarray(iters, np.float64) * per).sum())


# DRAM traffic of the step kernel per scene-iteration: dram__bytes_read.sum +
# dram__bytes_write.sum of one ncu capture of one step of 608 scenes of this workload (after
# one warm-up step), divided by that step's scene-iterations, keyed by (precision, launch
# shape): the resident scenes' working set, and so the L2 hit rate, depends on the blocks per
# SM. A launch's traffic is this times its scene-iterations (traffic grows with the
# iterations each scene runs); a launch shape without a capture reports none.
TRAFFIC_PER_SCENE_ITER = {
    ("mixed", "256x2"): (2.329572352e9 + 2.059303424e9) / (608 * 239.94572368421052),
    ("fp64", "256x2"): (82.794049792e9 + 60.314018048e9) / (608 * 239.94078947368422),
}


# FP64 operations of the plain FP64 step kernel per PNCG iteration, counted from its source
# (adds, subtracts, multiplies and divides; a fused multiply-add counts two; log and sqrt one
# each; compares and min/max none):
#   per triangle: gradient and Jacobi-diagonal pass 115, curvature and inversion-cap pass 83,
#                 the nodes' gather of its three corner sums 12
#   per node:     inertia 4, mask and the five Dai-Kou dot products 32, direction, p^T M p and
#                 |p| 15, position update 4
# The boundary nodes' collider terms add a few more per boundary node and are left out.
FP64_OPS_PER_TRI_ITER = 115 + 83 + 12
FP64_OPS_PER_NODE_ITER = 4 + 32 + 15 + 4


def fp64_ops(prob, iters):
    """Counted FP64 operations of one FP64 step at the iteration counts run."""
    B = int(prob["B"])
    n = np.bincount(np.asarray(prob["node2env"]), minlength=B)
    t = np.bincount(np.asarray(prob["tri2env"]), minlength=B)
    return float((np.asarray(iters, np.float64) * (FP64_OPS_PER_TRI_ITER * t + FP64_OPS_PER_NODE_ITER * n)).sum())


def fp64_peak(dev, n=4096, reps=5):
    """Measured FP64 rate of this GPU: cuBLAS DGEMM (torch.matmul on float64, n^3), best of
    `reps`, in TFLOP/s."""
    import torch
    a = torch.randn(n, n, dtype=torch.float64, device=dev)
    b = torch.randn(n, n, dtype=torch.float64, device=dev)
    torch.matmul(a, b)
    torch.cuda.synchronize(dev)
    best = float("inf")
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize(dev)
        best = min(best, e0.elapsed_time(e1) / 1e3)
    del a, b
    torch.cuda.empty_cache()
    return 2.0 * n ** 3 / best / 1e12


# ----------------------------------------------------------------------------- CPU baseline
def cpu_sample(prob, state_x, state_v, n_threads, per_thread, seed=1):
    """The serial FP64 oracle on a bounded sample: n_threads threads, each advancing its own
    subset of `per_thread` scenes by one step from the given state. Returns
    (scene-steps/s over all threads, sample description)."""
    import oracle
    from diff_2d_fem_gb300.scene import subset_problem
    rng = np.random.default_rng(seed)
    B = int(prob["B"])
    picks = rng.choice(B, size=min(B, n_threads * per_thread), replace=False)
    groups = [np.sort(picks[i::n_threads]) for i in range(n_threads)]
    full = dict(prob)
    if state_x is not None:
        full["x"], full["v"] = state_x, state_v
    solvers = [oracle.OracleSolver(subset_problem(full, g)) for g in groups if len(g)]
    t0 = time.perf_counter()
    th = [threading.Thread(target=s.step) for s in solvers]
    for t in th:
        t.start()
    for t in th:
        t.join()
    dt = time.perf_counter() - t0
    n = sum(len(g) for g in groups)
    return n / dt, f"{n} of {B} scenes x 1 step, {len(solvers)} threads x {per_thread} scenes, {dt:.1f} s"


def _reference_status():
    """Whether the reference installed under baseline/_ref imports here (it needs warp-lang)."""
    ref = os.path.join(os.path.dirname(os.path.abspath(__file__)), "baseline", "_ref")
    if not os.path.isdir(os.path.join(ref, "Diff_2D_FEM")):
        return "reference not installed under baseline/_ref"
    import importlib.util
    if importlib.util.find_spec("warp") is None:
        return "reference installed under baseline/_ref but not importable (warp-lang absent on this box)"
    return "warp-lang present, but the reference's CPU path is not wired into this arm"


def run_reference(args, rank, world):
    if rank != 0:
        return
    from diff_2d_fem_gb300 import workloads, scene, ImplicitIntegrator
    m, kw, dt = workloads.rectangles_on_ground(args.scenes, seed=0)
    prob = scene.solver_problem(m, ImplicitIntegrator(**kw), dt)
    threads = min(os.cpu_count() or 1, 64)
    vals = []
    desc = ""
    for k in range(args.warmup + args.steps):
        v, desc = cpu_sample(prob, None, None, threads, 2, seed=k)
        if k >= args.warmup:
            vals.append(v)
    val = float(np.mean(vals))
    print(json.dumps({
        "metric": "batched scene-steps/s (implicit PNCG step)", "value": val, "unit": "scene-steps/s",
        "impl": "reference", "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded)", "config": {"workload": f"rectangles_on_ground x{args.scenes}", "dt": dt},
        "cpu_baseline": {"value": val, "unit": "scene-steps/s", "cores": threads, "kind": "port",
                         "sample": desc + "; " + _reference_status() + ", so this times the oracle port "
                                          "(the reference's step restated serially in C)"},
        "e2e": {"value": val, "unit": "scene-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))


# ----------------------------------------------------------------------------- gradients
def _grads_at(args, dev, arms, max_iter=None, eps=None, fd_entries=32, h=1e-3, stencil=2, warm=True):
    """One gradient of the differentiation workload (`arms` tendon-driven arms, the loss
    sum_b |x_tip,b - target_b|^2 after `grad_steps` steps) by the checkpointed adjoint
    (checkpoints every 10 steps), timed with CUDA events (after a short warm-up rollout when
    `warm`), and its accuracy at the same settings: `fd_entries` entries (3/4 pixel moduli,
    1/4 step tensions), each in its own arm, perturbed relative by +/- h (stencil 2: central
    differences) or also +/- 2h (stencil 4: (8 (L(h) - L(-h)) - (L(2h) - L(-2h))) / 12h, error
    O(h^4)) and +/- 3h (stencil 6: (45 D1 - 9 D2 + D3) / 60h with Dk = L(kh) - L(-kh), error
    O(h^6)) in more rollouts of the whole batch (arms are independent), against the adjoint
    gradient, relative to the entry or to 1 % of the largest checked entry for smaller ones.
    The forward steps and their replay run in mixed precision, the adjoint solves in FP64 at
    those states. max_iter / eps: the forward's iteration budget and energy-decrease
    tolerance (None: the reference's CFL budget and 1e-10)."""
    import torch
    from diff_2d_fem_gb300 import workloads, ImplicitIntegrator
    from diff_2d_fem_gb300.adjoint import Rollout
    T = args.grad_steps
    m, kw, dt, ex = workloads.tendon_arms(arms, seed=0, steps=T)
    integ = ImplicitIntegrator(**kw, max_iter=max_iter, eps=eps)
    s = integ.attach(m, dt)
    nt = int(s.desc.T)
    x0 = s.x.detach().clone()
    tip = torch.as_tensor(ex["tip"], device=dev)
    tgt = torch.as_tensor(ex["target"], device=dev)
    stream = torch.cuda.current_stream(dev)

    def rollout(steps, ckpt, E, ten, grad):
        ro = Rollout(s, steps=steps, record=[steps], checkpoint_every=ckpt, rtol=1e-9, max_iter=20000,
                     forward_precision="mixed")
        Et = torch.as_tensor(E, device=dev).clone().requires_grad_(grad)
        Tt = torch.as_tensor(ten, device=dev).clone().requires_grad_(grad)
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record(stream)
        out = ro(Et, Tt, x0, torch.zeros_like(x0))
        e1.record(stream)
        per_arm = ((out[0][tip] - tgt) ** 2).sum(dim=1)
        if grad:
            per_arm.sum().backward()
        e2.record(stream)
        torch.cuda.synchronize(dev)
        ro.close()
        return ro, Et.grad, Tt.grad, e0.elapsed_time(e1), e1.elapsed_time(e2), per_arm.detach().cpu().numpy()

    ones, ten0 = np.ones(nt), np.asarray(ex["tension"][:T], np.float64)
    if warm:
        rollout(2, 1, ones, ten0[:2], True)                   # warm-up: buffers, launch paths
    ro, gE, gT, f_ms, b_ms, L = rollout(T, 10, ones, ten0, True)
    info = dict(ro.info)
    # the checked entries, one per arm
    rng = np.random.default_rng(7)
    quad = np.asarray(m.me.tri_quad)
    n_fd = min(fd_entries, arms)
    n_pix = (3 * n_fd) // 4
    gE_, gT_ = gE.cpu().numpy(), gT.cpu().numpy()
    sel_e, sel_t, adj = {}, {}, []
    for i in range(n_fd):
        if i < n_pix:
            el = m.body_elements(ex["handles"][i])
            sel_e[i] = el[quad[el] == rng.choice(np.unique(quad[el]))]
            adj.append(gE_[sel_e[i]].sum())
        else:
            sel_t[i] = int(rng.integers(T))
            adj.append(gT_[sel_t[i], i] * ten0[sel_t[i], i])
    adj = np.asarray(adj)

    def perturbed_loss(c):                                   # every checked entry scaled by (1 + c)
        E, ten = ones.copy(), ten0.copy()
        for i, el in sel_e.items():
            E[el] = 1.0 + c
        for i, k in sel_t.items():
            ten[k, i] = ten0[k, i] * (1.0 + c)
        return rollout(T, 10, E, ten, False)[-1][:n_fd]

    if stencil == 6:
        d1, d2, d3 = (perturbed_loss(k * h) - perturbed_loss(-k * h) for k in (1, 2, 3))
        fd = (45.0 * d1 - 9.0 * d2 + d3) / (60 * h)
    elif stencil == 4:
        fd = (8.0 * (perturbed_loss(h) - perturbed_loss(-h)) - (perturbed_loss(2 * h) - perturbed_loss(-2 * h))) / (12 * h)
    else:
        fd = (perturbed_loss(h) - perturbed_loss(-h)) / (2 * h)
    err = np.abs(fd - adj) / np.maximum(np.abs(adj), 1e-2 * np.abs(adj).max())
    its = info["adjoint_total_iters"]
    unconv = int(info["forward_unconverged_steps"].sum())
    return {"value": arms / ((f_ms + b_ms) / 1e3), "unit": "grads/s",
            "workload": f"tendon_arms x{arms} (16x64 px of 0.5 mm, E log-U[0.2,1.5] MPa per pixel, "
                        f"tendon on node row 2, piecewise-linear tension in [0,50] N/m), {T} steps, dt {dt}",
            "forward_budget": {"iter_max": int(s.iter_max), "eps": float(integ.eps)},
            "gradient": f"dL/dE per element ({nt // arms} per arm) and dL/dtension per step; "
                        "checkpoints every 10 steps",
            "dtype": "forward and replay mixed-f32/f64, adjoint CG f64",
            "ms_per_grad_batch": f_ms + b_ms, "forward_ms": f_ms, "backward_ms": b_ms,
            "adjoint_cg_iters_per_solve_mean": float(its.mean() / T),
            "adjoint_worst_status": int(np.abs(info["adjoint_worst_status"]).max()),
            "forward_unconverged_scene_steps": unconv, "forward_scene_steps": int(arms * T),
            "forward_unconverged_fraction": unconv / float(arms * T),
            "replay_mismatch": info["replay_mismatch"],
            "grad_err_vs_fd": {"max": float(err.max()), "median": float(np.median(err)), "entries": int(n_fd),
                               "h_rel": h, "stencil": stencil, "pixel_moduli": int(n_pix),
                               "step_tensions": int(n_fd - n_pix)},
            "grad_finite": bool(np.isfinite(gE_).all() and np.isfinite(gT_).all()),
            "loss": float(L.sum())}


def measure_grads(args, dev):
    """grads/s of the differentiation workload with the accuracy of its gradient stated at
    the same settings. The headline runs every forward step to convergence (iteration budget
    --grad-iters, energy-decrease tolerance 1e-13): the adjoint differentiates the converged
    step (the implicit-function argument), so its gradient is the forward map's. The checked
    entries use a 6-point stencil at h = 5e-2 (truncation O(h^6)): the converged forward
    stops where its energy test first passes, which moves the positions by ~1e-10 from one
    perturbed run to the next, and central differences at h = 1e-3 amplify that past 1e-4 on
    the smallest entries, while the 4-point stencil's O(h^4) truncation at this h left 2.6e-4
    on the most nonlinear entry. `at_reference_budget`: the same at
    the reference's CFL iteration budget, where the forward steps stop at the cap before
    converging and the gradient is not the truncated forward map's."""
    out = _grads_at(args, dev, args.arms, max_iter=args.grad_iters, eps=1e-13, h=5e-2, stencil=6)
    out["at_reference_budget"] = _grads_at(args, dev, args.arms, warm=False)
    return out


def measure_single_strip(args, dev):
    """The single-scene configuration: one 6 x 72-pixel strip (511 nodes, 864 triangles) on
    the ground, dt 2 ms, the reference's default integrator. Scene-steps/s of the FP64 path
    (the reference's arithmetic) and of the mixed path over `strip_steps` steps after 5
    warm-up steps (CUDA events), and their position difference after those steps."""
    import torch
    from diff_2d_fem_gb300 import workloads, scene, ImplicitIntegrator
    from diff_2d_fem_gb300.device import DeviceSolver
    m, kw, dt = workloads.strip_on_ground()
    prob = scene.solver_problem(m, ImplicitIntegrator(**kw), dt)
    prob["rest"] = np.asarray(m.me.rest_pos, np.float64)
    stream = torch.cuda.current_stream(dev)
    out, xs = {}, {}
    for prec in ("fp64", "mixed"):
        s = DeviceSolver(prob, precision=prec)
        for _ in range(5):
            s.step()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(dev)
        e0.record(stream)
        for _ in range(args.strip_steps):
            s.step()
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1) / args.strip_steps
        it, _, st = s.stats()
        xs[prec] = s.get_x()
        out[prec] = {"value": 1e3 / ms, "unit": "scene-steps/s", "ms_per_step": ms, "iters_last": int(it[0]),
                     "status_ok": bool((st == 0).all())}
        s.close()
    out["pos_err_mixed_rel_to_coords"] = float(np.abs(xs["mixed"] - xs["fp64"]).max() / np.abs(xs["fp64"]).max())
    out["workload"] = (f"strip_on_ground: 6x72 px (511 nodes, 864 triangles), E 0.5 MPa, nu 0.40, ground mu 0.8, "
                       f"dt {dt}, iter_max {int(prob['iter_max'])}, steps 6..{5 + args.strip_steps}")
    return out


def measure_contact_batch(args, dev):
    """The contact-heavy configuration: 512 scenes of a soft pad pushed by a kinematic jaw
    squeezing an affine 1 GPa block against a second pad (IPC contact with per-scene
    friction, d-hat 0.1 mm, dt 1 ms). Both precisions advance the same scenes the same
    `contact_steps` steps from rest (the jaw's targets of each step); the mixed path is the
    headline. Reported: scene-steps/s of each (CUDA events over the steps), the position
    difference between them, and the difference of the step energies at the two end states
    (every term, barriers included), evaluated by the FP64 energy read-out."""
    import warnings
    import torch
    from diff_2d_fem_gb300 import workloads, scene, ImplicitIntegrator
    from diff_2d_fem_gb300.device import DeviceSolver
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")              # mixed pixel sizes, as configured
        m, kw, dt, ex = workloads.pads_and_block(args.contact_scenes, seed=0)
    ex["command"](0)
    prob = scene.solver_problem(m, ImplicitIntegrator(**kw), dt)
    prob["rest"] = np.asarray(m.me.rest_pos, np.float64)
    bc = np.asarray(prob["bc_idx"])
    targets = []
    for k in range(args.contact_steps):
        ex["command"](k)
        targets.append(np.asarray(m._targets, np.float64).copy())
    stream = torch.cuda.current_stream(dev)
    out, xs, its = {}, {}, {}
    for prec in ("mixed", "fp64"):
        s = DeviceSolver(prob, precision=prec)
        ms = 0.0
        for k in range(args.contact_steps):
            s.set_targets(targets[k])
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            s.step()
            e1.record(stream)
            torch.cuda.synchronize(dev)
            ms += e0.elapsed_time(e1)
        it, ac, st = s.stats()
        xs[prec], its[prec] = s.get_x(), it
        out[prec] = {"value": prob["B"] * args.contact_steps / (ms / 1e3), "unit": "scene-steps/s",
                     "ms_per_step": ms / args.contact_steps, "iters_mean_last": float(it.mean()),
                     "converged_last": float((ac == 0).mean()), "status_ok": bool((st == 0).all())}
        s.close()
        torch.cuda.empty_cache()
    x64, xmx = xs["fp64"], xs["mixed"]
    out["pos_err_rel_to_coords"] = float(np.abs(xmx - x64).max() / np.abs(x64).max())
    # step energy (inertia, elastic, barriers, friction, forces) with the FP64 end state as x_n
    # and x_hat, at the FP64 and at the mixed end state: the first is the potential energy
    # there, the difference the energy error of the mixed state
    ev = DeviceSolver(prob, precision="fp64")
    ev.set_targets(targets[-1])
    ref = torch.as_tensor(x64, device=dev)
    ev.x.copy_(ref)
    ev.xn.copy_(ref)
    ev.xhat.copy_(ref)
    e64 = ev.energy()
    ev.x.copy_(torch.as_tensor(xmx, device=dev))
    emx = ev.energy()
    ev.close()
    out["energy_err_rel"] = float(np.max(np.abs(emx - e64) / np.maximum(np.abs(e64), 1e-300)))
    out["energy_err_rel_median"] = float(np.median(np.abs(emx - e64) / np.maximum(np.abs(e64), 1e-300)))
    out["speedup_mixed_vs_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    out["workload"] = (f"pads_and_block x{prob['B']}: 40x40-px pad (E 0.3 MPa) pushed at 10 mm/s, 16x16-px affine "
                       f"block (1 GPa), second pad; d-hat 0.1 mm, mu U[0.4, 0.8], offset U[-2, 2] mm; dt {dt}, "
                       f"iter_max {int(prob['iter_max'])}, steps 1..{args.contact_steps} from rest")
    return out


def measure_large_scene(args, dev):
    """The large-scene workload: a 256 x 1024-pixel slab (0.5 mm pixels, E 1 MPa, nu 0.40) with
    200 holes and 32 affine discs dropped onto it, dt 1e-3, one scene and a batch of 8, mixed
    precision on a thread-block cluster per scene (the library's default for such batches),
    and the single scene again with every SM on it (`B1_all_sms`, blocks_per_scene =
    D2F_ALL_SMS). Scene-steps/s from CUDA events over `large_steps` steps after one warm-up
    step; the position error of the first step (from rest) against the FP64 path on the same
    scene (the FP64 path runs a block per scene), and the all-SM first step against the
    cluster's."""
    import warnings
    import torch
    from diff_2d_fem_gb300 import workloads, scene, ImplicitIntegrator
    from diff_2d_fem_gb300.device import DeviceSolver
    out = {}
    stream = torch.cuda.current_stream(dev)
    for B, bps in ((1, 0), (8, 0), (1, -1)):
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            m, kw, dt = workloads.slab_with_holes(B, seed=0)
            prob = scene.solver_problem(m, ImplicitIntegrator(**kw), dt)
        s = DeviceSolver(prob, precision="mixed", blocks_per_scene=bps)
        blocks, threads, cs = s.launch_shape()
        s.step()
        x1 = s.get_x()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(dev)
        e0.record(stream)
        for _ in range(args.large_steps):
            s.step()
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1) / args.large_steps
        it, _, st = s.stats()
        s.close()
        rec = {"value": B / (ms / 1e3), "unit": "scene-steps/s", "ms_per_step": ms,
               "nodes": int(prob["x"].shape[0]), "triangles": int(len(prob["tri"])),
               "boundary_nodes": int(len(prob["bnd"])), "iter_max": int(prob["iter_max"]),
               "iters_mean": float(np.mean(it)), "status_ok": bool((st == 0).all()),
               "launch": {"blocks": blocks, "threads": threads, "blocks_per_scene": cs}}
        if bps == -1:  # every SM on the scene (D2F_ALL_SMS), against the default cluster
            rec["first_step_vs_cluster_rel_to_coords"] = float(np.abs(x1 - x1_cluster).max() / np.abs(x1_cluster).max())
            del s
            torch.cuda.empty_cache()
            out["B1_all_sms"] = rec
            continue
        if B == 1:
            x1_cluster = x1
            s64 = DeviceSolver(prob, precision="fp64")
            t64 = time.perf_counter()
            s64.step()
            torch.cuda.synchronize(dev)
            rec["fp64_first_step_s"] = time.perf_counter() - t64
            x64 = s64.get_x()
            s64.close()
            rec["pos_err_rel_to_coords_first_step"] = float(np.abs(x1 - x64).max() / np.abs(x64).max())
        del s
        torch.cuda.empty_cache()
        out[f"B{B}"] = rec
    out["workload"] = ("slab_with_holes: 256x1024 px of 0.5 mm, 200 holes r~U{3..12} px, 32 affine discs "
                       "r~U{8..20} px dropped from 5-50 mm, dt 1e-3, mixed precision")
    return out


# ----------------------------------------------------------------------------- replicas
class Replicas:
    """The host side of N replicas, one rank per GPU: every rank advances its own batch; the
    ranks meet only at a barrier before and after the timed region and in the maximum over
    ranks of the elapsed time; the job's throughput counts every rank's scenes over that
    maximum. `sync` waits for the rank's device work; `reduce_device` holds the all-reduce's
    tensor (a CUDA device under NCCL, the CPU under gloo)."""

    def __init__(self, world, sync=None, reduce_device="cpu"):
        self.world, self.sync, self.reduce_device = world, sync or (lambda: None), reduce_device

    def barrier(self):
        self.sync()
        if self.world > 1:
            import torch.distributed as tdist
            tdist.barrier()

    def maxr(self, v):
        """The maximum of v over the ranks (every rank gets it)."""
        if self.world <= 1:
            return v
        import torch
        import torch.distributed as tdist
        t = torch.tensor([v], dtype=torch.float64, device=self.reduce_device)
        tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
        return float(t.item())

    def timed(self, step, K, W, clock):
        """W untimed calls of step(), a barrier, K timed calls, a barrier; clock() starts a
        timer and returns the function that stops it and gives the elapsed milliseconds.
        Returns this rank's milliseconds (take maxr of it for the job's)."""
        for _ in range(W):
            step()
        self.barrier()
        stop = clock()
        for _ in range(K):
            step()
        ms = stop()
        self.barrier()
        return ms

    def value(self, scenes_per_rank, K, ms_max):
        """Job throughput in scene-steps/s: every rank's scenes over the slowest rank's time."""
        return scenes_per_rank * K * self.world / (ms_max / 1e3)


# ----------------------------------------------------------------------------- GPU arm
def run_ours(args, rank, world):
    import torch
    from diff_2d_fem_gb300 import workloads, scene, ImplicitIntegrator
    from diff_2d_fem_gb300.device import DeviceSolver

    dist = world > 1
    if dist:
        import torch.distributed as tdist
        local = int(os.environ.get("LOCAL_RANK", rank))
        torch.cuda.set_device(local)
        tdist.init_process_group("nccl")
    dev = torch.device("cuda", torch.cuda.current_device())

    if args.profile_large:  # the large-scene step alone, for profilers: warmup + steps, nothing else
        import warnings
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            m, kw, dt = workloads.slab_with_holes(args.profile_large, seed=0)
            prob = scene.solver_problem(m, ImplicitIntegrator(**kw), dt)
        sol = DeviceSolver(prob, precision="mixed", blocks_per_scene=args.profile_bps)
        for _ in range(args.warmup + args.steps):
            sol.step()
        torch.cuda.synchronize(dev)
        it, ac, st = sol.stats()
        print(json.dumps({"profile_large": True, "scenes": int(prob["B"]), "launch": sol.launch_shape(),
                          "iters_mean": float(np.mean(it)), "status_ok": bool((st == 0).all())}))
        return
    m, kw, dt = workloads.rectangles_on_ground(args.scenes, seed=rank)
    integ = ImplicitIntegrator(precision=args.precision, **kw)
    integ.threads, integ.blocks_per_sm = 0, 0
    prob = scene.solver_problem(m, integ, dt)
    prob["rest"] = np.asarray(m.me.rest_pos, np.float64)
    mixed = args.precision == "mixed"
    stream = torch.cuda.current_stream(dev)

    rep = Replicas(world, sync=lambda: torch.cuda.synchronize(dev), reduce_device=dev)
    barrier, maxr = rep.barrier, rep.maxr

    def timed(solver, K, W):
        def clock():
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            return lambda: (ev1.record(stream), torch.cuda.synchronize(dev), ev0.elapsed_time(ev1))[-1]
        ms = rep.timed(solver.step, K, W, clock)
        it, ac, st = solver.stats()
        return ms, it, st

    if args.profile_only:  # the step kernel alone, for profilers: warmup + steps, nothing else
        sol = DeviceSolver(prob, precision=args.precision, threads=args.threads or 128,
                           blocks_per_sm=args.bps or 4)
        for _ in range(args.warmup + args.steps):
            sol.step()
        torch.cuda.synchronize(dev)
        it, ac, st = sol.stats()
        print(json.dumps({"profile_only": True, "precision": args.precision, "scenes": int(prob["B"]),
                          "iters_mean": float(np.mean(it)), "status_ok": bool((st == 0).all())}))
        return

    # ---- launch shape: the autotuner, on a sample of this batch's scenes (untimed)
    from diff_2d_fem_gb300.tune import tune
    shapes = {}
    for prec in ("mixed", "fp64"):
        if args.threads:
            shapes[prec] = ((args.threads, args.bps), [])
        else:
            shapes[prec] = tune(prob, prec, sample=args.tune_sample)
    head_nt, head_bps = shapes[args.precision][0]

    # ---- headline arm (device-resident)
    sol = DeviceSolver(prob, precision=args.precision, threads=head_nt, blocks_per_sm=head_bps)
    with Clocks(int(os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0]) if rank == 0 else 0) as clk:
        ms, it_last, st = timed(sol, args.steps, args.warmup)
    ms = maxr(ms)
    n_sc = prob["B"]
    value = rep.value(n_sc, args.steps, ms)
    x_head, v_head = sol.get_x(), sol.get_v()
    bytes_last = algorithmic_bytes(prob, it_last, mixed)

    # per-launch time of the step kernel, on the launching stream (one launch = one step)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    sol.step()
    e1.record(stream)
    torch.cuda.synchronize(dev)
    launch_ms = e0.elapsed_time(e1)
    it_l, _, _ = sol.stats()
    launch_bytes = algorithmic_bytes(prob, it_l, mixed)
    sol.close()
    del sol
    torch.cuda.empty_cache()

    # ---- the other precision on the same batch, same steps, for the ratio and the error
    other = "fp64" if mixed else "mixed"
    sol2 = DeviceSolver(prob, precision=other, threads=shapes[other][0][0], blocks_per_sm=shapes[other][0][1])
    ms2, it2, st2 = timed(sol2, args.steps, args.warmup)
    ms2 = maxr(ms2)
    value2 = rep.value(n_sc, args.steps, ms2)
    x2 = sol2.get_x()
    sol2.close()
    del sol2
    torch.cuda.empty_cache()
    x64, xmx = (x2, x_head) if mixed else (x_head, x2)
    disp = np.abs(x64 - prob["x"]).max()
    pos_err_rel = float(np.abs(xmx - x64).max() / np.abs(x64).max())
    pos_err_disp = float(np.abs(xmx - x64).max() / max(disp, 1e-300))

    # ---- end to end through the public API: loads up (pinned), simulate, positions down
    fext = prob["fext"]
    f_pin = torch.from_numpy(np.ascontiguousarray(fext)).pin_memory()
    x_pin = torch.empty((prob["x"].shape[0], 2), dtype=torch.float64).pin_memory()
    m._solver = None
    integ.threads, integ.blocks_per_sm = head_nt, head_bps
    integ.simulate(m, dt)                                   # build
    s = m._solver
    for _ in range(args.warmup):
        integ.simulate(m, dt)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        s.tensor("fext").copy_(f_pin, non_blocking=True)   # the step's loads
        integ.simulate(m, dt)
        x_pin.copy_(s.x, non_blocking=True)                 # the step's result
        torch.cuda.current_stream(dev).synchronize()
    barrier()
    e2e_s = maxr(time.perf_counter() - t0)
    e2e = n_sc * args.steps * world / e2e_s
    h2d = int(f_pin.numel() * 8)
    d2h = int(x_pin.numel() * 8)
    x_e2e = x_pin.numpy().copy()
    m._solver.close()
    torch.cuda.empty_cache()

    grads = None if args.no_grads else measure_grads(args, dev)
    large = None if args.no_large else measure_large_scene(args, dev)
    strip = None if args.no_strip else measure_single_strip(args, dev)
    contact = None if args.no_contact else measure_contact_batch(args, dev)

    if rank != 0:
        if dist:
            tdist.destroy_process_group()
        return

    # ---- CPU baseline: the oracle on a bounded sample, from the benchmarked state (the GPU
    # arm's state after its warm-up and timed steps; the sample times the next step)
    threads = min(os.cpu_count() or 1, 16)
    cpu_val, cpu_desc = cpu_sample(prob, x_head, v_head, threads, 4)
    cpu_desc += f" (step {args.warmup + args.steps + 1}, from the GPU arm's state after its timed steps)"

    # ---- FP64 fraction of the plain FP64 kernel: counted FP64 operations per step over its
    # time per step, against this GPU's measured DGEMM rate
    t64_ms = (ms2 if mixed else ms) / args.steps
    it64 = it2 if mixed else it_last
    fp64_rate = fp64_ops(prob, it64) / (t64_ms / 1e3) / 1e12
    fp64_pk = fp64_peak(dev)

    peaks, src = _peaks()
    hbm = float(peaks.get("hbm_gbs", HBM_FALLBACK_GBS))
    achieved = launch_bytes / (launch_ms / 1e3) / 1e9
    tshape = f"{head_nt}x{head_bps}"
    tps = TRAFFIC_PER_SCENE_ITER.get((args.precision, tshape))
    traffic = float(tps * np.sum(it_l)) if tps is not None else None
    rec = {
        "metric": "batched scene-steps/s (implicit PNCG step)",
        "value": value, "unit": "scene-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "mixed-f32/f64" if mixed else "f64", "data": "synthetic (seeded)",
        "config": {"workload": f"rectangles_on_ground x{n_sc} (H~U{{4..16}}, W~U{{32..128}}, 0.75 mm px, "
                               f"E log-U[0.1,2] MPa, mu~U[0.3,0.9], p~U[0,5] kPa)",
                   "dt": dt, "gtol": kw.get("gtol"), "iter_max": int(prob["iter_max"]),
                   "nodes": int(prob["x"].shape[0]), "triangles": int(len(prob["tri"])),
                   "l2": "inputs larger than L2 (per-step working set several GB)",
                   "precision": args.precision, "parallelism": f"replicas x{world}",
                   "launch_shape": {p: {"threads": v[0][0], "blocks_per_sm": v[0][1],
                                        "tuned_ms": [[round(t[0], 2), t[1], t[2]] for t in v[1]]}
                                    for p, v in shapes.items()}},
        "precision_compare": {"other": other, "other_value": value2,
                              "speedup_vs_other": value / value2 if value2 else None,
                              "pos_err_rel_to_coords": pos_err_rel, "pos_err_rel_to_displacement": pos_err_disp},
        "iters_mean": float(np.mean(it_last)), "iters_max": int(np.max(it_last)),
        "status_ok": bool((st == 0).all()),
        "gpu_launches": args.steps,
        "clocks": clk.summary(),
        "e2e": {"value": e2e, "unit": "scene-steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": traffic, "peak_source": src,
                     "traffic_source": (f"ncu capture of 608 scenes ({tshape} launch shape), scaled by "
                                        f"scene-iterations ({int(np.sum(it_l))} in this launch)")
                                       if traffic is not None else f"no ncu capture at the {tshape} launch shape",
                     "algorithmic_bytes_per_launch": launch_bytes, "launch_ms": launch_ms},
        "cpu_baseline": {"value": cpu_val, "unit": "scene-steps/s", "cores": threads, "kind": "port",
                         "sample": cpu_desc},
        "grads": grads,
        "large_scene": large,
        "single_strip": strip,
        "contact_batch": contact,
        "fp64_fraction": {"achieved": fp64_rate, "peak": fp64_pk, "unit": "TFLOP/s", "frac": fp64_rate / fp64_pk,
                          "ops_per_triangle_iter": FP64_OPS_PER_TRI_ITER, "ops_per_node_iter": FP64_OPS_PER_NODE_ITER,
                          "peak_source": "measured: cuBLAS DGEMM (torch.matmul float64, 4096^3), best of 5",
                          "kernel": "the plain FP64 step kernel on this batch"},
    }
    print(json.dumps(rec))
    if dist:
        tdist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--scenes", type=int, default=4096)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--threads", type=int, default=0, help="launch shape; 0 = autotune")
    ap.add_argument("--bps", type=int, default=0)
    ap.add_argument("--tune-sample", type=int, default=1024)
    ap.add_argument("--arms", type=int, default=256, help="differentiation workload: arms per batch")
    ap.add_argument("--grad-steps", type=int, default=100, help="differentiation workload: steps")
    ap.add_argument("--grad-iters", type=int, default=3000,
                    help="differentiation workload: forward iteration budget (steps stop on the energy test)")
    ap.add_argument("--no-grads", action="store_true", help="skip the grads/s measurement")
    ap.add_argument("--no-large", action="store_true", help="skip the large-scene measurement")
    ap.add_argument("--large-steps", type=int, default=3, help="large-scene workload: timed steps")
    ap.add_argument("--strip-steps", type=int, default=50, help="single-strip workload: timed steps")
    ap.add_argument("--no-strip", action="store_true", help="skip the single-strip measurement")
    ap.add_argument("--contact-scenes", type=int, default=512, help="contact-heavy workload: scenes")
    ap.add_argument("--contact-steps", type=int, default=20, help="contact-heavy workload: steps from rest")
    ap.add_argument("--no-contact", action="store_true", help="skip the contact-heavy measurement")
    ap.add_argument("--profile-large", type=int, default=0,
                    help="run only the large-scene step (this many slabs), for profilers")
    ap.add_argument("--profile-bps", type=int, default=0,
                    help="with --profile-large: blocks per scene (0 library default, -1 every SM)")
    ap.add_argument("--profile-only", action="store_true",
                    help="run only warmup + steps of the step kernel (for ncu)")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world)


if __name__ == "__main__":
    main()
