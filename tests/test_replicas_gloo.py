"""The multi-GPU form of the step is N replicas: scenes are independent, so each rank
advances its own batch and the ranks meet only at the barriers around the timed region and
in the max-over-ranks of the elapsed time. This runs bench.py's own replica logic
(bench.Replicas: barriers, timed region, max over ranks, job throughput) at world size 2
over gloo on the CPU, the oracle standing in for the device step: each rank builds the
rectangles batch with its own seed (as bench.py does), steps it, and reports its time; the
job's time is the slowest rank's and the throughput counts every rank's scenes.

Checks: the replicas are different batches of the same size, each replica ends exactly where
the same batch run alone ends (nothing crosses ranks), and every rank sees the same maximum."""
import os
import socket
import tempfile
import time
import warnings

import numpy as np

SCENES, STEPS, WORLD = 3, 2, 2


def _batch(seed):
    from diff_2d_fem_gb300 import ImplicitIntegrator, scene, workloads
    m, kw, dt = workloads.rectangles_on_ground(SCENES, seed=seed)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        return scene.solver_problem(m, ImplicitIntegrator(precision="fp64", **kw), dt)


def _rank(rank, port, out):
    import sys
    import torch
    import torch.distributed as dist
    import oracle
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=WORLD)
    try:
        prob = _batch(rank)
        solver = oracle.OracleSolver(prob)
        rep = bench.Replicas(WORLD, reduce_device="cpu")

        def clock():
            t0 = time.perf_counter()
            return lambda: (time.perf_counter() - t0) * 1e3
        ms = rep.timed(solver.step, STEPS, 1, clock)
        ms_max = rep.maxr(ms)
        n = torch.tensor([int(prob["B"])], dtype=torch.int64)
        dist.all_reduce(n)
        np.savez(os.path.join(out, f"rank{rank}.npz"), x=solver.x, ms=ms, ms_max=ms_max,
                 scenes=int(prob["B"]), scenes_all=int(n.item()), value=rep.value(int(prob["B"]), STEPS, ms_max))
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_replicas_share_nothing_but_the_clock():
    import torch.multiprocessing as mp
    import oracle
    with tempfile.TemporaryDirectory() as out:
        mp.start_processes(_rank, args=(_free_port(), out), nprocs=WORLD, start_method="spawn", join=True)
        r = [dict(np.load(os.path.join(out, f"rank{k}.npz"))) for k in range(WORLD)]
    assert r[0]["x"].shape != r[1]["x"].shape or not np.array_equal(r[0]["x"], r[1]["x"])
    for k in range(WORLD):
        assert int(r[k]["scenes"]) == SCENES and int(r[k]["scenes_all"]) == WORLD * SCENES
        assert float(r[k]["ms_max"]) == max(float(q["ms"]) for q in r)
        assert float(r[k]["value"]) == float(r[0]["value"])
        _, xs, _ = oracle.run(_batch(k), STEPS + 1)       # one warm-up step and the timed ones
        assert np.array_equal(r[k]["x"], xs[-1]), k
        assert float(r[k]["value"]) == SCENES * STEPS * WORLD / (float(r[k]["ms_max"]) / 1e3)
