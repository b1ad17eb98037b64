"""Serving loop: jobs of different size, depth, window and method submitted
together (continuous batching under a memory budget) give exactly the
results of running each job alone, and jobs overlap on the GPU."""
import numpy as np
import pytest

from fringe_gb300 import synth

pytestmark = pytest.mark.gpu

SPECS = [  # (rows, cols, nbands, ny, nx, method, seed)
    (64, 64, 12, 3, 3, "MLE", 11),
    (40, 96, 30, 5, 10, "MLE", 12),
    (96, 48, 20, 2, 5, "EVD", 13),
    (32, 32, 45, 5, 10, "MLE", 14),
    (80, 64, 10, 1, 1, "EVD", 15),
    (48, 48, 60, 3, 5, "MLE", 16),
]


@pytest.mark.parametrize("budget_mb,precision", [(4096, "fp32"), (6, "fp32"), (4096, "mixed"), (6, "both")])
def test_served_results_equal_single_runs(gpu_lib, budget_mb, precision):
    from fringe_gb300 import phase_link
    from fringe_gb300.serve import Server
    scenes = [synth.scene("voronoi", R, C, N, ny, nx, seed=sd) for R, C, N, ny, nx, m, sd in SPECS]
    precs = [precision if precision != "both" else ("mixed" if k % 2 else "fp32") for k in range(len(SPECS))]
    ref = [phase_link(st, nm, (ny, nx), method=m, precision=p)
           for (st, nm), (R, C, N, ny, nx, m, sd), p in zip(scenes, SPECS, precs)]
    # a small wave budget forces several waves per job (slices that do not
    # start on the 8-row tile grid); a small memory budget forces admission
    # to wait for earlier jobs to finish
    srv = Server(memory_budget=budget_mb << 20, wave_pixels=2048)
    tickets = [srv.submit(st, nm, (ny, nx), method=m, precision=p)
               for (st, nm), (R, C, N, ny, nx, m, sd), p in zip(scenes, SPECS, precs)]
    infos = [srv.wait(t) for t in tickets]
    for t, r in zip(tickets, ref):
        got = srv.result(t)
        for key in ("phase", "tcorr", "comp"):
            assert np.array_equal(got[key], r[key], equal_nan=True), key
    assert all(i["total_ms"] > 0 for i in infos)
    srv.close()


def test_jobs_overlap_in_time(gpu_lib):
    from fringe_gb300.serve import Server
    srv = Server(wave_pixels=4096)
    scenes = [synth.scene("voronoi", 64, 64, 30, 5, 10, seed=20 + k) for k in range(4)]
    tickets = [srv.submit(st, nm, (5, 10)) for st, nm in scenes]
    infos = [srv.wait(t) for t in tickets]
    # with waves of 4096 pixels every job needs several waves: admitted
    # together, they share the waves, so each job's run time exceeds a
    # quarter of the total and the queueing delay stays small
    assert max(i["queue_ms"] for i in infos) < max(i["run_ms"] for i in infos)
    srv.close()
