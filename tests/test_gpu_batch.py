"""Batches: jobs of different size, stack depth, window and method in one
persistent launch (fpl_batch_*) give exactly the results of running each
job alone, with and without CUDA-graph replay and autotuning, in the plain
FP32 form, the mixed-precision form, and a mix of the two."""
import numpy as np
import pytest

from fringe_gb300 import synth

pytestmark = pytest.mark.gpu

SPECS = [  # (rows, cols, nbands, ny, nx, method, mini_stack_count, seed)
    (40, 48, 10, 5, 5, "MLE", 1, 1),
    (24, 64, 15, 3, 5, "EVD", 2, 2),
    (48, 40, 20, 5, 10, "MLE", 3, 3),
    (32, 56, 30, 5, 10, "MLE", 1, 4),
    (28, 36, 30, 2, 3, "EVD", 4, 5),
    (20, 32, 45, 5, 10, "MLE", 1, 6),
]


def _jobs(torch):
    jobs = []
    for R, C, N, ny, nx, m, k, seed in SPECS:
        st, nm = synth.scene("voronoi", R, C, N, ny, nx, seed=seed)
        jobs.append({"stack": torch.from_numpy(st).cuda(), "nmap": torch.from_numpy(nm.view(np.int32)).cuda(),
                     "half_window": (ny, nx), "method": m, "mini_stack_count": k})
    return jobs


@pytest.mark.parametrize("graph,autotune,precision", [
    (True, False, "fp32"), (False, False, "fp32"), (True, True, "fp32"),
    (True, False, "mixed"), (False, False, "mixed"), (True, True, "mixed"), (True, False, "both")])
def test_batch_equals_single_jobs(gpu_lib, graph, autotune, precision):
    torch = pytest.importorskip("torch")
    from fringe_gb300.linker import PhaseLinkBatch, phase_link
    jobs = _jobs(torch)
    for k, j in enumerate(jobs):
        j["precision"] = precision if precision != "both" else ("mixed" if k % 2 else "fp32")
    ref = []
    for j in jobs:
        r = phase_link(j["stack"], j["nmap"], j["half_window"], method=j["method"],
                       mini_stack_count=j["mini_stack_count"], precision=j["precision"])
        ref.append({k: v.clone() for k, v in r.items()})
    torch.cuda.synchronize()
    b = PhaseLinkBatch(jobs, graph=graph, autotune=autotune)
    for rep in range(2):
        for o in b.outputs:
            for v in o.values():
                v.zero_()
        out = b.run()
        torch.cuda.synchronize()
        for k, (o, r) in enumerate(zip(out, ref)):
            for key in ("phase", "tcorr", "comp"):
                a, c = o[key].cpu().numpy(), r[key].cpu().numpy()
                assert np.array_equal(a, c, equal_nan=True), (k, key, rep)
    st = b.stats()
    assert st["pixels"] == sum(R * C for R, C, *_ in SPECS)
    b.close()


def test_mixed_batch_over_several_waves(gpu_lib):
    """Mixed-form jobs larger than one wave (2^20 pixels) are cut into row
    pieces whose tiles straddle piece boundaries; results still equal the
    single runs bit for bit."""
    torch = pytest.importorskip("torch")
    from fringe_gb300.linker import PhaseLinkBatch, phase_link
    jobs = []
    for R, C, N, ny, nx, seed in [(1100, 1000, 12, 3, 5, 31), (300, 700, 30, 5, 10, 32)]:
        st, nm = synth.scene("voronoi", R, C, N, ny, nx, seed=seed)
        jobs.append({"stack": torch.from_numpy(st).cuda(), "nmap": torch.from_numpy(nm.view(np.int32)).cuda(),
                     "half_window": (ny, nx), "method": "MLE", "precision": "mixed"})
    ref = [{k: v.clone() for k, v in phase_link(j["stack"], j["nmap"], j["half_window"],
                                                 precision="mixed").items()} for j in jobs]
    b = PhaseLinkBatch(jobs, graph=True)
    out = b.run()
    torch.cuda.synchronize()
    for o, r in zip(out, ref):
        for key in ("phase", "tcorr", "comp"):
            assert np.array_equal(o[key].cpu().numpy(), r[key].cpu().numpy(), equal_nan=True), key
    b.close()
