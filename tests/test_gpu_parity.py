"""GPU parity: the CUDA path (through the C ABI) against the CPU oracle.

Every case runs the same seeded inputs through libfringe_gb300.so and through
the oracle's FP64 restatement of the reference loop, and checks validity codes
(exact), wrapped phase RMS (<= 1e-3 rad), temporal coherence (<= 1e-4) and the
exact zeros of skipped pixels.
"""
import numpy as np
import pytest

import oracle
from fringe_gb300 import synth
from tests.parity import assert_parity, codes, compare, load_golden

pytestmark = pytest.mark.gpu


def _run_both(stack, nmap, ny, nx, **kw):
    from fringe_gb300 import phase_link
    g = phase_link(stack, nmap, (ny, nx), want_status=True, **kw)
    okw = {k: v for k, v in kw.items() if k in ("method", "semantics", "mini_stack_count",
                                                  "band_width", "min_neighbors")}
    o = oracle.run(stack, nmap, ny, nx, **okw)
    return g, o


@pytest.fixture(scope="module")
def vor30():
    return synth.scene("voronoi", 40, 72, 30, 5, 10, seed=1002)


@pytest.mark.parametrize("method,semantics,extra", [
    ("MLE", "evd", {}),
    ("EVD", "evd", {}),
    ("STBAS", "evd", {"band_width": 5}),
    ("MLE", "phase_link", {"min_neighbors": 5}),
    ("EVD", "phase_link", {}),
    ("STBAS", "phase_link", {"band_width": 7}),
    ("MLE", "evd", {"mini_stack_count": 4}),
    ("EVD", "evd", {"mini_stack_count": 30}),
])
def test_voronoi_n30(gpu_lib, vor30, method, semantics, extra):
    stack, nmap = vor30
    g, o = _run_both(stack, nmap, 5, 10, method=method, semantics=semantics, **extra)
    m = compare(g, o)
    assert m["valid_both"] > 1000, m
    assert_parity(m)


@pytest.mark.parametrize("method", ["EVD", "MLE"])
def test_uniform_n10(gpu_lib, method):
    stack, nmap = synth.scene("uniform", 48, 48, 10, 5, 5, seed=1001)
    g, o = _run_both(stack, nmap, 5, 5, method=method)
    m = compare(g, o)
    assert m["valid_both"] == 48 * 48, m
    assert_parity(m)


@pytest.mark.parametrize("precision", ["fp32", "mixed"])
@pytest.mark.parametrize("method", ["EVD", "MLE"])
def test_cpu_runnable_configuration_full_scene(gpu_lib, method, precision):
    """The CPU-runnable configuration at its full size: 200x200 pixels,
    N = 10, half-window 5x5, all-ones SHP map (edge-clipped windows at the
    borders); every pixel valid in both."""
    stack, nmap = synth.scene("uniform", 200, 200, 10, 5, 5, seed=1001)
    g, o = _run_both(stack, nmap, 5, 5, method=method, precision=precision)
    m = compare(g, o)
    assert m["valid_both"] == 200 * 200, m
    assert_parity(m)


@pytest.mark.parametrize("precision", ["fp32", "mixed"])
def test_ill_conditioned_64_dates_tile(gpu_lib, precision):
    """A tile of the ill-conditioned 64-date configuration (per-pixel
    coherence U(0.05, 0.9), decorrelated pixels): MLE through the FP32 band
    and the FP64 settle."""
    stack, nmap = synth.scene("illcond", 48, 64, 64, 5, 10, seed=1003)
    g, o = _run_both(stack, nmap, 5, 10, method="MLE", precision=precision)
    m = compare(g, o)
    assert m["valid_both"] > 1000, m
    assert_parity(m)


@pytest.mark.parametrize("nb", [1, 2, 3, 15, 16, 17, 31, 32, 33, 47, 63, 64])
def test_depths(gpu_lib, nb):
    stack, nmap = synth.scene("voronoi", 20, 24, nb, 2, 3, seed=100 + nb)
    for method, sem in (("MLE", "evd"), ("EVD", "evd"), ("MLE", "phase_link")):
        g, o = _run_both(stack, nmap, 2, 3, method=method, semantics=sem)
        m = compare(g, o)
        assert_parity(m)
        if nb == 1:
            both = (g["tcorr"] != 0) | np.isnan(g["tcorr"])
            assert np.array_equal(np.isnan(g["tcorr"]), np.isnan(o["tcorr"]))


def test_illconditioned_n64(gpu_lib):
    stack, nmap = synth.scene("illcond", 24, 40, 64, 5, 10, seed=1003)
    for method, sem in (("MLE", "evd"), ("MLE", "phase_link"), ("EVD", "evd")):
        g, o = _run_both(stack, nmap, 5, 10, method=method, semantics=sem)
        assert_parity(compare(g, o))


def test_edge_masks_and_shapes(gpu_lib):
    # empty nmap: every centre bit clear -> all outputs exactly zero
    stack, nmap = synth.scene("uniform", 12, 15, 8, 2, 2, seed=5)
    z = np.zeros_like(nmap)
    g, o = _run_both(stack, z, 2, 2, method="MLE")
    assert not np.any(g["phase"]) and not np.any(g["tcorr"]) and not np.any(g["comp"])
    assert np.all(g["status"] == 1)
    # centre bit only -> npix = 1 < 2 -> skipped
    c = np.zeros_like(nmap)
    flat = 2 * 5 + 2
    c[..., flat // 32] = np.uint32(1 << (flat % 32))
    g, o = _run_both(stack, c, 2, 2, method="EVD")
    assert not np.any(g["phase"]) and np.all(g["status"] == 2)
    # window larger than the scene, and a single row / column
    for shape in ((3, 4), (1, 17), (19, 1), (1, 1)):
        st, nm = synth.scene("uniform", shape[0], shape[1], 6, 5, 10, seed=9)
        for method in ("MLE", "EVD"):
            g, o = _run_both(st, nm, 5, 10, method=method)
            assert_parity(compare(g, o))
    # phase_link min_neighbors above the window size -> everything skipped
    g, o = _run_both(stack, nmap, 2, 2, method="MLE", semantics="phase_link", min_neighbors=26)
    assert not np.any(g["tcorr"]) and not np.any(o["tcorr"])


def test_no_data_dates(gpu_lib):
    """A date with zero power in a window gives 0/0 coherence; the defined
    result is the failure code of the first eigen call (the reference's
    LAPACK output is undefined there)."""
    stack, nmap = synth.scene("uniform", 16, 16, 10, 2, 2, seed=5)
    stack[3, :8, :8] = 0
    stack[:, 12:, 12:] = 0
    for method, sem in (("MLE", "evd"), ("EVD", "evd"), ("MLE", "phase_link")):
        g, o = _run_both(stack, nmap, 2, 2, method=method, semantics=sem)
        assert_parity(compare(g, o))


def test_fp64_form_matches_oracle_tightly(gpu_lib, vor30):
    from fringe_gb300 import _lib, phase_link
    stack, nmap = vor30
    ctx = _lib.Context(0)
    ctx.set_tuning(force_fp64=True)
    for method, sem in (("MLE", "evd"), ("EVD", "evd"), ("MLE", "phase_link")):
        g = phase_link(stack, nmap, (5, 10), method=method, semantics=sem, ctx=ctx)
        o = oracle.run(stack, nmap, 5, 10, method=method, semantics=sem)
        m = compare(g, o)
        assert_parity(m, phase_tol=1e-5, tcorr_tol=1e-5)
    ctx.close()


def test_fp64_form_64_dates_matches_oracle(gpu_lib):
    """The FP64 form at 64 dates keeps C in tensor memory (two warps per SM);
    every pixel of an ill-conditioned scene takes it."""
    from fringe_gb300 import _lib, phase_link
    stack, nmap = synth.scene("illcond", 20, 24, 64, 5, 10, seed=1003)
    ctx = _lib.Context(0)
    ctx.set_tuning(force_fp64=True)
    for method, sem in (("MLE", "evd"), ("EVD", "evd"), ("STBAS", "evd"), ("MLE", "phase_link")):
        extra = {"band_width": 9} if method == "STBAS" else {}
        g = phase_link(stack, nmap, (5, 10), method=method, semantics=sem, ctx=ctx, want_status=True, **extra)
        o = oracle.run(stack, nmap, 5, 10, method=method, semantics=sem, **extra)
        m = compare(g, o)
        assert m["valid_both"] > 100, m
        assert_parity(m, phase_tol=1e-5, tcorr_tol=1e-5)
    ctx.close()


@pytest.mark.parametrize("shift,backoff", [(1.5, 0.97), (1.5, 1.5)])
def test_mle_fallback_paths(gpu_lib, vor30, shift, backoff):
    """A first shift above lambda_1 makes the Cholesky of M - sigma I fail:
    (1.5, 0.97) takes the second attempt at the backed-off shift, (1.5, 1.5)
    fails both and takes the Householder path; both agree with the oracle."""
    from fringe_gb300 import _lib, phase_link
    stack, nmap = vor30
    ctx = _lib.Context(0)
    ctx.set_shift(shift, backoff)
    for prec in ("fp32", "mixed"):
        for sem in ("evd", "phase_link"):
            g = phase_link(stack, nmap, (5, 10), method="MLE", semantics=sem, precision=prec,
                           want_status=True, ctx=ctx)
            o = oracle.run(stack, nmap, 5, 10, method="MLE", semantics=sem)
            m = compare(g, o)
            assert m["valid_both"] > 1000, m
            assert_parity(m)
    # host-memory run: the statistics count the pixels that left the fast path
    phase_link(stack, nmap, (5, 10), method="MLE", ctx=ctx)
    assert ctx.stats()["slow_path_pixels"] > 1000
    ctx.close()


def test_row_range_and_torch_device_path(gpu_lib, vor30):
    torch = pytest.importorskip("torch")
    from fringe_gb300 import phase_link
    stack, nmap = vor30
    full = phase_link(stack, nmap, (5, 10), method="MLE")
    part = phase_link(stack, nmap, (5, 10), method="MLE", rows=(10, 25))
    assert np.array_equal(part["phase"][:, 10:25], full["phase"][:, 10:25])
    assert np.array_equal(part["tcorr"][10:25], full["tcorr"][10:25])
    ts = torch.from_numpy(stack).cuda()
    tn = torch.from_numpy(nmap.view(np.int32)).cuda()
    dev = phase_link(ts, tn, (5, 10), method="MLE")
    torch.cuda.synchronize()
    assert np.array_equal(dev["phase"].cpu().numpy(), full["phase"])
    assert np.array_equal(dev["tcorr"].cpu().numpy(), full["tcorr"])
    assert np.array_equal(dev["comp"].cpu().numpy(), full["comp"])


@pytest.mark.parametrize("precision", ["fp32", "mixed"])
def test_golden_vectors_from_the_reference(gpu_lib, precision):
    """Both forms against golden vectors made with the reference's own
    EVWorker + LAPACK (tests/golden/make_golden.py); the mixed form at its
    stated tolerances (1e-3 rad RMS, |dtcorr| <= 2e-4)."""
    from fringe_gb300 import phase_link
    tol = dict(phase_tol=1e-3, tcorr_tol=2e-4) if precision == "mixed" else {}
    for case, g in load_golden().items():
        for var, (method, sem, extra, ref) in g["variants"].items():
            got = phase_link(g["stack"], g["nmap"], (g["ny"], g["nx"]), method=method,
                             semantics=sem, precision=precision, **extra)
            m = compare(got, ref)
            # a variant may code every pixel (-4 everywhere on the indefinite-|C| scenes)
            assert m["valid_both"] > 0 or np.all(codes(ref) < 0), (case, var, m)
            assert_parity(m, **tol)


def test_scene_past_32_bit_indices(gpu_lib):
    """A 8448 x 8704 scene of 30 dates (N * pixels > 2^31) tiled on the device
    from a seeded 256 x 256 block: pixels whose windows lie inside one copy
    equal the block's own results bit for bit (mixed form over the whole
    scene, plain FP32 form over its last rows)."""
    torch = pytest.importorskip("torch")
    from fringe_gb300 import phase_link
    B, N, ny, nx = 256, 30, 5, 10
    stack, nmap = synth.scene("voronoi", B, B, N, ny, nx, seed=808)
    ref_mixed = phase_link(stack, nmap, (ny, nx), precision="mixed")
    ref_fp32 = phase_link(stack, nmap, (ny, nx), precision="fp32")
    TR, TC = 33, 34
    d_stack = torch.from_numpy(stack).cuda().repeat(1, TR, TC)
    d_nmap = torch.from_numpy(nmap.view(np.int32)).cuda().repeat(TR, TC, 1)
    R, C = B * TR, B * TC
    assert N * R * C > 2 ** 31
    inner = (slice(ny, B - ny), slice(nx, B - nx))
    out = phase_link(d_stack, d_nmap, (ny, nx), precision="mixed")
    for tr, tc in ((0, 0), (TR - 1, TC - 1), (17, 5)):
        sl = (slice(tr * B, (tr + 1) * B), slice(tc * B, (tc + 1) * B))
        t = out["tcorr"][sl].cpu().numpy()[inner]
        assert np.array_equal(t, ref_mixed["tcorr"][inner], equal_nan=True), (tr, tc)
        p = out["phase"][:, sl[0], sl[1]].cpu().numpy()[:, inner[0], inner[1]]
        assert np.array_equal(p, ref_mixed["phase"][:, inner[0], inner[1]]), (tr, tc)
    del out
    r0 = (TR - 1) * B
    out = phase_link(d_stack, d_nmap, (ny, nx), precision="fp32", rows=(r0, R))
    t = out["tcorr"][r0:, (TC - 1) * B:].cpu().numpy()[inner]
    assert np.array_equal(t, ref_fp32["tcorr"][inner], equal_nan=True)


def test_host_run_with_many_settled_pixels_equals_device_run(gpu_lib):
    """A host-memory run puts the FP64-settled pixels in place on the host,
    split over several threads once there are more than 512 of them; its
    outputs equal those of the device-memory run bit for bit."""
    torch = pytest.importorskip("torch")
    from fringe_gb300 import _lib, phase_link
    stack, nmap = synth.scene("illcond", 320, 320, 64, 5, 10, seed=1003)
    ctx = _lib.Context(0)
    host = phase_link(stack, nmap, (5, 10), method="MLE", precision="mixed", want_status=True, ctx=ctx)
    settled = ctx.stats()["fp64_pixels"]
    assert settled > 2 * 512, settled
    ts = torch.from_numpy(stack).cuda()
    tn = torch.from_numpy(nmap.view(np.int32)).cuda()
    dev = phase_link(ts, tn, (5, 10), method="MLE", precision="mixed", want_status=True, ctx=ctx)
    torch.cuda.synchronize()
    assert ctx.stats()["fp64_pixels"] == settled
    for key in ("phase", "tcorr", "comp", "status"):
        assert np.array_equal(dev[key].cpu().numpy().view(np.uint8), host[key].view(np.uint8)), key
