"""Comparison helpers for parity tests (GPU result vs oracle result)."""
import numpy as np

PHASE_RMS_TOL = 1e-3     # rad, wrapped difference, dates referenced to mini-1
TCORR_TOL = 1e-4         # absolute
# compressed SLC (scene-normalised, see compare): its error follows the
# phase error (measured against the oracle on the GPU: RMS <= 8e-6, max
# <= 1.4e-4 for both forms), so its RMS tolerance is the phase tolerance
# capped at COMP_RMS_TOL, and its maximum COMP_MAX_FACTOR times that
COMP_RMS_TOL = 5e-5
COMP_MAX_FACTOR = 10


def codes(res):
    """Per-pixel validity: the reference's negative tcorr codes, else 0."""
    t = res["tcorr"]
    return np.where(t < 0, t, 0).astype(np.float32)


def compare(g, o):
    """Metrics of GPU result g against oracle result o over pixels valid in both."""
    cg, co = codes(g), codes(o)
    vg = (cg == 0) & (np.abs(g["phase"]).sum(axis=0) > 0)
    vo = (co == 0) & (np.abs(o["phase"]).sum(axis=0) > 0)
    both = vg & vo
    d = np.angle(g["phase"][:, both] * np.conj(o["phase"][:, both]))
    rms = float(np.sqrt(np.mean(d.astype(np.float64) ** 2))) if d.size else 0.0
    mx = float(np.max(np.abs(d))) if d.size else 0.0
    tg, to = g["tcorr"][both], o["tcorr"][both]
    # NaN (0/0 for a single date, as the reference) must agree exactly
    nan_g, nan_o = np.isnan(tg), np.isnan(to)
    dt = float(np.max(np.abs(tg - to)[~(nan_g & nan_o)], initial=0.0)) if tg.size else 0.0
    if np.any(nan_g != nan_o):
        dt = float("inf")
    # compressed SLC: |comp_gpu - comp_oracle| in units of the scene's mean
    # |comp_oracle| over the pixels valid in both (per pixel the difference
    # is at most the pixel's mean amplitude times its largest phase error)
    cgc = g["comp"][both].astype(np.complex128)
    coc = o["comp"][both].astype(np.complex128)
    scale = float(np.mean(np.abs(coc))) if coc.size else 1.0
    ce = np.abs(cgc - coc) / max(scale, 1e-30)
    if np.any(~np.isfinite(cgc) != ~np.isfinite(coc)):
        ce = np.full_like(ce, np.inf)
    ce = np.where(np.isfinite(coc), ce, 0.0)
    zero_g = (np.abs(g["phase"]).sum(axis=0) == 0)
    zero_o = (np.abs(o["phase"]).sum(axis=0) == 0)
    return {
        "valid_both": int(both.sum()),
        "valid_only_gpu": int((vg & ~vo).sum()),
        "valid_only_oracle": int((vo & ~vg).sum()),
        "code_mismatch": int((cg != co).sum()),
        "phase_rms": rms,
        "phase_max": mx,
        "tcorr_max": dt,
        "comp_rms": float(np.sqrt(np.mean(ce ** 2))) if ce.size else 0.0,
        "comp_max": float(np.max(ce)) if ce.size else 0.0,
        # skipped pixels must be exactly zero in both (phase and compressed SLC)
        "zero_mismatch": int(((~vg) & (~vo) & (cg == co) & ~(zero_g & zero_o)).sum()),
        "comp_zero_mismatch": int(((~vg) & (~vo) & (cg == co) &
                                   ((g["comp"] != 0) | (o["comp"] != 0))).sum()),
    }


def assert_parity(m, phase_tol=PHASE_RMS_TOL, tcorr_tol=TCORR_TOL, max_code_mismatch=0,
                  comp_tol=None, comp_max_tol=None):
    """Codes identical, phase RMS, |dtcorr| and the compressed SLC within
    tolerance.  The compressed-SLC error (scene-normalised, see compare) is
    linear in the phase error, so its RMS tolerance defaults to the phase
    tolerance capped at COMP_RMS_TOL and its maximum to COMP_MAX_FACTOR
    times that."""
    comp_tol = min(phase_tol, COMP_RMS_TOL) if comp_tol is None else comp_tol
    comp_max_tol = COMP_MAX_FACTOR * phase_tol if comp_max_tol is None else comp_max_tol
    assert m["code_mismatch"] <= max_code_mismatch, m
    assert m["phase_rms"] <= phase_tol, m
    assert m["tcorr_max"] <= tcorr_tol, m
    assert m["zero_mismatch"] == 0, m
    assert m["comp_zero_mismatch"] == 0, m
    assert m["comp_rms"] <= comp_tol, m
    assert m["comp_max"] <= comp_max_tol, m


GOLDEN = __import__("os").path.join(__import__("os").path.dirname(__import__("os").path.abspath(__file__)),
                                    "golden", "golden_phase_link.npz")


def load_golden():
    """Golden vectors made by tests/golden/make_golden.py from the reference's
    own EVWorker + LAPACK.  Returns {case: {"stack", "nmap", "ny", "nx",
    "variants": {key: (method, semantics, extra, result)}}}."""
    d = np.load(GOLDEN)
    cases = {}
    for name in d.files:
        if name.endswith("/shape"):
            case = name.split("/")[0]
            R, C, N, ny, nx = [int(x) for x in d[name]]
            cases[case] = {"stack": d[case + "/stack"], "nmap": d[case + "/nmap"],
                           "ny": ny, "nx": nx, "variants": {}}
    for name in d.files:
        if not name.endswith("/tcorr"):
            continue
        case, var = name.split("/")[:2]
        parts = var.split("_")
        method, sem = parts[0], parts[1]
        if sem == "phase":                    # "phase_link"
            sem = "phase_link"
        extra = {}
        # extras are encoded as _<name><value>
        tail = var[len(method) + 1 + len(sem):]
        for key in ("band_width", "min_neighbors", "mini_stack_count"):
            tag = "_" + key
            if tag in tail:
                val = tail.split(tag, 1)[1]
                num = ""
                for ch in val:
                    if ch.isdigit():
                        num += ch
                    else:
                        break
                extra[key] = int(num)
        k = case + "/" + var
        ang = d[k + "/phase_angle"]
        zero = d[k + "/phase_zero"]
        phase = np.exp(1j * ang.astype(np.float64)).astype(np.complex64)
        phase[:, zero] = 0
        res = {"phase": phase, "tcorr": d[k + "/tcorr"], "comp": d[k + "/comp"]}
        cases[case]["variants"][var] = (method, sem, extra, res)
    return cases
