"""Comparison helpers for parity tests (GPU result vs oracle result)."""
import numpy as np

PHASE_RMS_TOL = 1e-3     # rad, wrapped difference, dates referenced to mini-1
TCORR_TOL = 1e-4         # absolute


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
    cgc, coc = g["comp"][both], o["comp"][both]
    den = np.maximum(np.abs(coc), 1e-6)
    dc = float(np.max(np.abs(cgc - coc) / den)) if cgc.size else 0.0
    return {
        "valid_both": int(both.sum()),
        "valid_only_gpu": int((vg & ~vo).sum()),
        "valid_only_oracle": int((vo & ~vg).sum()),
        "code_mismatch": int((cg != co).sum()),
        "phase_rms": rms,
        "phase_max": mx,
        "tcorr_max": dt,
        "comp_rel_max": dc,
        # skipped pixels must be exactly zero in both
        "zero_mismatch": int(((~vg) & (~vo) & (cg == co) &
                              ((np.abs(g["phase"]).sum(axis=0) != 0) |
                               (np.abs(o["phase"]).sum(axis=0) != 0))).sum()),
    }


def assert_parity(m, phase_tol=PHASE_RMS_TOL, tcorr_tol=TCORR_TOL, max_code_mismatch=0):
    assert m["code_mismatch"] <= max_code_mismatch, m
    assert m["phase_rms"] <= phase_tol, m
    assert m["tcorr_max"] <= tcorr_tol, m
    assert m["zero_mismatch"] == 0, m


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
