"""Helpers shared by the GPU parity tests (GPU engine vs CPU oracle)."""
import numpy as np

STATE_FIELDS = ["position", "velocity", "massDensity", "specificThermalEnergy", "H", "pressure", "soundSpeed",
                "omegaGradh"]
DERIV_FIELDS = ["massDensitySum", "normalization", "DxDt", "DvDt", "DrhoDt", "DepsDt", "DvDx", "internalDvDx",
                "gradRho", "M", "localM", "maxViscousPressure", "effViscousPressure", "DHDt", "Hideal",
                "massZerothMoment", "massFirstMoment"]


def rel_err(a, b):
    """Normwise relative error per field: max|a - b| / max|b| (max|b| floored
    at the tiniest positive double so all-zero fields compare exactly)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = max(np.max(np.abs(b)), 1e-300)
    return float(np.max(np.abs(a - b)) / scale)


def elementwise_rel_err(a, b, floor_frac=1e-3):
    """max_i |a_i - b_i| / max(|b_i|, floor_frac * max|b|)."""
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    floor = max(floor_frac * np.max(np.abs(b)), 1e-300)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor)))


def compare_fields(eng, orc, names, tol, elementwise_tol=None):
    bad = {}
    for name in names:
        a = eng.field(name)
        b = orc.field(name)
        e = rel_err(a, b)
        ee = elementwise_rel_err(a, b) if elementwise_tol else 0.0
        if e > tol or (elementwise_tol and ee > elementwise_tol):
            bad[name] = (e, ee)
    return bad


def ordered_pairs_from_oracle(orc, periodic_axes):
    i, j, im = orc.pairs()
    s = set()
    for a, b, c in zip(i.tolist(), j.tolist(), im.tolist()):
        s.add((a, b, c))
        inv = 0
        for ax in range(3):
            code = (c >> (2 * ax)) & 3
            if code and ax in periodic_axes:
                code = 3 - code
            inv |= code << (2 * ax)
        s.add((b, a, inv))
    return s


def periodic_axes(problem):
    return tuple(b["axis"] for b in problem.boundaries if b["type"] == 0)
