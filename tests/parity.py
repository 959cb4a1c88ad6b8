"""Helpers for comparing a GPU state with the oracle's (test-only)."""
import numpy as np

from channel_flow_gb300.fields import FIELD_NAMES, MEAN_NAMES

ALL = FIELD_NAMES + MEAN_NAMES
# prognostic arrays: held to the strict bars
PROG = FIELD_NAMES + ("au0", "w0")
# (0,0)-mode Lamb histories: plane averages of products with heavy
# cancellation (sum |terms| / |result| ~ 1e3..1e6), so their relative error
# is set by the conditioning of the reference algorithm itself
HIST = ("clamb1n", "clamb1nm1", "clamb3n", "clamb3nm1")


def rel_l2(a, b, floor=1e-300):
    na = np.linalg.norm(b)
    return np.linalg.norm(a - b) / max(na, floor)


def split(a, name):
    """Field arrays split into the physical modes, the spanwise Nyquist slot
    (never used by the reference's transforms; it only carries history
    values) and the (0,0) mode (the ill-conditioned plane average H1/H3 right
    after getnonlinear)."""
    if name not in FIELD_NAMES:
        return {name: a}
    nyq = a.shape[1] // 2
    phys = a.copy()
    phys[:, nyq, :] = 0.0
    phys[:, 0, :2] = 0.0
    return {name: phys, name + "@nyq": a[:, nyq, :], name + "@00": a[:, 0, :2]}


def compare(gpu, ref, names=ALL):
    """Per-part relative L2 error; parts whose reference norm is below 1e-14
    of the largest part are compared absolutely against that scale."""
    g, r = {}, {}
    for k in names:
        g.update(split(gpu[k], k))
        r.update(split(ref[k], k))
    scale = max(np.linalg.norm(v) for v in r.values())
    out = {}
    for k in r:
        nb = np.linalg.norm(r[k])
        if "@" in k:
            # Nyquist slot / (0,0) plane average: relative to the whole field,
            # since for smooth states these parts are rounding noise
            whole = np.linalg.norm(ref[k.split("@")[0]])
            out[k] = np.linalg.norm(g[k] - r[k]) / max(nb, whole, 1e-300)
        elif nb < 1e-14 * scale:
            out[k] = np.linalg.norm(g[k] - r[k]) / scale
        else:
            out[k] = rel_l2(g[k], r[k])
    return out


def worst(errs):
    k = max(errs, key=errs.get)
    return k, errs[k]


def check(gpu, ref, prog_tol, hist_tol):
    """Prognostic physical modes to prog_tol; histories, Nyquist slots and the
    (0,0) plane averages to hist_tol."""
    errs = compare(gpu, ref)
    bad = {k: e for k, e in errs.items() if e >= (prog_tol if k in PROG else hist_tol)}
    assert not bad, (bad, errs)
    return errs
