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


def compare(gpu, ref, names=ALL, scale=None):
    """Per-array relative L2 error; arrays whose reference norm is below
    1e-14 * scale are compared absolutely against scale."""
    if scale is None:
        scale = max(np.linalg.norm(ref[k]) for k in names)
    out = {}
    for k in names:
        nb = np.linalg.norm(ref[k])
        if nb < 1e-14 * scale:
            out[k] = np.linalg.norm(gpu[k] - ref[k]) / scale
        else:
            out[k] = rel_l2(gpu[k], ref[k])
    return out


def worst(errs):
    k = max(errs, key=errs.get)
    return k, errs[k]


def check(gpu, ref, prog_tol, hist_tol):
    errs = compare(gpu, ref)
    bad = {k: e for k, e in errs.items() if e >= (prog_tol if k in PROG else hist_tol)}
    assert not bad, (bad, errs)
    return errs
