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


def oracle_sensitivity(oracle_mod, cfg, st, run, names=ALL, eps=2.2e-16, seed=1):
    """Per-part relative change of the oracle's result when every input value
    is multiplied by (1 + eps * N(0,1)): the rounding-level conditioning
    floor of that result.  run(oracle) performs the calls under test."""
    rng = np.random.default_rng(seed)
    pert = {k: v * (1.0 + eps * rng.standard_normal(v.shape)) for k, v in st.items()}
    outs = []
    for s in (st, pert):
        o = oracle_mod.Oracle.from_config(cfg)
        o.setup()
        o.set_state(s)
        run(o)
        outs.append(o.get_state())
    return compare(outs[1], outs[0], names=names)


def bad_parts(errs, prog_tol, hist_tol, floor=None, factor=4.0):
    """Parts above their bar: prog_tol for prognostic arrays, hist_tol for the
    rest, each raised to factor x the conditioning floor where one is given."""
    bad = {}
    for k, e in errs.items():
        tol = prog_tol if k in PROG else hist_tol
        if floor is not None:
            tol = max(tol, factor * floor.get(k, 0.0))
        if e >= tol:
            bad[k] = e
    return bad


def check(gpu, ref, prog_tol, hist_tol, sensitivity=None):
    """Prognostic physical modes to prog_tol; histories, Nyquist slots and the
    (0,0) plane averages to hist_tol.  If a part misses its bar and
    sensitivity() (the oracle's conditioning floor, oracle_sensitivity) is
    given, the bar of that part becomes 4x its floor."""
    errs = compare(gpu, ref)
    bad = bad_parts(errs, prog_tol, hist_tol)
    if bad and sensitivity is not None:
        floor = sensitivity()
        bad = bad_parts(errs, prog_tol, hist_tol, floor)
        assert not bad, (bad, errs, {k: floor.get(k) for k in bad})
    assert not bad, (bad, errs)
    return errs
