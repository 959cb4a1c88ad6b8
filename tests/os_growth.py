"""Growth of a seeded Orr-Sommerfeld eigenmode, measured from a run.

The run starts from fields.orr_sommerfeld_state: laminar Poiseuille flow plus
the least-stable 2D eigenmode of streamwise mode kx = 1 at amplitude 1e-6, so
the perturbation stays linear.  Every ``chunk`` steps the state is read back
and two histories are kept:

* the complex amplitude A(t) of the v coefficients of mode (kx=1, ky=0)
  projected on the initial profile: A ~ exp(sigma t), so the slope of log A
  gives sigma (growth rate and phase speed);
* the perturbation energy E(t), the Chebyshev-coefficient energy of u, v, w
  over every mode but (0,0): E ~ exp(2 Re(sigma) t).

The first ``skip`` samples are left out of the fits: the run starts with zero
nonlinear-term histories (rhsvn, rhsomegayn; the AB2 sums at
poiseuilleflow.f90:253-256 then lack their second term), so the first step
is off by O(dt) and excites a small transient.
"""
import numpy as np

from channel_flow_gb300 import fields


def _perturbation_energy(st):
    e = 0.0
    for name in ("unp1", "vnp1", "wnp1"):
        a = fields.as_complex(st[name]).copy()
        a[:, 0, 0] = 0.0
        nyq = a.shape[1] // 2
        a[:, nyq, :] = 0.0
        e += float(np.sum(np.abs(a) ** 2))
    return e


def run_history(step, read, st0, cfg, nsteps, chunk):
    """step(n) advances n steps, read() returns the state dict."""
    a0 = fields.as_complex(st0["vnp1"])[:, 0, 1].copy()
    phi = a0 / np.linalg.norm(a0)
    ref = np.vdot(phi, a0)
    t, amp, en = [], [], []
    for i in range(nsteps // chunk):
        step(chunk)
        st = read()
        a = fields.as_complex(st["vnp1"])[:, 0, 1]
        t.append((i + 1) * chunk * cfg.dt)
        amp.append(np.vdot(phi, a) / ref)
        en.append(_perturbation_energy(st))
    return np.array(t), np.array(amp), np.array(en)


def fit_rates(t, amp, en, skip):
    """(sigma from the amplitude history, Re(sigma) from the energy history)."""
    la = np.log(amp[skip:])
    re = np.polyfit(t[skip:], la.real, 1)[0]
    im = np.polyfit(t[skip:], np.unwrap(la.imag), 1)[0]
    er = 0.5 * np.polyfit(t[skip:], np.log(en[skip:]), 1)[0]
    return complex(re, im), er
