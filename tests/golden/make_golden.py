"""Generate the golden fixtures in tests/golden/ (test infrastructure).

lamb_<name>.npz : a seeded state and its dealiased Lamb vector H1, H2, H3
                  evaluated in extended precision (tests/exact_lamb.py).
steps_<name>.npz: the same state after the reference start-up (getnonlinear,
                  solve) and after 1 and 5 further steps of the oracle.
Run from the repository root: python tests/golden/make_golden.py
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

import numpy as np  # noqa: E402

import oracle  # noqa: E402
from channel_flow_gb300 import config, fields  # noqa: E402
from exact_lamb import lamb  # noqa: E402

CASES = {
    "tiny8": config.small(nnx=8, nny=4, nnz=8, aphi=1.0, beta=0.5, dt=5e-4, re=180.0, re_p=1.0),
    "tiny12": config.small(nnx=12, nny=8, nnz=10, aphi=0.75, beta=1.5, dt=1e-3, re=500.0, re_p=0.004),
}


def state(cfg, seed):
    return fields.reference_like_state(cfg, seed=seed, epsilon=0.3, noise=0.02, gamma=5.0)


def main():
    for name, cfg in CASES.items():
        st = state(cfg, 11)
        h1, h2, h3 = lamb(cfg, st)
        np.savez_compressed(os.path.join(HERE, f"lamb_{name}.npz"), h1=h1, h2=h2, h3=h3,
                            **{"in_" + k: v for k, v in st.items()})
        o = oracle.Oracle.from_config(cfg)
        o.setup()
        o.set_state(st)
        o.getnonlinear()
        o.solve()
        s0 = o.get_state()
        o.step(1)
        s1 = o.get_state()
        o.step(4)
        s5 = o.get_state()
        out = {"in_" + k: v for k, v in st.items()}
        out.update({"s0_" + k: v for k, v in s0.items()})
        out.update({"s1_" + k: v for k, v in s1.items()})
        out.update({"s5_" + k: v for k, v in s5.items()})
        np.savez_compressed(os.path.join(HERE, f"steps_{name}.npz"), **out)
        print("wrote", name)


if __name__ == "__main__":
    main()
