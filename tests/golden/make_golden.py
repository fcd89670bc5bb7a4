"""Generates the golden fixtures of tests/golden from the CPU oracle.

    python tests/golden/make_golden.py

eos_points.npz       2000 seeded (p, T, y1, y2) -> deteos_prop dv(18), tv(2)
residual_<case>.npz  seeded case at reduced size: residual of the initial state and the
                     padded pv after one LU-SGS pseudo-iteration
The reference cannot be built here, so these vectors pin the oracle against regressions
and give the GPU tests a second anchor; they are not reference outputs.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from cfd3d_gb300 import cases  # noqa: E402
from oracle import oracle_py  # noqa: E402


def main():
    rng = np.random.default_rng(2024)
    n = 2000
    p = rng.uniform(2e3, 3e5, n)
    t = rng.uniform(280.0, 320.0, n)
    y1 = rng.uniform(0.0, 0.3, n) * (rng.uniform(size=n) < 0.3)
    y2 = 10.0 ** rng.uniform(-7, -3, n)
    dv, tv = oracle_py.eos(p, t, y1, y2, prop=True)
    np.savez_compressed(os.path.join(HERE, "eos_points.npz"), p=p, t=t, y1=y1, y2=y2, dv=dv, tv=tv)
    for name, scale in (("plain_small", 8), ("cavitating", 16)):
        c = cases.make(name, scale=scale)
        o = oracle_py.Oracle(c)
        o.initialize(c["pv0"])
        res = o.residual(0)["res"]
        o.iterate(1, 1)
        pv1 = o.get_state(0)["pv"]
        np.savez_compressed(os.path.join(HERE, f"residual_{name}.npz"), scale=scale, res=res, pv1=pv1)
    print("golden fixtures written")


if __name__ == "__main__":
    main()
