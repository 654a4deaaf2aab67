"""Regenerates the regression fixtures of tests/golden from the CPU oracle.

The reference ships no tests, golden vectors or fixtures, and it cannot be
built here (Fortran), so these fixtures are the oracle's own outputs on
small seeded cases: they pin the oracle against later changes of itself
(tests/test_golden_cpu.py) and give the CUDA library fixed targets
(tests/test_golden_gpu.py).  Run from the repository root:

    python tests/golden/make_golden.py
"""
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import bsam_oracle as om  # noqa: E402

CASES = {
    # name: (ndims, nrvars, problem, params, n, minlevel, mthbc)
    "ch2d_periodic_16": (2, 2, "ch", [1e-3, 0.01], 16, -3, [2, 2, 2, 2, 10, 10]),
    "ch3d_dirichlet_8": (3, 2, "ch", [5e-4, 0.02], 8, -2, [10] * 6),
    "bio2d_neumann_16": (2, 2, "biogrowth", [0.1, 0.05, 1.5, 2.0, 0.5], 16, -3, [10] * 6),
    "growth3d_8": (3, 3, "growth", [0.01, 0.025, 1.5, 2.0, 0.5, 1.0], 8, -2, [10] * 6),
}


def build(name):
    nd, nv, prob, params, n, mn, mthbc = CASES[name]
    o = om.OracleHierarchy(nd, nv, prob, params)
    o.build_uniform([n] * nd + [1] * (3 - nd), mn, mthbc, [0, 0, 0], [1, 1, 1])
    o.commit()
    return o


def inputs(name, o):
    """Seeded fields of the root (q, qold, f) in the Fortran layout."""
    rng = np.random.default_rng(sum(map(ord, name)))
    out = {}
    for fld in ("q", "qold", "f"):
        out[fld] = rng.uniform(-1, 1, size=o.field_size(0, fld))
    return out


def run(name, fields):
    """SetGhost, one V-cycle from the root, then one time step; returns
    the root q after each and the step's residual history."""
    o = build(name)
    nd, nv, prob, params, n, mn, mthbc = CASES[name]
    for fld, a in fields.items():
        o.put(0, fld, a)
    o.set_ghost(0, 0)
    o.vcycle(0, mn, 2)
    q_vcycle = o.get(0, "q")
    ncyc, res = o.time_step(False, 0, mn, tol=1e-10, maxvcycles=12)
    return q_vcycle, o.get(0, "q"), np.array(res), ncyc


def main():
    for name in CASES:
        o = build(name)
        fields = inputs(name, o)
        qv, qs, res, ncyc = run(name, fields)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), q=fields["q"], qold=fields["qold"], f=fields["f"],
                            q_vcycle=qv, q_step=qs, residuals=res, ncycles=ncyc)
        print(name, "ncycles", ncyc, "final residual", res[-1] if len(res) else None)
    vals = np.array([0.0, -0.0, 2.0 ** -13, -(2.0 ** -13), 1e-13, 0.5, -1.25, 1234.5678901234567, 1e11, 1e12, -1e11,
                     float("nan"), float("inf"), -float("inf")])
    np.savez_compressed(os.path.join(HERE, "f25.npz"), values=vals,
                        text=np.array([om.format_f25(v) for v in vals]))


if __name__ == "__main__":
    main()
