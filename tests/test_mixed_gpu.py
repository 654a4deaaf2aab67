"""Mixed-precision path (FP32 correction V-cycle in an FP64 defect-correction
loop) against the FP64 oracle (needs a GB300).

Both paths stop when the FP64 residual norm falls below the tolerance, so
they stop at slightly different iterates; the stated error bound is the
max-norm difference of phi after the time steps, relative to max |phi|.
"""
import numpy as np
import pytest

from tests import hierarchies as H
from tests.test_parity_gpu import CH2, CH3, uniform_spec, make_pair, PERIODIC2, PERIODIC3, NEUMANN2, DIRICHLET3

pytestmark = pytest.mark.gpu

MIXED_CASES = {
    "ch2d-periodic-64": (CH2, lambda: uniform_spec(2, 64, PERIODIC2), 1e-9, 2e-7),
    "ch2d-neumann-64": (CH2, lambda: uniform_spec(2, 64, NEUMANN2), 1e-9, 2e-7),
    "ch3d-periodic-32": (CH3, lambda: uniform_spec(3, 32, PERIODIC3), 1e-8, 2e-6),
    "ch3d-dirichlet-16": (CH3, lambda: uniform_spec(3, 16, DIRICHLET3), 1e-8, 2e-6),
    "ch2d-amr-periodic": (CH2, lambda: H.amr2d(periodic=True), 1e-9, 2e-6),
}


@pytest.mark.parametrize("case", list(MIXED_CASES))
def test_mixed_converges_to_fp64_solution(pkg, ctx, oracle_mod, case):
    cfg, mk, tol, bound = MIXED_CASES[case]
    spec = mk()
    g, o = make_pair(pkg, ctx, oracle_mod, cfg, spec)
    nd = cfg["ndims"]
    for p in spec.patches:
        shape = tuple(p["mx"][:nd])
        q = pkg.initial.ch_spinodal(shape, cfg["params"][1], p["dx"][0], seed=31 + p["id"])
        g.put(p["id"], "q", q)
        o.put(p["id"], "q", q)
    fin, mn = spec.finest(), spec.minlevel()
    for step in range(3):
        ng, rg = g.time_step(step == 0, fin, mn, tol=tol, maxvcycles=30, mode="mixed")
        no, ro = o.time_step(step == 0, fin, mn, tol=tol, maxvcycles=30)
        assert rg[-1] < tol, (step, rg)
        assert ng <= no + 3, (step, ng, no, rg, ro)
    worst = 0.0
    for p in spec.patches:
        a, b = g.get(p["id"], "q"), o.get(p["id"], "q")
        n = a.size // 2
        worst = max(worst, float(np.max(np.abs(a[:n] - b[:n])) / np.max(np.abs(b[:n]))))
    print(f"{case}: mixed vs FP64 oracle, max rel error of phi = {worst:.3e}")
    assert worst <= bound
