"""AMR regrid of the library (bsamg_regrid) vs the oracle's restatement, and
time steps on regridded meshes (needs a GB300).

The regrid itself is host work in both (tagging, clustering, prolongation);
the library executes SetGhost through its compiled ghost programs and hands
the new mesh to the device.  Patch tables must be identical and every field
value bit-identical; time steps on the new mesh then run the plain FP64 path,
whose parity with the oracle is bit-exact per V-cycle.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EPS = 0.01
RTOL = 1e-12


def circle2d(eps=EPS):
    def fn(level, mx, dx, xl):
        n = [m + 2 for m in mx]
        x = xl[0] + (np.arange(n[0]) - 0.5) * dx[0]
        y = xl[1] + (np.arange(n[1]) - 0.5) * dx[1]
        X, Y = np.meshgrid(x, y, indexing="ij")
        q = np.zeros(n + [2], order="F")
        q[..., 0] = np.tanh((np.sqrt((X - 0.5) ** 2 + (Y - 0.5) ** 2) - 0.25) / (math.sqrt(2) * eps))
        return q
    return fn


def sphere3d(eps=0.05):
    def fn(level, mx, dx, xl):
        n = [m + 2 for m in mx]
        ax = [xl[d] + (np.arange(n[d]) - 0.5) * dx[d] for d in range(3)]
        X, Y, Z = np.meshgrid(*ax, indexing="ij")
        q = np.zeros(n + [2], order="F")
        q[..., 0] = np.tanh((np.sqrt((X - 0.5) ** 2 + (Y - 0.45) ** 2 + (Z - 0.5) ** 2) - 0.3) / (math.sqrt(2) * eps))
        return q
    return fn


def pair(pkg, ctx, oracle_mod, nd, n, periodic, fn, params=(1e-3, EPS)):
    g = pkg.Hierarchy(ctx, nd, 2, "ch", list(params))
    o = oracle_mod.OracleHierarchy(nd, 2, "ch", list(params))
    if nd == 2:
        mthbc = [2, 2, 2, 2, 10, 10] if periodic else [10] * 6
        mx = [n, n, 1]
    else:
        mthbc = [2] * 6 if periodic else [10] * 6
        mx = [n, n, n]
    minlevel = -int(math.log2(n)) + 1
    for h in (g, o):
        h.build_uniform(mx, minlevel, mthbc, [0, 0, 0], [1, 1, 1])
        h.commit()
        h.put(0, "q", fn(0, mx[:nd], [1.0 / n] * nd, [0.0] * nd))
    return g, o, minlevel


def same(g, o):
    tg, to = g.patch_table(), o.patch_table()
    assert len(tg) == len(to)
    for a, b in zip(tg, to):
        for k in ("level", "id", "parent_id", "mx", "mglobal", "mbounds", "mthbc"):
            assert a[k] == b[k], (k, a, b)
        assert a["dx"] == b["dx"] and a["xlower"] == b["xlower"]
    for p in tg:
        for fld in ("q", "qold"):
            x, y = g.get(p["id"], fld), o.get(p["id"], fld)
            bad = np.flatnonzero(x != y)
            assert bad.size == 0, (p["id"], fld, bad[:5], x[bad[:5]], y[bad[:5]])
    return tg


def test_initial_mesh_2d_matches_oracle(pkg, ctx, oracle_mod):
    g, o, _ = pair(pkg, ctx, oracle_mod, 2, 64, True, circle2d())
    prm = pkg.regrid_params(3, tagging="gradient", initial=True, maxside=64, qtolerance=0.25)
    oprm = oracle_mod.regrid_params(3, tagging="gradient", initial=True, maxside=64, qtolerance=0.25)
    g2 = g.regrid(prm, circle2d())
    o2 = oracle_mod.regrid(o, oprm, circle2d())
    tab = same(g2, o2)
    assert max(p["level"] for p in tab) == 3


def test_regrid_after_steps_2d_neumann_matches_oracle(pkg, ctx, oracle_mod):
    g, o, mn = pair(pkg, ctx, oracle_mod, 2, 64, False, circle2d())
    prm = pkg.regrid_params(2, tagging="ch", initial=True, qtolerance=0.02)
    oprm = oracle_mod.regrid_params(2, tagging="ch", initial=True, qtolerance=0.02)
    g, o = g.regrid(prm, circle2d()), oracle_mod.regrid(o, oprm, circle2d())
    same(g, o)
    for step in range(2):
        fin = max(p["level"] for p in g.patch_table())
        ng, rg = g.time_step(step == 0, fin, mn, tol=1e-9, maxvcycles=30)
        no, ro = o.time_step(step == 0, fin, mn, tol=1e-9, maxvcycles=30)
        assert ng == no
        prm = pkg.regrid_params(2, tagging="ch", initial=False, qtolerance=0.02, first_id=2000 * (step + 1))
        oprm = oracle_mod.regrid_params(2, tagging="ch", initial=False, qtolerance=0.02, first_id=2000 * (step + 1))
        g, o = g.regrid(prm), oracle_mod.regrid(o, oprm)
        same(g, o)


def test_regrid_3d_matches_oracle(pkg, ctx, oracle_mod):
    g, o, mn = pair(pkg, ctx, oracle_mod, 3, 16, True, sphere3d(), params=(5e-4, 0.05))
    prm = pkg.regrid_params(2, tagging="ch", initial=True, qtolerance=0.05)
    oprm = oracle_mod.regrid_params(2, tagging="ch", initial=True, qtolerance=0.05)
    g2, o2 = g.regrid(prm, sphere3d()), oracle_mod.regrid(o, oprm, sphere3d())
    tab = same(g2, o2)
    assert max(p["level"] for p in tab) >= 1
    prm = pkg.regrid_params(2, tagging="ch", initial=False, qtolerance=0.05, first_id=3000)
    oprm = oracle_mod.regrid_params(2, tagging="ch", initial=False, qtolerance=0.05, first_id=3000)
    same(g2.regrid(prm), oracle_mod.regrid(o2, oprm))


def test_regrid_every_step_matches_oracle(pkg, ctx, oracle_mod):
    """TakeTimeSteps with AMR: regrid, then one time step, four times."""
    g, o, mn = pair(pkg, ctx, oracle_mod, 2, 64, True, circle2d())
    for step in range(4):
        kw = dict(tagging="gradient", initial=step == 0, maxside=64, qtolerance=0.25, first_id=1000 * (step + 1))
        g = g.regrid(pkg.regrid_params(3, **kw), circle2d() if step == 0 else None)
        o = oracle_mod.regrid(o, oracle_mod.regrid_params(3, **kw), circle2d() if step == 0 else None)
        tab = same(g, o)
        fin = max(p["level"] for p in tab)
        ng, rg = g.time_step(step == 0, fin, mn, tol=1e-9, maxvcycles=30)
        no, ro = o.time_step(step == 0, fin, mn, tol=1e-9, maxvcycles=30)
        assert ng == no, (step, rg, ro)
        np.testing.assert_allclose(rg, ro, rtol=1e-10, atol=0)
        worst = 0.0
        for p in tab:
            a, b = g.get(p["id"], "q"), o.get(p["id"], "q")
            worst = max(worst, float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)))
        assert worst <= RTOL, (step, worst)


def test_growth3d_regrid_and_steps_match_oracle(pkg, ctx, oracle_mod):
    """The three-variable growth plugin on a regridded 3D mesh (cfg4's shape
    at 16^3): meshes, fields and time steps as the oracle's."""
    params = [0.01, 0.025, 1.5, 2.0, 0.5, 1.0]
    fn = pkg.initial.growth_sphere(0.025, seed=9, radius=0.25)
    g = pkg.Hierarchy(ctx, 3, 3, "growth", params)
    o = oracle_mod.OracleHierarchy(3, 3, "growth", params)
    for h in (g, o):
        h.build_uniform([16, 16, 16], -3, [10] * 6, [0, 0, 0], [1, 1, 1])
        h.commit()
        h.put(0, "q", fn(0, [16] * 3, [1 / 16] * 3, [0.0] * 3))
    for step in range(3):
        kw = dict(tagging="gradient", initial=step == 0, qtolerance=0.25, first_id=1000 * (step + 1))
        g = g.regrid(pkg.regrid_params(2, **kw), fn if step == 0 else None)
        o = oracle_mod.regrid(o, oracle_mod.regrid_params(2, **kw), fn if step == 0 else None)
        tab = same(g, o)
        fin = max(p["level"] for p in tab)
        assert fin >= 1
        ng, rg = g.time_step(step == 0, fin, -3, tol=1e-9, maxvcycles=30)
        no, ro = o.time_step(step == 0, fin, -3, tol=1e-9, maxvcycles=30)
        assert ng == no, (step, rg, ro)
        np.testing.assert_allclose(rg, ro, rtol=1e-10, atol=0)
