"""Known answers for the oracle's AMR regrid (no GPU).

The regrid (bsamroutines.f90:657-689, :966-1951) is pinned by properties
that hold for the reference's algorithm: children nest in their parents and
follow NewSubGrids' size rules (even lengths, odd starts, at least
minimumgridpoints coarse cells), siblings do not overlap, every buffered tag
is covered by a child (Berger-Rigoutsos clusters all tagged cells), the
mass-corrected prolongation of InitFields keeps every parent cell's value
as the mean of its children, TransferValues carries previous values, and the
result is deterministic.
"""
import math

import numpy as np
import pytest

from tests import hierarchies as H

EPS = 0.01


def circle(eps=EPS, cx=0.5, cy=0.5, r0=0.25):
    def fn(level, mx, dx, xl):
        n = [m + 2 for m in mx]
        x = xl[0] + (np.arange(n[0]) - 0.5) * dx[0]
        y = xl[1] + (np.arange(n[1]) - 0.5) * dx[1]
        X, Y = np.meshgrid(x, y, indexing="ij")
        q = np.zeros(n + [2], order="F")
        q[..., 0] = np.tanh((np.sqrt((X - cx) ** 2 + (Y - cy) ** 2) - r0) / (math.sqrt(2) * eps))
        return q
    return fn


def root2d(oracle_mod, n=64, periodic=True, fn=None):
    o = oracle_mod.OracleHierarchy(2, 2, "ch", [1e-3, EPS])
    mthbc = [2, 2, 2, 2, 10, 10] if periodic else [10] * 6
    o.build_uniform([n, n, 1], -int(math.log2(n)) + 1, mthbc, [0, 0, 0], [1, 1, 1])
    o.commit()
    o.put(0, "q", (fn or circle())(0, [n, n], [1.0 / n] * 2, [0.0, 0.0]))
    return o


def tags(q, mx, rule, tol, nd=2):
    phi = q[..., 0]
    c = tuple(slice(1, m + 1) for m in mx)
    if rule == "ch":
        s = 0
        for d in range(nd):
            lo = tuple(slice(0, m) if e == d else slice(1, m + 1) for e, m in enumerate(mx))
            hi = tuple(slice(2, m + 2) if e == d else slice(1, m + 1) for e, m in enumerate(mx))
            s = s + np.abs(phi[hi] - 2.0 * phi[c] + phi[lo])
        return s > nd * tol
    g = 0
    for d in range(nd):
        lo = tuple(slice(0, m) if e == d else slice(1, m + 1) for e, m in enumerate(mx))
        hi = tuple(slice(2, m + 2) if e == d else slice(1, m + 1) for e, m in enumerate(mx))
        g = g + ((phi[hi] - phi[lo]) * 0.5) ** 2
    return g > tol * tol


def check_structure(tab, mgp=4, maxside=0, nd=2):
    by_id = {p["id"]: p for p in tab}
    for p in tab:
        if p["level"] <= 0:
            continue
        par = by_id[p["parent_id"]]
        for d in range(nd):
            lo, hi = p["mbounds"][2 * d], p["mbounds"][2 * d + 1]
            assert 1 <= lo <= hi <= par["mx"][d]
            assert lo % 2 == 1 and hi % 2 == 0 and hi - lo + 1 >= mgp
            assert p["mx"][d] == 2 * (hi - lo + 1)
            if maxside:
                assert p["mx"][d] <= maxside
            g0 = par["mglobal"][2 * d] + lo - 1
            assert p["mglobal"][2 * d] == 2 * g0 - 1
            assert p["mglobal"][2 * d + 1] - p["mglobal"][2 * d] + 1 == p["mx"][d]
    levels = sorted({p["level"] for p in tab if p["level"] > 0})
    for l in levels:
        ps = [p for p in tab if p["level"] == l]
        for a in range(len(ps)):
            for b in range(a + 1, len(ps)):
                overlap = all(max(ps[a]["mglobal"][2 * d], ps[b]["mglobal"][2 * d]) <=
                              min(ps[a]["mglobal"][2 * d + 1], ps[b]["mglobal"][2 * d + 1]) for d in range(nd))
                assert not overlap, (ps[a]["id"], ps[b]["id"])


def test_initial_mesh_structure_and_coverage(oracle_mod):
    om = oracle_mod
    o = root2d(om)
    prm = om.regrid_params(3, tagging="gradient", initial=True, maxside=64, qtolerance=0.25, ibuffer=1)
    n = om.regrid(o, prm, circle())
    tab = n.patch_table()
    levels = {p["level"] for p in tab}
    assert {1, 2, 3} <= levels
    check_structure(tab, maxside=64)
    # every tagged (and buffered) cell of level l lies under a level-(l+1) child
    for l in (0, 1, 2):
        kids = [p for p in tab if p["level"] == l + 1]
        covered = set()
        for c in kids:
            for gx in range(c["mglobal"][0], c["mglobal"][1] + 1, 2):
                for gy in range(c["mglobal"][2], c["mglobal"][3] + 1, 2):
                    covered.add(((gx + 1) // 2, (gy + 1) // 2))
        nglob = 64 << l
        for p in [p for p in tab if p["level"] == l]:
            mx = p["mx"][:2]
            q = n.get(p["id"], "q").reshape(mx[0] + 2, mx[1] + 2, 2, order="F")
            t = tags(q, mx, "gradient", 0.25)
            for i, j in zip(*np.nonzero(t)):
                g = (i + p["mglobal"][0], j + p["mglobal"][2])
                for di in (-1, 0, 1):  # ibuffer = 1, periodic images
                    for dj in (-1, 0, 1):
                        cell = ((g[0] + di - 1) % nglob + 1, (g[1] + dj - 1) % nglob + 1)
                        inside = any(pp["mglobal"][0] <= cell[0] <= pp["mglobal"][1] and
                                     pp["mglobal"][2] <= cell[1] <= pp["mglobal"][3]
                                     for pp in tab if pp["level"] == l)
                        if inside:
                            assert cell in covered, (l, cell)


def test_prolongation_conserves_each_parent_cell(oracle_mod):
    om = oracle_mod
    o = root2d(om, periodic=False)
    prm = om.regrid_params(1, tagging="ch", initial=False, qtolerance=1e-3, ibuffer=1)
    n = om.regrid(o, prm)
    tab = n.patch_table()
    kids = [p for p in tab if p["level"] == 1]
    assert kids
    root = n.get(0, "q").reshape(66, 66, 2, order="F")
    for c in kids:
        mx = c["mx"][:2]
        q = n.get(c["id"], "q").reshape(mx[0] + 2, mx[1] + 2, 2, order="F")
        lo = (c["mbounds"][0], c["mbounds"][2])
        for v in range(2):
            fine = q[1:-1, 1:-1, v]
            mean = 0.25 * (fine[0::2, 0::2] + fine[1::2, 0::2] + fine[0::2, 1::2] + fine[1::2, 1::2])
            par = root[lo[0]:lo[0] + mx[0] // 2, lo[1]:lo[1] + mx[1] // 2, v]
            assert np.allclose(mean, par, rtol=0, atol=1e-14)


def test_transfer_keeps_previous_level_values(oracle_mod):
    om = oracle_mod
    o = root2d(om)
    prm = om.regrid_params(2, tagging="gradient", initial=True, qtolerance=0.25)
    a = om.regrid(o, prm, circle())
    # mark the finest level's values so that transferred cells are
    # recognisable (the finest level is not tagged, so the mesh stays)
    tab = a.patch_table()
    fin = max(p["level"] for p in tab)
    for p in tab:
        if p["level"] == fin:
            q = a.get(p["id"], "q")
            a.put(p["id"], "q", q + 10.0)
    prm2 = om.regrid_params(2, tagging="gradient", initial=False, qtolerance=0.25, first_id=5000)
    b = om.regrid(a, prm2)
    assert [(p["level"], p["mglobal"]) for p in b.patch_table()] == [(p["level"], p["mglobal"]) for p in tab]
    old = {tuple(p["mglobal"]): p for p in tab if p["level"] > 0}
    for p in b.patch_table():
        if p["level"] != fin:
            continue
        qa = a.get(old[tuple(p["mglobal"])]["id"], "q").reshape(p["mx"][0] + 2, p["mx"][1] + 2, 2, order="F")
        qb = b.get(p["id"], "q").reshape(p["mx"][0] + 2, p["mx"][1] + 2, 2, order="F")
        assert np.array_equal(qa[1:-1, 1:-1], qb[1:-1, 1:-1])


def test_regrid_is_deterministic_and_time_steps_converge(oracle_mod):
    om = oracle_mod
    o = root2d(om)
    prm = om.regrid_params(3, tagging="gradient", initial=True, maxside=64, qtolerance=0.25)
    a = om.regrid(o, prm, circle())
    b = om.regrid(o, prm, circle())
    assert a.patch_table() == b.patch_table()
    for p in a.patch_table():
        assert np.array_equal(a.get(p["id"], "q"), b.get(p["id"], "q"))
    fin = max(p["level"] for p in a.patch_table())
    n, res = a.time_step(True, fin, -5, tol=1e-9, maxvcycles=30)
    assert res[-1] < 1e-9
