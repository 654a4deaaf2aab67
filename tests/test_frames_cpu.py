"""Frame files, restart and after-step statistics: known answers on the CPU.

The text format is WriteQ's (LIBRARY/bsaminputoutput.f90:60-181): F25.12
reals, I3/I8 header integers, one record per ghosted cell.  F25.12 is pinned
against Python's correctly rounded '%25.12f' (ties to even), for the oracle's
formatter and for the library's own (pure host code, no GPU call).  The
statistics (AfterStepStatistics, LIBRARY/bsamroutines.f90:918-963, with
CH/problem.f90:149-215 and :518-547) are pinned by exact integrals: a
constant field, a linear field's gradient energy, and the composite mass of
a hierarchy whose parents are the restrictions of their children.
"""
import math
import random

import numpy as np
import pytest

from tests import hierarchies as H
from tests.test_regrid_cpu import circle, root2d

EPS = 0.01


def f25_expected(x):
    if math.isnan(x):
        return " " * 22 + "NaN"
    if math.isinf(x):
        s = "-Infinity" if x < 0 else "Infinity"
        return " " * (25 - len(s)) + s
    s = "%25.12f" % x
    return "*" * 25 if len(s) > 25 else s


def f25_values():
    rng = random.Random(11)
    vals = [0.0, -0.0, 2.0 ** -13, -(2.0 ** -13), 3 * 2.0 ** -14, 0.5e-12, -0.5e-12, 1e-12, 999999999999.9999,
            -99999999999.99999, 123456789012.5, 1e13, 1e300, 5e-324, -5e-324, 2.0 ** 59, 2.0 ** 60, 2.0 ** 61,
            float("nan"), float("inf"), -float("inf")]
    for _ in range(20000):
        vals.append(rng.choice([-1.0, 1.0]) * 10.0 ** rng.uniform(-16, 13))
    for k in range(1, 2000):  # exact ties at the 13th decimal
        vals += [k * 2.0 ** -13, -k * 2.0 ** -14, k * 2.0 ** -40 + 7]
    return vals


def test_oracle_f25_matches_correctly_rounded_fixed_notation(oracle_mod):
    for x in f25_values():
        assert oracle_mod.format_f25(x) == f25_expected(x), x


def test_library_f25_matches_correctly_rounded_fixed_notation(pkg):
    for x in f25_values():
        assert pkg.format_f25(x) == f25_expected(x), x


def test_stats_record_format(pkg, oracle_mod):
    for args in ((0.1, [1.5, -2.25], 12345), (2.0, [0.0, -0.0], 0), (1e-3, [1e13, 3.0], 123456789)):
        want = f25_expected(args[0]) + f25_expected(args[1][0]) + f25_expected(args[1][1]) + " "
        want += "%8d" % args[2] if args[2] < 10 ** 8 else "*" * 8
        assert oracle_mod.format_stats_line(*args) == want + "\n"
        assert pkg.format_stats_line(*args) == want + "\n"


def uniform(om, nd, n, problem="ch", params=(1e-3, EPS)):
    nv = 3 if problem == "growth" else 2
    o = om.OracleHierarchy(nd, nv, problem, list(params))
    mx = [n, n, n if nd == 3 else 1]
    o.build_uniform(mx, -int(math.log2(n)) + 1, [2] * 6 if nd == 3 else [2, 2, 2, 2, 10, 10], [0, 0, 0], [1, 1, 1])
    o.commit()
    return o


def put_fn(o, nd, n, fn, nv=2):
    ax = [(np.arange(n + 2) - 0.5) / n for _ in range(nd)]
    X = np.meshgrid(*ax, indexing="ij")
    q = np.zeros([n + 2] * nd + [nv], order="F")
    q[..., 0] = fn(*X)
    o.put(0, "q", q)


def test_stats_constant_and_linear_fields(oracle_mod):
    om = oracle_mod
    o = uniform(om, 2, 32)
    put_fn(o, 2, 32, lambda x, y: 0.3 + 0.0 * x)
    m, e, ms = o.after_step_stats(0)
    assert ms == 32 * 32
    assert abs(m - 0.3) < 1e-14
    c2 = 0.09
    assert abs(e - c2 * (c2 - 2) / 4) < 1e-14
    # phi = a x + b y: the four squared differences per cell are 2(a h)^2 +
    # 2(b h)^2, so the gradient term integrates to eps^2 (a^2 + b^2) / 2
    a, b = 0.25, -0.5
    put_fn(o, 2, 32, lambda x, y: a * x + b * y)
    m, e, _ = o.after_step_stats(0)
    assert abs(m - (a + b) / 2) < 1e-13
    h = 1 / 32
    xs = (np.arange(1, 33) - 0.5) * h
    X, Y = np.meshgrid(xs, xs, indexing="ij")
    c = a * X + b * Y
    ff = np.sum(c * c * (c * c - 2) / 4) * h * h
    assert abs(e - (ff + EPS ** 2 * (a * a + b * b) / 2)) < 1e-13
    # 3D CH: the integral of phi only; BioGrowth 3D: nothing
    o3 = uniform(om, 3, 16, params=(5e-4, 0.02))
    put_fn(o3, 3, 16, lambda x, y, z: 0.5 + x * 0)
    m, e, ms = o3.after_step_stats(0)
    assert abs(m - 0.5) < 1e-14 and e == 0.0 and ms == 16 ** 3
    b3 = uniform(om, 3, 16, problem="biogrowth", params=(1e-3, 0.05, 1.0, 1.0, 0.5))
    put_fn(b3, 3, 16, lambda x, y, z: 0.5 + x * 0)
    assert b3.after_step_stats(0)[:2] == (0.0, 0.0)


def test_composite_mass_equals_root_mass_after_fill_down(oracle_mod):
    """Each level > 0 patch adds h^d sum(q) and removes (2h)^d times its
    parent's cells under it; when the parents hold the restriction of their
    children (FillDown) the two cancel and the composite integral is the
    root's.  The composite mesh size counts every leaf cell once."""
    om = oracle_mod
    a = om.regrid(root2d(om), om.regrid_params(3, tagging="gradient", initial=True, maxside=64, qtolerance=0.25),
                  circle())
    tab = a.patch_table()
    fin = max(p["level"] for p in tab)
    a.fill_down("q", fin, -5)
    m, e, ms = a.after_step_stats(fin)
    m0, e0, ms0 = a.after_step_stats(0)
    assert ms0 == 64 * 64
    assert ms == 64 * 64 + sum(3 * p["mx"][0] * p["mx"][1] // 4 for p in tab if p["level"] > 0)
    assert abs(m - m0) < 1e-13
    assert abs(e - e0) > 1e-6  # the energy sees the finer gradients


def parse_frame(path, nd):
    """A reader of the frame format that follows the MATLAB post-processor
    (PROBLEM/MATLAB/interface2d.m): whitespace-separated numbers."""
    tok = open(path).read().split()
    t, fin = float(tok[0]), int(tok[1])
    k, blocks = 2, []
    while k < len(tok):
        level, rnd, r, nv = (int(x) for x in tok[k:k + 4])
        k += 4
        dx = [float(x) for x in tok[k:k + nd]]
        xl = [float(x) for x in tok[k + nd:k + 2 * nd]]
        xu = [float(x) for x in tok[k + 2 * nd:k + 3 * nd]]
        k += 3 * nd
        mx = [int(x) for x in tok[k:k + nd]]
        mg = [int(x) for x in tok[k + nd:k + 3 * nd]]
        k += 3 * nd
        n = int(np.prod([m + 2 for m in mx]))
        data = np.array([float(x) for x in tok[k:k + n * nv]]).reshape(n, nv)
        k += n * nv
        blocks.append(dict(level=level, ndims=rnd, r=r, nv=nv, dx=dx, xl=xl, xu=xu, mx=mx, mg=mg, data=data))
    return t, fin, blocks


def amr2d(om):
    a = om.regrid(root2d(om), om.regrid_params(2, tagging="gradient", initial=True, maxside=64, qtolerance=0.25),
                  circle())
    fin = max(p["level"] for p in a.patch_table())
    return a, fin


def test_frame_layout_and_values(oracle_mod, tmp_path):
    om = oracle_mod
    a, fin = amr2d(om)
    path = tmp_path / "m00001.dat"
    a.write_q(path, 0.125, fin)
    lines = open(path).read().split("\n")
    assert lines[0] == f25_expected(0.125) and lines[1] == "%3d" % fin and lines[2] == "  "
    assert lines[3] == "  0   2   2   2"
    assert lines[4] == f25_expected(1 / 64) + " " + f25_expected(1 / 64)
    assert lines[7] == "%8d %8d" % (64, 64) and lines[8] == "%8d %8d %8d %8d" % (1, 64, 1, 64)
    assert len(lines[9]) == 52  # two fields and one 2X
    t, f, blocks = parse_frame(path, 2)
    tab = [p for p in a.patch_table() if 0 <= p["level"] <= fin]
    assert t == 0.125 and f == fin and len(blocks) == len(tab)
    # WriteQ visits each level youngest node first (ApplyOnLevel,
    # treeops.f90:536-550): the reverse of the table's order of creation
    tab = [p for lev in range(fin + 1) for p in reversed([q for q in tab if q["level"] == lev])]
    for b, p in zip(blocks, tab):
        assert b["level"] == p["level"] and b["mx"] == p["mx"][:2] and b["mg"] == p["mglobal"][:4]
        q = a.get(p["id"], "q").reshape(-1, 2, order="F")
        assert np.max(np.abs(b["data"] - q)) <= 5.1e-13


def test_write_read_write_is_identical(oracle_mod, tmp_path):
    om = oracle_mod
    a, fin = amr2d(om)
    p1, p2 = tmp_path / "a.dat", tmp_path / "b.dat"
    a.write_q(p1, 0.5, fin)
    root = root2d(om)
    b, t = om.read_q(root, p1, first_id=500)
    assert t == 0.5
    b.write_q(p2, t, fin)
    # ReadQ creates the nodes in the file's order, so each level's youngest
    # node (written first) is the file's last block of that level: a second
    # frame lists every level's blocks in the reverse order, with the same
    # bytes per block; a third frame is the first again
    (_, _, b1), (_, _, b2) = parse_frame(p1, 2), parse_frame(p2, 2)
    key = lambda b: (b["level"], b["mg"])
    assert sorted(map(key, b1)) == sorted(map(key, b2))
    for x, y in zip(sorted(b1, key=key), sorted(b2, key=key)):
        assert np.array_equal(x["data"], y["data"]) and x["dx"] == y["dx"] and x["xl"] == y["xl"]
    c, _ = om.read_q(root2d(om), p2, first_id=900)
    p3 = tmp_path / "c.dat"
    c.write_q(p3, t, fin)
    assert open(p1).read() == open(p3).read()
    ta, tb = a.patch_table(), b.patch_table()
    assert sorted((p["level"], p["mglobal"], p["mbounds"], p["mthbc"]) for p in ta) == \
           sorted((p["level"], p["mglobal"], p["mbounds"], p["mthbc"]) for p in tb)


def test_restart_then_regrid_matches_the_uninterrupted_run(oracle_mod, tmp_path):
    """A frame written at full precision by WriteQ carries 12 decimals; after
    ReadQ the first regrid rebuilds the mesh from the root and transfers the
    restart patches' values, so meshes agree and fields agree to the
    rounding of the file."""
    om = oracle_mod
    a, fin = amr2d(om)
    a.time_step(True, fin, -5, tol=1e-9, maxvcycles=30)
    path = tmp_path / "m.dat"
    a.write_q(path, 1e-3, fin)
    b, _ = om.read_q(root2d(om), path, first_id=900)
    prm = dict(tagging="gradient", initial=False, maxside=64, qtolerance=0.25, first_id=2000)
    a2, b2 = om.regrid(a, om.regrid_params(2, **prm)), om.regrid(b, om.regrid_params(2, **prm))
    ta, tb = a2.patch_table(), b2.patch_table()
    assert [(p["level"], p["mglobal"]) for p in ta] == [(p["level"], p["mglobal"]) for p in tb]
    for p, r in zip(ta, tb):
        if p["level"] >= 0:
            assert np.max(np.abs(a2.get(p["id"], "q") - b2.get(r["id"], "q"))) <= 1e-12


def test_read_rejects_inconsistent_or_truncated_frames(oracle_mod, tmp_path):
    om = oracle_mod
    a, fin = amr2d(om)
    good = tmp_path / "g.dat"
    a.write_q(good, 0.0, fin)
    text = open(good).read().split("\n")
    cases = {
        "trunc": "\n".join(text[: len(text) // 2]),
        "ndims": "\n".join(text[:3] + ["  0   3   2   2"] + text[4:]),
        "ratio": "\n".join(text[:3] + ["  0   2   4   2"] + text[4:]),
        "dx": "\n".join(text[:4] + [f25_expected(1 / 32) + " " + f25_expected(1 / 32)] + text[5:]),
    }
    for name, body in cases.items():
        p = tmp_path / (name + ".dat")
        p.write_text(body)
        with pytest.raises(RuntimeError):
            om.read_q(root2d(om), p)
    with pytest.raises(RuntimeError):
        om.read_q(root2d(om), tmp_path / "missing.dat")


def test_uniform_mesh_of_a_linear_field_is_the_field(oracle_mod, tmp_path):
    """The mass-corrected bilinear prolongation reproduces a linear field
    (its children's mean is the coarse value, so the correction is zero);
    the patches copied over it hold the same field, so the uniform composite
    is the linear field at the finest cell centres, away from the physical
    boundary (whose reflected ghost values enter the prolongation within a
    few cells of it).  Cells under a finest patch hold that patch's values
    (to the 12 decimals of the file)."""
    om = oracle_mod
    lin = lambda x, y: 0.25 * x - 0.5 * y + 0.125
    o = om.OracleHierarchy(2, 2, "ch", [1e-3, EPS])
    o.build_uniform([32, 32, 1], -4, [10] * 6, [0, 0, 0], [1, 1, 1])
    o.commit()

    def fn(level, mx, dx, xl):
        n = [m + 2 for m in mx]
        x = xl[0] + (np.arange(n[0]) - 0.5) * dx[0]
        y = xl[1] + (np.arange(n[1]) - 0.5) * dx[1]
        X, Y = np.meshgrid(x, y, indexing="ij")
        q = np.zeros(n + [2], order="F")
        q[..., 0] = lin(X, Y)
        return q
    o.put(0, "q", fn(0, [32, 32], [1 / 32] * 2, [0.0, 0.0]))
    prm = om.regrid_params(2, tagging="ch", initial=False, qtolerance=-1.0)  # tag everything
    a = om.regrid(o, prm)
    fin = max(p["level"] for p in a.patch_table())
    assert fin == 2
    path = tmp_path / "u.dat"
    a.write_uniform_q(path, 0.0, fin)
    t, f, blocks = parse_frame(path, 2)
    assert f == 0 and len(blocks) == 1
    b = blocks[0]
    assert b["mx"] == [128, 128] and b["mg"] == [1, 128, 1, 128] and b["dx"] == [1 / 128] * 2
    full = b["data"][:, 0].reshape(130, 130, order="F")
    u = full[1:-1, 1:-1]
    xs = (np.arange(1, 129) - 0.5) / 128
    X, Y = np.meshgrid(xs, xs, indexing="ij")
    band = slice(8, 120)
    assert np.max(np.abs(u - lin(X, Y))[band, band]) < 1e-12
    for p in a.patch_table():
        if p["level"] == fin:
            q = a.get(p["id"], "q").reshape(p["mx"][0] + 2, p["mx"][1] + 2, 2, order="F")[1:-1, 1:-1, 0]
            g = p["mglobal"]
            assert np.max(np.abs(full[g[0]:g[1] + 1, g[2]:g[3] + 1] - q)) <= 5.1e-13  # 12 decimals
