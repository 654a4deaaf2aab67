"""Frame files, restart and after-step statistics of the library vs the
oracle (needs a GB300).

* bsamg_after_step_stats is a device reduction; its terms are the
  reference's, its sum order a fixed tree, so it agrees with the oracle's
  sequential sums to rounding: |lib - oracle| <= 1e-12 (the integrals are of
  order one).
* bsamg_write_q / bsamg_write_uniform_q write the same bytes as the oracle
  (the uniform composite is built on the device in the reference's
  operation order, so it is bit-identical).
* bsamg_read_q of the same file gives the same patch table and bit-identical
  fields; a restarted run regrids and steps as the oracle's does.
"""
import numpy as np
import pytest

from tests.test_regrid_gpu import circle2d, pair, same, sphere3d

pytestmark = pytest.mark.gpu

ATOL = 1e-12


def amr_pair(pkg, ctx, om, nd, n, periodic, fn, params, maxlevel, tagging, qtol):
    g, o, mn = pair(pkg, ctx, om, nd, n, periodic, fn, params=params)
    kw = dict(tagging=tagging, initial=True, maxside=64, qtolerance=qtol)
    g = g.regrid(pkg.regrid_params(maxlevel, **kw), fn)
    o = om.regrid(o, om.regrid_params(maxlevel, **kw), fn)
    tab = same(g, o)
    return g, o, mn, max(p["level"] for p in tab)


CASES = {
    "ch2d-amr-periodic": (2, 64, True, circle2d, (1e-3, 0.01), 3, "gradient", 0.25),
    "ch2d-amr-neumann": (2, 64, False, circle2d, (1e-3, 0.01), 2, "ch", 0.02),
    "ch3d-amr": (3, 16, True, sphere3d, (5e-4, 0.05), 2, "ch", 0.05),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_stats_after_steps_match_oracle(pkg, ctx, oracle_mod, case):
    nd, n, per, fn, prm, ml, tag, qt = CASES[case]
    g, o, mn, fin = amr_pair(pkg, ctx, oracle_mod, nd, n, per, fn(), prm, ml, tag, qt)
    for step in range(2):
        g.time_step(step == 0, fin, mn, tol=1e-9, maxvcycles=30)
        o.time_step(step == 0, fin, mn, tol=1e-9, maxvcycles=30)
        for f in range(fin + 1):
            mg, eg, sg = g.after_step_stats(f)
            mo, eo, so = o.after_step_stats(f)
            assert sg == so
            assert abs(mg - mo) <= ATOL and abs(eg - eo) <= ATOL, (step, f, mg - mo, eg - eo)
            if nd == 3:
                assert eg == 0.0


def test_stats_of_growth_and_biogrowth(pkg, ctx, oracle_mod):
    fn = pkg.initial.growth_sphere(0.025, seed=3, radius=0.25)
    params = [0.01, 0.025, 1.5, 2.0, 0.5, 1.0]
    for problem, nv, nd in (("growth", 3, 3), ("biogrowth", 2, 2), ("biogrowth", 2, 3)):
        g = pkg.Hierarchy(ctx, nd, nv, problem, params[: 6 if nv == 3 else 5])
        o = oracle_mod.OracleHierarchy(nd, nv, problem, params[: 6 if nv == 3 else 5])
        mx = [16, 16, 16 if nd == 3 else 1]
        for h in (g, o):
            h.build_uniform(mx, -3, [10] * 6, [0, 0, 0], [1, 1, 1])
            h.commit()
            q = fn(0, [16] * nd, [1 / 16] * nd, [0.0] * nd)[..., :nv].copy(order="F")
            h.put(0, "q", q)
            h.time_step(True, 0, -3, tol=1e-9, maxvcycles=20)
        a, b = g.after_step_stats(0), o.after_step_stats(0)
        assert a[2] == b[2] and abs(a[0] - b[0]) <= ATOL and abs(a[1] - b[1]) <= ATOL, (problem, nd, a, b)
        if problem == "biogrowth" and nd == 3:
            assert a[:2] == (0.0, 0.0)


def test_stats_on_the_periodic_box_path(pkg, ctx, oracle_mod):
    """The mixed box path keeps its iterate in float pairs and writes the FP64
    q back after every step; the statistics read that q."""
    n = 32
    g = pkg.Hierarchy(ctx, 3, 2, "ch", [5e-4, 0.02])
    g.build_uniform([n] * 3, -4, [2] * 6, [0, 0, 0], [1, 1, 1])
    g.commit()
    g.put(0, "q", pkg.initial.ch_spinodal((n,) * 3, 0.02, 1 / n, seed=4))
    for s in range(2):
        g.time_step(s == 0, 0, -4, tol=1e-8, maxvcycles=20, mode="mixed")
    o = oracle_mod.OracleHierarchy(3, 2, "ch", [5e-4, 0.02])
    o.build_uniform([n] * 3, -4, [2] * 6, [0, 0, 0], [1, 1, 1])
    o.commit()
    o.put(0, "q", g.get(0, "q"))
    a, b = g.after_step_stats(0), o.after_step_stats(0)
    assert a[2] == b[2] == n ** 3 and abs(a[0] - b[0]) <= ATOL


@pytest.mark.parametrize("case", sorted(CASES))
def test_frame_and_uniform_files_are_the_oracles(pkg, ctx, oracle_mod, case, tmp_path):
    nd, n, per, fn, prm, ml, tag, qt = CASES[case]
    g, o, mn, fin = amr_pair(pkg, ctx, oracle_mod, nd, n, per, fn(), prm, ml, tag, qt)
    g.time_step(True, fin, mn, tol=1e-9, maxvcycles=30)
    o.time_step(True, fin, mn, tol=1e-9, maxvcycles=30)
    for f in sorted({0, fin}):
        g.write_q(tmp_path / "g.dat", 0.25, f)
        o.write_q(tmp_path / "o.dat", 0.25, f)
        assert (tmp_path / "g.dat").read_bytes() == (tmp_path / "o.dat").read_bytes()
        g.write_uniform_q(tmp_path / "gu.dat", 0.25, f)
        o.write_uniform_q(tmp_path / "ou.dat", 0.25, f)
        assert (tmp_path / "gu.dat").read_bytes() == (tmp_path / "ou.dat").read_bytes()


def test_restart_matches_oracle(pkg, ctx, oracle_mod, tmp_path):
    """ReadQ of one frame into both, then TakeTimeSteps' regrid and a step:
    meshes, fields and residual histories as the oracle's."""
    om = oracle_mod
    g, o, mn, fin = amr_pair(pkg, ctx, om, 2, 64, True, circle2d(), (1e-3, 0.01), 3, "gradient", 0.25)
    g.time_step(True, fin, mn, tol=1e-9, maxvcycles=30)
    o.time_step(True, fin, mn, tol=1e-9, maxvcycles=30)
    path = tmp_path / "m00003.dat"
    o.write_q(path, 3e-3, fin)
    groot, oroot, _ = pair(pkg, ctx, om, 2, 64, True, circle2d())
    g2, tg = groot.read_q(path, first_id=700)
    o2, to = om.read_q(oroot, path, first_id=700)
    assert tg == to == 3e-3
    same(g2, o2)
    # a frame written after ReadQ lists each level in the reverse order (ReadQ
    # creates the nodes in file order, WriteQ visits youngest first), as
    # the oracle's does; written once more after reading that, it is the
    # original again
    g2.write_q(tmp_path / "again.dat", tg, fin)
    o2.write_q(tmp_path / "again_oracle.dat", tg, fin)
    assert (tmp_path / "again.dat").read_bytes() == (tmp_path / "again_oracle.dat").read_bytes()
    g4, _ = groot.read_q(tmp_path / "again.dat", first_id=800)
    g4.write_q(tmp_path / "third.dat", tg, fin)
    assert (tmp_path / "third.dat").read_bytes() == path.read_bytes()
    kw = dict(tagging="gradient", initial=False, maxside=64, qtolerance=0.25, first_id=4000)
    g3, o3 = g2.regrid(pkg.regrid_params(3, **kw)), om.regrid(o2, om.regrid_params(3, **kw))
    tab = same(g3, o3)
    fin3 = max(p["level"] for p in tab)
    ng, rg = g3.time_step(True, fin3, mn, tol=1e-9, maxvcycles=30)
    no, ro = o3.time_step(True, fin3, mn, tol=1e-9, maxvcycles=30)
    assert ng == no
    np.testing.assert_allclose(rg, ro, rtol=1e-10, atol=0)


def test_read_rejects_a_frame_of_another_grid(pkg, ctx, oracle_mod, tmp_path):
    g, o, mn = pair(pkg, ctx, oracle_mod, 2, 64, True, circle2d())
    other, _, _ = pair(pkg, ctx, oracle_mod, 2, 32, True, circle2d())
    other.write_q(tmp_path / "o.dat", 0.0, 0)
    with pytest.raises(pkg.BsamgError):
        g.read_q(tmp_path / "o.dat")
    with pytest.raises(pkg.BsamgError):
        g.read_q(tmp_path / "missing.dat")


def test_growth_amr_frames_stats_and_restart_match_oracle(pkg, ctx, oracle_mod, tmp_path):
    """The three-variable growth plugin on a regridded 3D mesh: frame and
    uniform-mesh files byte-identical to the oracle's, statistics within
    1e-12, and a restart read back into both gives the same hierarchy."""
    params = [0.01, 0.025, 1.5, 2.0, 0.5, 1.0]
    fn = pkg.initial.growth_sphere(0.025, seed=9, radius=0.25)
    g = pkg.Hierarchy(ctx, 3, 3, "growth", params)
    o = oracle_mod.OracleHierarchy(3, 3, "growth", params)
    for h in (g, o):
        h.build_uniform([16, 16, 16], -3, [10] * 6, [0, 0, 0], [1, 1, 1])
        h.commit()
        h.put(0, "q", fn(0, [16] * 3, [1 / 16] * 3, [0.0] * 3))
    kw = dict(tagging="gradient", initial=True, qtolerance=0.25, first_id=1000)
    g = g.regrid(pkg.regrid_params(2, **kw), fn)
    o = oracle_mod.regrid(o, oracle_mod.regrid_params(2, **kw), fn)
    tab = same(g, o)
    fin = max(p["level"] for p in tab)
    g.time_step(True, fin, -3, tol=1e-9, maxvcycles=30)
    o.time_step(True, fin, -3, tol=1e-9, maxvcycles=30)
    a, b = g.after_step_stats(fin), o.after_step_stats(fin)
    assert a[2] == b[2] and abs(a[0] - b[0]) <= ATOL and a[1] == b[1] == 0.0
    for name, wg, wo in (("m.dat", g.write_q, o.write_q), ("u.dat", g.write_uniform_q, o.write_uniform_q)):
        wg(tmp_path / ("g" + name), 0.01, fin)
        wo(tmp_path / ("o" + name), 0.01, fin)
        assert (tmp_path / ("g" + name)).read_bytes() == (tmp_path / ("o" + name)).read_bytes(), name
    groot = pkg.Hierarchy(ctx, 3, 3, "growth", params)
    oroot = oracle_mod.OracleHierarchy(3, 3, "growth", params)
    for h in (groot, oroot):
        h.build_uniform([16, 16, 16], -3, [10] * 6, [0, 0, 0], [1, 1, 1])
        h.commit()
    g2, _ = groot.read_q(tmp_path / "om.dat", first_id=50)
    o2, _ = oracle_mod.read_q(oroot, tmp_path / "om.dat", first_id=50)
    same(g2, o2)
