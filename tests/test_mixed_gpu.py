"""Mixed-precision path (FP32 correction V-cycle in an FP64 defect-correction
loop) against the FP64 oracle (needs a GB300).

Both paths stop when the FP64 residual norm of the finest level falls below
the tolerance, so at the configuration tolerance they stop at different
iterates and differ by about what the tolerance allows (the FP64 path's own
error against a fully converged solve is 3e-8 relative in 2D at 1e-9 and
2e-7 in 3D at 1e-8).  Converged tightly, both must reach the same discrete
solution; that is the parity statement for this path.
"""
import numpy as np
import pytest

from tests import hierarchies as H
from tests.test_parity_gpu import CH2, CH3, uniform_spec, make_pair, PERIODIC2, PERIODIC3, NEUMANN2, DIRICHLET3

pytestmark = pytest.mark.gpu


def levels_spec(nd, n, minlevel, mthbc):
    """uniform root of n cells per side and the levels below it down to
    minlevel (extents that are not powers of two, all even)"""
    s = H.Spec(nd)
    s.root_and_below(n, minlevel, mthbc, 1.0)
    return s


# case: (config, hierarchy, config tolerance, its error bound, tight tolerance, tight bound).
# The bounds are what the path delivers with a margin of about three: the
# largest errors measured on a GB300 were 3.4e-8 (3D) and 7.8e-9 (2D) at the
# configuration tolerances, 5.4e-11 (3D at 1e-11) and 5.7e-12 (2D at 1e-12)
# tightly converged.
B2, B2T, B3, B3T = 3e-8, 3e-11, 1e-7, 2e-10
MIXED_CASES = {
    "ch2d-periodic-64": (CH2, lambda: uniform_spec(2, 64, PERIODIC2), 1e-9, B2, 1e-12, B2T),
    "ch2d-neumann-64": (CH2, lambda: uniform_spec(2, 64, NEUMANN2), 1e-9, B2, 1e-12, B2T),
    "ch3d-periodic-32": (CH3, lambda: uniform_spec(3, 32, PERIODIC3), 1e-8, B3, 1e-11, B3T),
    "ch3d-periodic-64": (CH3, lambda: uniform_spec(3, 64, PERIODIC3), 1e-8, B3, 1e-11, B3T),
    "ch3d-dirichlet-16": (CH3, lambda: uniform_spec(3, 16, DIRICHLET3), 1e-8, B3, 1e-11, B3T),
    # periodic boxes whose extents are not powers of two (48..6, 24..6): the
    # box path's coarse-end cycle takes cell coordinates by division
    "ch2d-periodic-48": (CH2, lambda: levels_spec(2, 48, -3, PERIODIC2), 1e-9, B2, 1e-12, B2T),
    "ch3d-periodic-24": (CH3, lambda: levels_spec(3, 24, -2, PERIODIC3), 1e-8, B3, 1e-11, B3T),
    "ch2d-amr-periodic": (CH2, lambda: H.amr2d(periodic=True), 1e-9, B2, 1e-12, B2T),
    "ch3d-amr-periodic": (CH3, lambda: H.amr3d(periodic=True), 1e-8, B3, 1e-11, B3T),
}


def _run(pkg, ctx, oracle_mod, cfg, spec, tol):
    g, o = make_pair(pkg, ctx, oracle_mod, cfg, spec)
    nd = cfg["ndims"]
    for p in spec.patches:
        shape = tuple(p["mx"][:nd])
        q = pkg.initial.ch_spinodal(shape, cfg["params"][1], p["dx"][0], seed=31 + p["id"])
        g.put(p["id"], "q", q)
        o.put(p["id"], "q", q)
    fin, mn = spec.finest(), spec.minlevel()
    for step in range(3):
        ng, rg = g.time_step(step == 0, fin, mn, tol=tol, maxvcycles=40, mode="mixed", strict=True)
        no, ro = o.time_step(step == 0, fin, mn, tol=tol, maxvcycles=40)
        assert rg[-1] < tol, (step, rg)
        assert ng <= no + 3, (step, ng, no, rg, ro)
    worst = 0.0
    for p in spec.patches:
        a, b = g.get(p["id"], "q"), o.get(p["id"], "q")
        n = a.size // 2
        worst = max(worst, float(np.max(np.abs(a[:n] - b[:n])) / np.max(np.abs(b[:n]))))
    return worst


@pytest.mark.parametrize("case", list(MIXED_CASES))
def test_mixed_reaches_the_fp64_solution(pkg, ctx, oracle_mod, case):
    cfg, mk, tol, bound, tight, tight_bound = MIXED_CASES[case]
    err_tight = _run(pkg, ctx, oracle_mod, cfg, mk(), tight)
    err = _run(pkg, ctx, oracle_mod, cfg, mk(), tol)
    print(f"{case}: max rel error of phi vs FP64 oracle: {err:.3e} at tol {tol:g}, "
          f"{err_tight:.3e} at tol {tight:g}")
    assert err_tight <= tight_bound, err_tight
    assert err <= bound, err


@pytest.mark.parametrize("mode", ["mixed", "fp64"])
@pytest.mark.parametrize("nd,n,levels", [(2, 64, 2), (3, 32, 1), (3, 16, 2)])
def test_coarse_tail_in_one_block_is_bit_identical(pkg, ctx, nd, n, levels, mode):
    """The single-block coarse tail of the V-cycle executes the same per-unit
    operations as the separate launches, phase by phase: the iterates after
    time steps are bit-identical with the tail on and off (FP64 and mixed
    paths), and the tail cuts the launches."""
    pats, mn = pkg.serve.nested_spec(nd, n, levels)
    res = {}
    for cells in (16384, 2048, 0):
        h = pkg.Hierarchy(ctx, nd, 2, "ch", [1e-3 if nd == 2 else 5e-4, 0.02])
        for p in pats:
            h.add_patch(p["level"], p["id"], p["parent_id"], p["mx"], p["mglobal"], p["mbounds"], p["mthbc"],
                        p["dx"], p["xlower"])
        h.commit()
        h.set_tail_cells(cells)
        h.set_solve(0)  # the per-launch path (its coarse tail is what this test measures)
        for p in pats:
            if p["level"] >= 0:
                h.seed_spinodal(p["id"], 5 + p["id"])
        fin = max(p["level"] for p in pats)
        l0 = h.launch_count()
        hist = [h.time_step(s == 0, fin, mn, 2, 30, 1e-8, mode=mode) for s in range(3)]
        res[cells] = (hist, {p["id"]: h.get(p["id"], "q") for p in pats if p["level"] >= 0}, h.launch_count() - l0)
        h.close()
    hb, qb, lb = res[0]
    for cells in (16384, 2048):  # 2048: the tail's arrays staged in shared memory
        ha, qa, la = res[cells]
        assert ha == hb, cells
        for pid in qa:
            assert np.array_equal(qa[pid], qb[pid]), (cells, pid)
        assert la < lb, (cells, la, lb)


def _growth_pair(pkg, ctx, amr):
    """Two identical growth hierarchies (16^3 root, Dirichlet/reflecting
    faces), regridded to two levels around the seed when amr."""
    params = [0.01, 0.025, 1.5, 2.0, 0.5, 1.0]
    fn = pkg.initial.growth_sphere(0.025, seed=5, radius=0.25)
    out = []
    for _ in range(2):
        h = pkg.Hierarchy(ctx, 3, 3, "growth", params)
        h.build_uniform([16, 16, 16], -3, [10] * 6, [0, 0, 0], [1, 1, 1])
        h.commit()
        h.put(0, "q", fn(0, [16] * 3, [1 / 16] * 3, [0.0] * 3))
        if amr:
            h = h.regrid(pkg.regrid_params(2, tagging="gradient", initial=True, qtolerance=0.25), fn)
        out.append(h)
    return out


@pytest.mark.parametrize("amr", [False, True])
def test_mixed_growth_reaches_the_fp64_solution(pkg, ctx, amr):
    """The growth plugin's correction V-cycle (three variables) converges to
    the FP64 path's discrete solution: tightly converged (1e-11) the iterates
    agree to 1e-12 relative, at the configuration's tolerance (1e-8) to 5e-9
    (measured on a GB300: 2.3e-13 and 1.1e-9 uniform, 1.6e-13 and 1.1e-10
    with refinement)."""
    for tol, bound in ((1e-11, 1e-12), (1e-8, 5e-9)):
        gm, gf = _growth_pair(pkg, ctx, amr)
        tab = gm.patch_table()
        fin = max(p["level"] for p in tab)
        for step in range(3):
            nm, rm = gm.time_step(step == 0, fin, -3, tol=tol, maxvcycles=40, mode="mixed", strict=True)
            nf, rf = gf.time_step(step == 0, fin, -3, tol=tol, maxvcycles=40, mode="fp64")
            assert rm[-1] < tol and nm <= nf + 3, (step, nm, nf, rm, rf)
        worst = 0.0
        for p in tab:
            if p["level"] < 0:
                continue
            a, b = gm.get(p["id"], "q"), gf.get(p["id"], "q")
            n = a.size // 3
            for v in range(3):
                scale = max(np.max(np.abs(b[v * n:(v + 1) * n])), 1e-30)
                worst = max(worst, float(np.max(np.abs(a[v * n:(v + 1) * n] - b[v * n:(v + 1) * n])) / scale))
        print(f"growth amr={amr}: max rel difference mixed vs FP64 {worst:.3e} at tol {tol:g}")
        assert worst <= bound, (tol, worst)


def test_box_sweep_forms_agree(pkg, ctx):
    """The forms of the 3D periodic-box smoothing (two or four rows per
    thread, rows staged in shared memory by bulk copies, or a whole V(2,2)
    smoothing in one pass over z-planes staged in shared memory) evaluate
    the same expressions on the same values.  The two direct forms and the
    one-pass form are bit-identical after mixed time steps on a 128^3 box;
    the staged one sums the neighbours in another order, so it agrees to
    FP32 rounding of the converged iterates and takes the same number of
    V-cycles (within one)."""
    n = 128
    out = {}
    for kind in (0, 1, 2, 3):
        h = pkg.Hierarchy(ctx, 3, 2, "ch", [5e-4, 0.02])
        h.build_uniform([n] * 3, -6, [2] * 6, [0, 0, 0], [1, 1, 1])
        h.commit()
        h.set_box_sweep(kind)
        h.seed_spinodal(0, 11, mean=0.1, amp=0.05)
        hist = [h.time_step(s == 0, 0, -6, tol=1e-9, maxvcycles=30, mode="mixed", strict=True) for s in range(3)]
        out[kind] = (hist, h.get(0, "q"))
        h.close()
    (h0, q0), (h1, q1), (h2, q2), (h3, q3) = out[0], out[1], out[2], out[3]
    assert h0 == h1 == h3
    assert np.array_equal(q0, q1)
    assert np.array_equal(q0, q3)
    assert all(abs(a[0] - b[0]) <= 1 for a, b in zip(h2, h0)), (h2, h0)
    k = q0.size // 2
    assert np.max(np.abs(q2[:k] - q0[:k])) <= 1e-6 * np.max(np.abs(q0[:k]))
    with pytest.raises(pkg.BsamgError):
        h = pkg.Hierarchy(ctx, 3, 2, "ch", [5e-4, 0.02])
        try:
            h.set_box_sweep(4)
        finally:
            h.close()


@pytest.mark.parametrize("mx,minlevel", [((256, 64, 32), -4), ((256, 16, 8), -2), ((256, 256, 16), -3)])
def test_box_one_pass_smoothing_bit_identical(pkg, ctx, mx, minlevel):
    """The one-pass V(2,2) smoothing on boxes whose halo rows and planes wrap
    around the box, with one or several tiles per plane and z ranges shorter
    than the halo: the mixed time steps equal the four-row sweeps' bit for
    bit, residual histories included (8 V-cycles a step, converged or not)."""
    out = {}
    for kind in (1, 3):
        h = pkg.Hierarchy(ctx, 3, 2, "ch", [5e-4, 0.02])
        h.build_uniform(list(mx), minlevel, [2] * 6, [0, 0, 0], [1, mx[1] / mx[0], mx[2] / mx[0]])
        h.commit()
        h.set_box_sweep(kind)
        h.seed_spinodal(0, 23, mean=0.1, amp=0.05)
        hist = [h.time_step(s == 0, 0, minlevel, tol=1e-12, maxvcycles=8, mode="mixed", strict=False)
                for s in range(3)]
        out[kind] = (hist, h.get(0, "q"))
        h.close()
    (ha, qa), (hb, qb) = out[1], out[3]
    assert ha == hb
    assert np.array_equal(qa, qb)


def test_box_step_reuses_the_last_residual(pkg, ctx):
    """A box solve that follows one on the same q starts from the residual
    the last one ended with, updated for the new f (r + (f_new - f_old)),
    instead of evaluating the double-float operator again.  Against runs
    forced to recompute it (any mutating call clears the reuse): the same
    V-cycle counts, residual histories to 1e-6 relative or 1e-12 absolute
    (the FP32 g rounds the two starting residuals differently) and iterates
    to 1e-9 (the FP32 corrections round differently from there on; the
    solve's tolerance is 1e-9); a put between steps is honoured."""
    n = 64
    runs = []
    for cold in (False, True):
        h = pkg.Hierarchy(ctx, 3, 2, "ch", [5e-4, 0.02])
        h.build_uniform([n] * 3, -5, [2] * 6, [0, 0, 0], [1, 1, 1])
        h.commit()
        h.seed_spinodal(0, 17, mean=0.1, amp=0.05)
        hist = []
        for s in range(5):
            if cold:
                h.set_box_sweep(1)  # clears the reuse (and keeps the default sweep)
            if s == 3:
                q = h.get(0, "q")
                h.put(0, "q", q * 0.999)
            hist.append(h.time_step(s == 0, 0, -5, tol=1e-9, maxvcycles=30, mode="mixed", strict=True))
        runs.append((hist, h.get(0, "q")))
        h.close()
    (ha, qa), (hb, qb) = runs
    for (na, ra), (nb, rb) in zip(ha, hb):
        assert na == nb, (ha, hb)
        np.testing.assert_allclose(ra, rb, rtol=1e-6, atol=1e-12)
    k = qa.size // 2
    assert np.max(np.abs(qa[:k] - qb[:k])) <= 1e-9 * np.max(np.abs(qb[:k]))


def test_box_smoother_timing_reports_the_one_pass_form(pkg, ctx):
    """bsamg_time_smoother times the smoother the V-cycle runs on a level:
    on a 256-wide periodic box level one launch is a whole V(2,2) smoothing
    (four colour half-sweeps), elsewhere one colour sweep; the FP64 path
    always sweeps one colour.  After the timing launches a time step still
    converges (the one-pass launches write only the level's second e array,
    the sweeps only e, which every cycle starts from zero)."""
    for mx, minlevel, kind, want in (((256, 16, 8), -2, 3, 4), ((256, 16, 8), -2, 1, 1), ((128, 128, 8), -2, 3, 1)):
        h = pkg.Hierarchy(ctx, 3, 2, "ch", [5e-4, 0.02])
        h.build_uniform(list(mx), minlevel, [2] * 6, [0, 0, 0], [1, mx[1] / mx[0], mx[2] / mx[0]])
        h.commit()
        h.set_box_sweep(kind)
        h.seed_spinodal(0, 5, mean=0.1, amp=0.05)
        assert h.smoother_colours(0, "mixed") == want, (mx, kind)
        assert h.smoother_colours(0, "fp64") == 1
        assert h.smoother_colours(minlevel, "mixed") == 1
        assert h.time_smoother(0, "mixed", reps=3) > 0.0
        n, res = h.time_step(True, 0, minlevel, tol=1e-6, maxvcycles=30, mode="mixed", strict=False)
        assert np.isfinite(res[-1])
        h.close()
