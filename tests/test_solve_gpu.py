"""The one-launch cluster solve of adaptive hierarchies (mixed mode, finest
level above 0) against the per-launch mixed path (needs a GB300).

The cluster program is recorded from the same schedule functions the
per-launch path launches, every unit computes the same expressions, and the
residual norm is reduced in the same order, so both must give the same
iterates bit for bit, the same V-cycle counts and the same residuals, for
every launch shape (CTAs per cluster, threads per CTA, coarse levels run by
one CTA).  The per-launch path itself is tied to the FP64 oracle by
tests/test_mixed_gpu.py.
"""
import numpy as np
import pytest

from tests import hierarchies as H
from tests.test_parity_gpu import CH2, CH3

pytestmark = pytest.mark.gpu

SHAPES = [
    (16, 512, 64, 8192),    # the default
    (16, 1024, 256, 0),     # every level cluster-wide, whole blocks
    (8, 256, 32, 1 << 30),  # the whole V-cycle in CTA 0
    (1, 512, 128, 2048),    # a cluster of one CTA
    (4, 1024, 64, 512),
]


def _ch_pair(pkg, ctx, cfg, spec):
    hs = []
    for _ in range(2):
        h = pkg.Hierarchy(ctx, cfg["ndims"], 2, "ch", cfg["params"])
        spec.apply(h)
        nd = cfg["ndims"]
        for p in spec.patches:
            shape = tuple(p["mx"][:nd])
            h.put(p["id"], "q", pkg.initial.ch_spinodal(shape, cfg["params"][1], p["dx"][0], seed=41 + p["id"]))
        hs.append(h)
    return hs


def _steps(h, fin, mn, mode, tol, steps=3):
    out = []
    for s in range(steps):
        out.append(h.time_step(s == 0, fin, mn, 2, 40, tol, mode="mixed"))
    return out


def _same_state(a, b, tab):
    for p in tab:
        qa, qb = a.get(p["id"], "q"), b.get(p["id"], "q")
        assert np.array_equal(qa, qb), p["id"]


CASES = {
    "ch2d-amr-periodic": (CH2, lambda: H.amr2d(periodic=True), 1e-9),
    "ch2d-amr-neumann": (CH2, lambda: H.amr2d(periodic=False), 1e-9),
    "ch3d-amr-periodic": (CH3, lambda: H.amr3d(periodic=True), 1e-8),
}


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: f"{s[0]}x{s[1]}-tile{s[2]}-solo{s[3]}")
def test_cluster_solve_is_bit_identical(pkg, ctx, case, shape):
    cfg, mk, tol = CASES[case]
    spec = mk()
    a, b = _ch_pair(pkg, ctx, cfg, spec)
    a.set_solve(0)
    b.set_solve(1, *shape)
    fin, mn = spec.finest(), spec.minlevel()
    la0, lb0 = a.launch_count(), b.launch_count()
    ha = _steps(a, fin, mn, "mixed", tol)
    hb = _steps(b, fin, mn, "mixed", tol)
    assert ha == hb
    _same_state(a, b, spec.patches)
    # the iterations of each step are one launch (plus the step's FP64 prologue)
    assert lb0 >= 0 and (b.launch_count() - lb0) < (a.launch_count() - la0)
    a.close()
    b.close()


def test_cluster_solve_after_regrid(pkg, ctx):
    """A regridded 2D hierarchy (the AMR workload's tagging and clustering,
    uneven patches of 8-32 cells per side, the mesh changing every step): the
    cluster solve and the per-launch path stay identical step after step."""
    fn = pkg.initial.ch_circle_patch(0.01, 20240503, radius=0.25, noise=0.01)
    hs = []
    for mode in (0, 1):
        h = pkg.Hierarchy(ctx, 2, 2, "ch", [1e-3, 0.01])
        h.build_uniform([64, 64, 1], -5, [2, 2, 2, 2, 10, 10], [0, 0, 0], [1, 1, 1])
        h.commit()
        h.put(0, "q", fn(0, [64, 64], [1 / 64] * 2, [0.0, 0.0]))
        h.set_solve(mode)
        hs.append(h)
    hist = [[], []]
    for s in range(4):
        for m in (0, 1):
            old = hs[m]
            prm = pkg.regrid_params(3, tagging="gradient", initial=s == 0, maxside=64, first_id=1000 * (s + 1),
                                    qtolerance=0.25)
            hs[m] = old.regrid(prm, fn if s == 0 else None)
            old.close()
            assert hs[m].get_solve()[0] == m  # carried over by the regrid
            fin = max(p["level"] for p in hs[m].patch_table())
            hist[m].append(hs[m].time_step(s == 0, fin, -5, 2, 30, 1e-9, mode="mixed", strict=True))
        assert hist[0][-1] == hist[1][-1], s
        tab = hs[0].patch_table()
        assert [(p["level"], p["mglobal"]) for p in tab] == [(p["level"], p["mglobal"]) for p in hs[1].patch_table()]
        _same_state(hs[0], hs[1], tab)
    for h in hs:
        h.close()


def test_cluster_solve_growth(pkg, ctx):
    """Three variables (the growth plugin) on a regridded 3D hierarchy."""
    params = [0.01, 0.025, 1.5, 2.0, 0.5, 1.0]
    fn = pkg.initial.growth_sphere(0.025, seed=5, radius=0.25)
    hs = []
    for mode in (0, 1):
        h = pkg.Hierarchy(ctx, 3, 3, "growth", params)
        h.build_uniform([16, 16, 16], -3, [10] * 6, [0, 0, 0], [1, 1, 1])
        h.commit()
        h.put(0, "q", fn(0, [16] * 3, [1 / 16] * 3, [0.0] * 3))
        h.set_solve(mode)
        hs.append(h.regrid(pkg.regrid_params(2, tagging="gradient", initial=True, qtolerance=0.25), fn))
        h.close()
    tab = hs[0].patch_table()
    fin = max(p["level"] for p in tab)
    out = [[h.time_step(s == 0, fin, -3, 2, 30, 1e-8, mode="mixed", strict=True) for s in range(3)] for h in hs]
    assert out[0] == out[1]
    _same_state(hs[0], hs[1], tab)
    for h in hs:
        h.close()


def test_cluster_solve_limits(pkg, ctx):
    """maxvcycles reached: the same residual history and the same
    not-converged report (strict) as the per-launch path; a bad shape is an
    argument error."""
    spec = H.amr2d(periodic=True)
    a, b = _ch_pair(pkg, ctx, CH2, spec)
    a.set_solve(0)
    b.set_solve(1)
    fin, mn = spec.finest(), spec.minlevel()
    ra = a.time_step(True, fin, mn, 2, 2, 1e-14, mode="mixed")
    rb = b.time_step(True, fin, mn, 2, 2, 1e-14, mode="mixed")
    assert ra == rb and ra[0] == 2
    for h in (a, b):
        with pytest.raises(pkg.BsamgError):
            h.time_step(False, fin, mn, 2, 2, 1e-14, mode="mixed", strict=True)
    with pytest.raises(pkg.BsamgError):
        b.set_solve(1, 17, 512, 64, 0)
    with pytest.raises(pkg.BsamgError):
        b.set_solve(1, 8, 384, 64, 0)
    with pytest.raises(pkg.BsamgError):
        b.set_solve(1, 8, 512, 48, 0)
    _same_state(a, b, spec.patches)
    a.close()
    b.close()


def test_autotuned_solve(pkg, tmp_path):
    """The autotuner (a fresh context, tuning on): the first solve of a size
    class times the candidate shapes from the same q and restores it, so the
    iterates equal the per-launch path's bit for bit; the choice is kept for
    the class, reused by a regridded hierarchy of the same class, and
    survives a JSON round trip."""
    import json

    ctx = pkg.Context(0)
    try:
        spec = H.amr2d(periodic=True)
        a, b = _ch_pair(pkg, ctx, CH2, spec)
        a.set_solve(0)
        fin, mn = spec.finest(), spec.minlevel()
        assert ctx.tune_count() == 0
        ha = _steps(a, fin, mn, "mixed", 1e-9)
        hb = _steps(b, fin, mn, "mixed", 1e-9)
        assert ha == hb
        _same_state(a, b, spec.patches)
        assert ctx.tune_count() == 1
        mode, ctas, threads, tile, solo = b.get_solve()
        path = tmp_path / "tune.json"
        ctx.tune_save(path)
        doc = json.loads(path.read_text())
        assert len(doc["entries"]) == 1
        e = doc["entries"][0]
        assert e["ctas"] in (0, 16) and e["us_per_cycle"] > 0  # 0: the per-launch path won
        if e["ctas"]:
            assert mode == 1 and (e["ctas"], e["threads"], e["tile"], e["solo_cells"]) == (ctas, threads, tile, solo)
            assert threads in (256, 512, 1024) and tile in (32, 64, 128)
        ctx2 = pkg.Context(0)
        try:
            ctx2.tune_load(path)
            assert ctx2.tune_count() == 1
            bad = tmp_path / "bad.json"
            bad.write_text('{"something": 2}')
            with pytest.raises(pkg.BsamgError):
                ctx2.tune_load(bad)
        finally:
            ctx2.close()
        a.close()
        b.close()
    finally:
        ctx.close()
