"""CUDA path vs the CPU oracle, through the C ABI (needs a GB300).

Tiers: (i) one colour half-sweep, (ii) one SetGhost of every kind,
(iii) one V-cycle, (iv) MultigridIterations, (v) time steps.  The plain FP64
path evaluates every expression in the reference's order without fused
multiply-adds, so tiers (i)-(iii) are compared bit for bit; from (iv) on the
residual norm is a parallel reduction whose order differs from the
reference's sequential SUM, so norms are compared to 1e-12 relative and the
fields to the benchmark spec's tolerance of 1e-12 relative in max-norm.
"""
import math

import numpy as np
import pytest

from tests import hierarchies as H

pytestmark = pytest.mark.gpu

RTOL = 1e-12
CH2 = dict(ndims=2, problem="ch", params=[1e-3, 0.01])
CH3 = dict(ndims=3, problem="ch", params=[5e-4, 0.02])
BIO2 = dict(ndims=2, problem="biogrowth", params=[0.1, 0.05, 1.5, 2.0, 0.5])
GROWTH3 = dict(ndims=3, problem="growth", params=[0.01, 0.025, 1.5, 2.0, 0.5, 1.0], nrvars=3)


def make_pair(pkg, ctx, oracle_mod, cfg, spec):
    nv = cfg.get("nrvars", 2)
    g = pkg.Hierarchy(ctx, cfg["ndims"], nv, cfg["problem"], cfg["params"])
    o = oracle_mod.OracleHierarchy(cfg["ndims"], nv, cfg["problem"], cfg["params"])
    spec.apply(g)
    spec.apply(o)
    return g, o


def uniform_spec(nd, n, mthbc, length=1.0):
    s = H.Spec(nd)
    s.root_and_below(n, -int(math.log2(n)) + 1, mthbc, length)
    return s


def random_fill(spec, hs, seed, fields=("q", "qold", "f")):
    rng = np.random.default_rng(seed)
    for p in spec.patches:
        for fld in fields:
            n = hs[0].field_size(p["id"], fld)
            a = rng.uniform(-1, 1, size=n)
            for h in hs:
                h.put(p["id"], fld, a)


def compare(spec, g, o, fields=("q",), exact=True, rtol=RTOL):
    worst = 0.0
    for p in spec.patches:
        for fld in fields:
            a, b = g.get(p["id"], fld), o.get(p["id"], fld)
            if exact:
                bad = np.flatnonzero(a != b)
                assert bad.size == 0, (f"patch {p['id']} field {fld}: {bad.size} cells differ, first "
                                       f"{bad[:5]}, gpu {a[bad[:5]]}, oracle {b[bad[:5]]}")
            else:
                scale = max(np.max(np.abs(b)), 1e-300)
                worst = max(worst, float(np.max(np.abs(a - b)) / scale))
    assert worst <= rtol, worst
    return worst


PERIODIC2 = [2, 2, 2, 2, 10, 10]
NEUMANN2 = [10, 10, 10, 10, 10, 10]
PERIODIC3 = [2, 2, 2, 2, 2, 2]
DIRICHLET3 = [10, 10, 10, 10, 10, 10]

CASES = {
    "ch2d-periodic": (CH2, lambda: uniform_spec(2, 32, PERIODIC2)),
    "ch2d-neumann": (CH2, lambda: uniform_spec(2, 32, NEUMANN2)),
    "ch3d-periodic": (CH3, lambda: uniform_spec(3, 16, PERIODIC3)),
    "ch3d-dirichlet": (CH3, lambda: uniform_spec(3, 16, DIRICHLET3)),
    "bio2d": (BIO2, lambda: uniform_spec(2, 32, NEUMANN2, 6.4)),
    "ch2d-amr-periodic": (CH2, lambda: H.amr2d(periodic=True)),
    "ch2d-amr-neumann": (CH2, lambda: H.amr2d(periodic=False)),
    "bio2d-amr": (BIO2, lambda: H.amr2d(periodic=False)),
    "ch3d-amr-periodic": (CH3, lambda: H.amr3d(periodic=True)),
    "ch3d-amr-dirichlet": (CH3, lambda: H.amr3d(periodic=False)),
    "growth3d": (GROWTH3, lambda: uniform_spec(3, 16, DIRICHLET3)),
    "growth3d-amr": (GROWTH3, lambda: H.amr3d(periodic=False)),
}


@pytest.mark.parametrize("case", list(CASES))
def test_relax_one_colour_bitexact(pkg, ctx, oracle_mod, case):
    cfg, mk = CASES[case]
    spec = mk()
    g, o = make_pair(pkg, ctx, oracle_mod, cfg, spec)
    random_fill(spec, (g, o), 11)
    for level in range(spec.minlevel(), spec.finest() + 1):
        for ipass in (1, 2):
            g.relax_level_color(level, ipass)
            o.relax_level_color(level, ipass)
    compare(spec, g, o)


@pytest.mark.parametrize("case", list(CASES))
def test_set_ghost_bitexact(pkg, ctx, oracle_mod, case):
    cfg, mk = CASES[case]
    spec = mk()
    g, o = make_pair(pkg, ctx, oracle_mod, cfg, spec)
    random_fill(spec, (g, o), 12, fields=("q",))
    for level in range(spec.finest(), spec.minlevel() - 1, -1):
        for ipass in (1, 2, 0):
            g.set_ghost(level, ipass)
            o.set_ghost(level, ipass)
            compare(spec, g, o)


@pytest.mark.parametrize("case", list(CASES))
def test_vcycle_bitexact(pkg, ctx, oracle_mod, case):
    cfg, mk = CASES[case]
    spec = mk()
    g, o = make_pair(pkg, ctx, oracle_mod, cfg, spec)
    random_fill(spec, (g, o), 13)
    fin, mn = spec.finest(), spec.minlevel()
    for h in (g, o):
        for level in range(0, fin + 1):
            h.set_ghost(level, 0)
        h.fill_down("q", fin, mn)
        h.copy_q_to_qold(mn, fin)
        h.vcycle(fin, mn, 2)
    compare(spec, g, o, fields=("q", "qc", "f", "rf"))


def _init(pkg, spec, hs, cfg, seed):
    nd = cfg["ndims"]
    for p in spec.patches:
        shape = tuple(p["mx"][:nd])
        h = p["dx"][0]
        if cfg["problem"] == "ch":
            q = pkg.initial.ch_spinodal(shape, cfg["params"][1], h, seed=seed + p["id"] + 50)
        elif cfg["problem"] == "growth":
            q = pkg.initial.growth_sphere(cfg["params"][1], seed=seed, radius=0.3)(
                p["level"], list(shape), p["dx"][:nd], p["xlower"][:nd])
        else:
            q = np.zeros(tuple(n + 2 for n in shape) + (2,), order="F")
            q[(slice(1, -1),) * nd + (0,)] = pkg.initial.splitmix_pm1(
                seed, pkg.initial.global_index(shape)).reshape(shape, order="F") * 0.9
            q[(slice(1, -1),) * nd + (1,)] = 1.0
        for hh in hs:
            hh.put(p["id"], "q", q)


@pytest.mark.parametrize("case", list(CASES))
def test_time_steps_match_oracle(pkg, ctx, oracle_mod, case):
    cfg, mk = CASES[case]
    spec = mk()
    g, o = make_pair(pkg, ctx, oracle_mod, cfg, spec)
    _init(pkg, spec, (g, o), cfg, 21)
    fin, mn = spec.finest(), spec.minlevel()
    for step in range(3):
        ng, rg = g.time_step(step == 0, fin, mn, tol=1e-9, maxvcycles=25)
        no, ro = o.time_step(step == 0, fin, mn, tol=1e-9, maxvcycles=25)
        assert ng == no, (step, ng, no, rg, ro)
        np.testing.assert_allclose(rg, ro, rtol=1e-10, atol=0)
    compare(spec, g, o, fields=("q",), exact=False)


def test_ch2d_128_ten_steps(pkg, ctx, oracle_mod):
    """The reference-runnable configuration: 2D CH 128^2 periodic, eps=0.01,
    dt=1e-3, V(2,2), tol 1e-9, 10 steps."""
    spec = uniform_spec(2, 128, PERIODIC2)
    g, o = make_pair(pkg, ctx, oracle_mod, CH2, spec)
    q = pkg.initial.ch_spinodal((128, 128), 0.01, 1.0 / 128, seed=2024)
    for h in (g, o):
        h.put(0, "q", q)
        h.set_ghost(0, 0)
        h.copy_q_to_qold(-6, 0)
    for step in range(10):
        ng, rg = g.time_step(step == 0, 0, -6, tol=1e-9, maxvcycles=20)
        no, ro = o.time_step(step == 0, 0, -6, tol=1e-9, maxvcycles=20)
        assert ng == no
    err = compare(spec, g, o, exact=False)
    print("128^2 x 10 steps: max rel diff", err)


def test_field_sections_read_and_write_the_fortran_box(pkg, ctx):
    """bsamg_put/get_field_section move exactly the Fortran section lo..hi of
    a patch field (ghost layers addressed at 1-mbc, variables last)."""
    h = pkg.Hierarchy(ctx, 3, 2, "ch", [5e-4, 0.02])
    h.build_uniform([8, 6, 4], -1, [2] * 6, [0, 0, 0], [1, 0.75, 0.5])
    h.commit()
    rng = np.random.default_rng(3)
    full = rng.standard_normal((10, 8, 6, 2))
    h.put(0, "q", np.asfortranarray(full))
    # q(1:8, 0:3, 2:5, 2:2): interior in x, lower ghost + 3 cells in y, variable 2
    lo, hi = [1, 0, 2, 2], [8, 3, 5, 2]
    sec = h.get_section(0, "q", lo, hi)
    assert sec.shape == (8, 4, 4, 1)
    assert np.array_equal(sec, full[1:9, 0:4, 2:6, 1:2])
    new = rng.standard_normal(sec.shape)
    h.put_section(0, "q", lo, hi, new)
    want = full.copy()
    want[1:9, 0:4, 2:6, 1:2] = new
    got = h.get(0, "q").reshape(want.shape, order="F")
    assert np.array_equal(got, want)
    # f is interior-only: f(1:8, 1:6, 1:4, 1:2)
    fsec = h.get_section(0, "f", [1, 1, 1, 1], [8, 6, 4, 2])
    assert fsec.shape == (8, 6, 4, 2)
    with pytest.raises(pkg.BsamgError):
        h.get_section(0, "f", [0, 1, 1, 1], [8, 6, 4, 2])  # f has no ghost layer
    with pytest.raises(pkg.BsamgError):
        h.get_section(0, "q", [1, 1, 1, 1], [8, 6, 4, 3])  # nrvars = 2
