"""Two ghost layers (mbc = 2) through the C ABI vs the oracle (needs a GB300).

With mbc = 2 the arrays q, qold and qc carry a second ghost layer: SetGhost
fills it from siblings, periodic images and physical boundaries; CorrectFine
corrects it with BiLin/TriLinProlongationP2 and InitFields fills it with
P2MC.  The plain FP64 path stays bit-exact per operation against the
oracle, full arrays included; the regrid, frame files and restart match the
oracle's; the interior and first layer equal the mbc = 1 run's bit for bit.
"""
import math

import numpy as np
import pytest

from tests import hierarchies as H
from tests.test_parity_gpu import BIO2, CH2, CH3, GROWTH3, DIRICHLET3, NEUMANN2, PERIODIC2, compare, random_fill
from tests.test_regrid_gpu import circle2d

pytestmark = pytest.mark.gpu

CASES = {
    "ch2d-neumann": (CH2, lambda: _uniform(2, 32, NEUMANN2)),
    "ch3d-dirichlet": (CH3, lambda: _uniform(3, 16, DIRICHLET3)),
    "ch2d-amr-periodic": (CH2, lambda: H.amr2d(periodic=True)),
    "ch2d-amr-neumann": (CH2, lambda: H.amr2d(periodic=False)),
    "bio2d-amr": (BIO2, lambda: H.amr2d(periodic=False)),
    "ch3d-amr-periodic": (CH3, lambda: H.amr3d(periodic=True)),
    "ch3d-amr-dirichlet": (CH3, lambda: H.amr3d(periodic=False)),
    "growth3d-amr": (GROWTH3, lambda: H.amr3d(periodic=False)),
}


def _uniform(nd, n, mthbc):
    s = H.Spec(nd)
    s.root_and_below(n, -int(math.log2(n)) + 1, mthbc)
    return s


def embed(q, mx, nv, mbc):
    """an array with one ghost layer placed at q(0:mx+1) of the mbc layout"""
    nd = len(mx)
    q = np.asarray(q, dtype=np.float64).reshape([m + 2 for m in mx] + [nv], order="F")
    out = np.zeros([m + 2 * mbc for m in mx] + [nv], order="F")
    g = mbc - 1
    out[tuple(slice(g, g + m + 2) for m in mx)] = q
    return out.ravel(order="F")


def inner(a, mx, nv, mbc):
    a = a.reshape([m + 2 * mbc for m in mx] + [nv], order="F")
    g = mbc - 1
    return a[tuple(slice(g, g + m + 2) for m in mx)]


def make(pkg, ctx, oracle_mod, cfg, spec, mbc=2, gpu_only=False):
    nv = cfg.get("nrvars", 2)
    g = pkg.Hierarchy(ctx, cfg["ndims"], nv, cfg["problem"], cfg["params"], mbc=mbc)
    spec.apply(g)
    if gpu_only:
        return g
    o = oracle_mod.OracleHierarchy(cfg["ndims"], nv, cfg["problem"], cfg["params"], mbc=mbc)
    spec.apply(o)
    return g, o


def initial_q(pkg, cfg, p, seed):
    nd = cfg["ndims"]
    shape = tuple(p["mx"][:nd])
    if cfg["problem"] == "ch":
        return pkg.initial.ch_spinodal(shape, cfg["params"][1], p["dx"][0], seed=seed + p["id"])
    if cfg["problem"] == "growth":
        return pkg.initial.growth_sphere(cfg["params"][1], seed=seed, radius=0.3)(
            p["level"], list(shape), p["dx"][:nd], p["xlower"][:nd])
    q = np.zeros(tuple(n + 2 for n in shape) + (2,), order="F")
    q[(slice(1, -1),) * nd + (0,)] = pkg.initial.splitmix_pm1(
        seed, pkg.initial.global_index(shape)).reshape(shape, order="F") * 0.9
    q[(slice(1, -1),) * nd + (1,)] = 1.0
    return q


@pytest.mark.parametrize("case", list(CASES))
def test_operations_bitexact_with_two_ghost_layers(pkg, ctx, oracle_mod, case):
    """One colour half-sweep per level, every SetGhost, one V-cycle: full
    arrays (both ghost layers) bit for bit."""
    cfg, mk = CASES[case]
    spec = mk()
    g, o = make(pkg, ctx, oracle_mod, cfg, spec)
    random_fill(spec, (g, o), 71, fields=("q", "qold", "f", "qc"))
    fin, mn = spec.finest(), spec.minlevel()
    for level in range(mn, fin + 1):
        for ipass in (1, 2):
            g.relax_level_color(level, ipass)
            o.relax_level_color(level, ipass)
    compare(spec, g, o)
    for level in range(fin, mn - 1, -1):
        for ipass in (1, 2, 0):
            g.set_ghost(level, ipass)
            o.set_ghost(level, ipass)
    compare(spec, g, o)
    for h in (g, o):
        h.fill_down("q", fin, mn)
        h.copy_q_to_qold(mn, fin)
        h.vcycle(fin, mn, 2)
        h.vcycle(fin, mn, 2)  # the second cycle reads the second ring of qc the first one left
    compare(spec, g, o, fields=("q", "qc", "f", "rf"))


@pytest.mark.parametrize("case", list(CASES))
def test_time_steps_with_two_ghost_layers_match_oracle(pkg, ctx, oracle_mod, case):
    cfg, mk = CASES[case]
    spec = mk()
    g, o = make(pkg, ctx, oracle_mod, cfg, spec)
    nv, nd = cfg.get("nrvars", 2), cfg["ndims"]
    for p in spec.patches:
        q = embed(initial_q(pkg, cfg, p, 23), p["mx"][:nd], nv, 2)
        g.put(p["id"], "q", q)
        o.put(p["id"], "q", q)
    fin, mn = spec.finest(), spec.minlevel()
    for step in range(3):
        ng, rg = g.time_step(step == 0, fin, mn, tol=1e-9, maxvcycles=25)
        no, ro = o.time_step(step == 0, fin, mn, tol=1e-9, maxvcycles=25)
        assert ng == no, (step, ng, no, rg, ro)
        np.testing.assert_allclose(rg, ro, rtol=1e-10, atol=0)
    compare(spec, g, o, fields=("q", "qc"), exact=False)


@pytest.mark.parametrize("case", ["ch2d-amr-periodic", "ch3d-amr-dirichlet"])
def test_two_ghost_layers_give_the_one_layer_run(pkg, ctx, oracle_mod, case):
    """The library with mbc = 2 gives its own mbc = 1 run's interior and
    first ghost layer bit for bit, residual histories included."""
    cfg, mk = CASES[case]
    spec = mk()
    nd = cfg["ndims"]
    hs = [make(pkg, ctx, oracle_mod, cfg, spec, mbc=m, gpu_only=True) for m in (1, 2)]
    for p in spec.patches:
        q = initial_q(pkg, cfg, p, 31)
        hs[0].put(p["id"], "q", q)
        hs[1].put(p["id"], "q", embed(q, p["mx"][:nd], 2, 2))
    fin, mn = spec.finest(), spec.minlevel()
    for step in range(3):
        r = [h.time_step(step == 0, fin, mn, tol=1e-9, maxvcycles=25) for h in hs]
        assert r[0][0] == r[1][0] and np.array_equal(r[0][1], r[1][1]), (step, r)
    for p in spec.patches:
        a = hs[0].get(p["id"], "q").reshape([m + 2 for m in p["mx"][:nd]] + [2], order="F")
        assert np.array_equal(a, inner(hs[1].get(p["id"], "q"), p["mx"][:nd], 2, 2)), p["id"]


def _regrid_pair(pkg, ctx, oracle_mod):
    g = pkg.Hierarchy(ctx, 2, 2, "ch", [1e-3, 0.01], mbc=2)
    o = oracle_mod.OracleHierarchy(2, 2, "ch", [1e-3, 0.01], mbc=2)
    for h in (g, o):
        h.build_uniform([64, 64, 1], -5, [2, 2, 2, 2, 10, 10], [0, 0, 0], [1, 1, 1])
        h.commit()
        h.put(0, "q", embed(circle2d()(0, [64, 64], [1 / 64] * 2, [0.0, 0.0]), [64, 64], 2, 2))
    return g, o


def _same(g, o):
    tg, to = g.patch_table(), o.patch_table()
    assert len(tg) == len(to)
    for a, b in zip(tg, to):
        for k in ("level", "id", "parent_id", "mx", "mglobal", "mbounds", "mthbc", "dx", "xlower"):
            assert a[k] == b[k], (k, a, b)
    for p in tg:
        for fld in ("q", "qold", "qc"):
            x, y = g.get(p["id"], fld), o.get(p["id"], fld)
            bad = np.flatnonzero(x != y)
            assert bad.size == 0, (p["id"], fld, bad[:5], x[bad[:5]], y[bad[:5]])
    return tg


def test_regrid_frames_and_restart_with_two_ghost_layers(pkg, ctx, oracle_mod, tmp_path):
    """Regrid every step (InitFields with P2MC, the persisting levels' qc
    kept), WriteQ / WriteUniformMeshQ bytes and ReadQ as the oracle's."""
    om = oracle_mod
    g, o = _regrid_pair(pkg, ctx, om)
    for step in range(3):
        kw = dict(tagging="gradient", initial=step == 0, maxside=64, qtolerance=0.25, first_id=1000 * (step + 1))
        g = g.regrid(pkg.regrid_params(3, **kw), circle2d() if step == 0 else None)
        o = om.regrid(o, om.regrid_params(3, **kw), circle2d() if step == 0 else None)
        tab = _same(g, o)
        fin = max(p["level"] for p in tab)
        ng, rg = g.time_step(step == 0, fin, -5, tol=1e-9, maxvcycles=30)
        no, ro = o.time_step(step == 0, fin, -5, tol=1e-9, maxvcycles=30)
        assert ng == no, (step, rg, ro)
        np.testing.assert_allclose(rg, ro, rtol=1e-10, atol=0)
    for f in (0, fin):
        g.write_q(tmp_path / "g.dat", 0.5, f)
        o.write_q(tmp_path / "o.dat", 0.5, f)
        assert (tmp_path / "g.dat").read_bytes() == (tmp_path / "o.dat").read_bytes()
        g.write_uniform_q(tmp_path / "gu.dat", 0.5, f)
        o.write_uniform_q(tmp_path / "ou.dat", 0.5, f)
        assert (tmp_path / "gu.dat").read_bytes() == (tmp_path / "ou.dat").read_bytes()
    path = tmp_path / "frame.dat"
    o.write_q(path, 0.5, fin)
    groot, oroot = _regrid_pair(pkg, ctx, om)
    g2, tg = groot.read_q(path, first_id=700)
    o2, to = om.read_q(oroot, path, first_id=700)
    assert tg == to == 0.5
    _same(g2, o2)
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


def test_mixed_path_with_two_ghost_layers(pkg, ctx, oracle_mod):
    """The FP32 correction cycle keeps one ghost layer; converged tightly
    it reaches the FP64 solution (interior and first layer) to 1e-9."""
    cfg, mk = CASES["ch2d-amr-periodic"]
    spec = mk()
    g, o = make(pkg, ctx, oracle_mod, cfg, spec)
    for p in spec.patches:
        q = embed(initial_q(pkg, cfg, p, 37), p["mx"][:2], 2, 2)
        g.put(p["id"], "q", q)
        o.put(p["id"], "q", q)
    fin, mn = spec.finest(), spec.minlevel()
    for step in range(3):
        ng, rg = g.time_step(step == 0, fin, mn, tol=1e-12, maxvcycles=40, mode="mixed", strict=True)
        no, ro = o.time_step(step == 0, fin, mn, tol=1e-12, maxvcycles=40)
        assert rg[-1] < 1e-12 and ng <= no + 3, (step, ng, no)
    worst = 0.0
    for p in spec.patches:
        a = inner(g.get(p["id"], "q"), p["mx"][:2], 2, 2)[..., 0]
        b = inner(o.get(p["id"], "q"), p["mx"][:2], 2, 2)[..., 0]
        worst = max(worst, float(np.max(np.abs(a - b)) / np.max(np.abs(b))))
    assert worst <= 1e-9, worst


@pytest.mark.parametrize("nd,mthbc", [(2, [10, 10, 10, 10]), (2, [2, 2, 10, 10]), (2, [2, 2, 2, 2]),
                                      (3, [10] * 6), (3, [2, 2, 10, 10, 2, 2]), (3, [2] * 6)])
@pytest.mark.parametrize("mbc", [1, 2])
def test_root_ghosts_with_offsets_match_oracle(pkg, ctx, oracle_mod, nd, mthbc, mbc):
    """SelfPeriodicBC with a quasi-periodic offset (qpo) and SetPhysicalBC on
    a root patch, one and two ghost layers: the whole array bit for bit."""
    mx = [12, 8, 6][:nd]
    qpo = [0.25, -0.5]
    hs = [pkg.Hierarchy(ctx, nd, 2, "ch", [1e-3, 0.02], qpo=qpo, mbc=mbc),
          oracle_mod.OracleHierarchy(nd, 2, "ch", [1e-3, 0.02], qpo=qpo, mbc=mbc)]
    a = np.random.default_rng(sum(mthbc) + 7 * mbc + nd).uniform(-1, 1, size=int(np.prod([m + 2 * mbc for m in mx])) * 2)
    for h in hs:
        h.build_uniform(mx + [1] * (3 - nd), 0, mthbc + [10] * (6 - 2 * nd), [0, 0, 0],
                        [mx[d] / mx[0] if d < nd else 1.0 for d in range(3)])
        h.commit()
        h.put(0, "q", a)
        h.set_ghost(0, 0)
    assert np.array_equal(hs[0].get(0, "q"), hs[1].get(0, "q"))


def test_regrid_3d_with_two_ghost_layers(pkg, ctx, oracle_mod):
    """3D regrid (InitFields with TriLinProlongationP2MC, qc of the new
    patches from their parents) and a time step, as the oracle's."""
    from tests.test_regrid_gpu import sphere3d
    om = oracle_mod
    params = [5e-4, 0.05]
    g = pkg.Hierarchy(ctx, 3, 2, "ch", params, mbc=2)
    o = om.OracleHierarchy(3, 2, "ch", params, mbc=2)
    q0 = embed(sphere3d()(0, [16] * 3, [1 / 16] * 3, [0.0] * 3), [16] * 3, 2, 2)
    for h in (g, o):
        h.build_uniform([16, 16, 16], -3, [2] * 6, [0, 0, 0], [1, 1, 1])
        h.commit()
        h.put(0, "q", q0)
    for step in range(2):
        kw = dict(tagging="ch", initial=step == 0, qtolerance=0.05, first_id=500 * (step + 1))
        g = g.regrid(pkg.regrid_params(2, **kw), sphere3d() if step == 0 else None)
        o = om.regrid(o, om.regrid_params(2, **kw), sphere3d() if step == 0 else None)
        tab = _same(g, o)
        fin = max(p["level"] for p in tab)
        assert fin >= 1
        ng, rg = g.time_step(step == 0, fin, -3, tol=1e-8, maxvcycles=30)
        no, ro = o.time_step(step == 0, fin, -3, tol=1e-8, maxvcycles=30)
        assert ng == no, (step, rg, ro)
        np.testing.assert_allclose(rg, ro, rtol=1e-10, atol=0)
