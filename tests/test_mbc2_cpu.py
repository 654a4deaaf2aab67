"""Two ghost layers (mbc = 2, which RootInit allows beside mbc = 1,
bsamroutines.f90:305-308), on the oracle (no GPU).

(i) The oracle's CorrectFine (afasroutines.f90:860-980) and InitFields
prolongations are checked against a literal numpy transcription of the
reference's array statements: BiLin/TriLinProlongationP1 and P2 and their
mass-corrected forms (gridutilities.f90:156-369, :510-829).
(ii) Every operator of the path reads one ghost layer, so a run with
mbc = 2 gives the mbc = 1 run's interior and first ghost layer bit for bit:
time steps on uniform and AMR hierarchies and a regrid.
"""
import numpy as np
import pytest

from tests import hierarchies as H
from tests.test_regrid_cpu import circle

CH2 = dict(ndims=2, problem="ch", params=[1e-3, 0.01])
CH3 = dict(ndims=3, problem="ch", params=[5e-4, 0.02])


# --- numpy transcription of the reference's statements -------------------
# Arrays carry their Fortran lower bound: index f of a P1 array (bounds
# 0:...) is python index f, of a P2 array (bounds -1:...) python f + 1.

def bilin_p1(a):
    cmx = [a.shape[0] - 2, a.shape[1] - 2]
    mx = [2 * c for c in cmx]
    nv = a.shape[2]
    b = np.zeros((mx[0] + 2, cmx[1] + 2, nv))
    b[0:mx[0] + 1:2] = 3.0 * a[0:cmx[0] + 1] + a[1:cmx[0] + 2]
    b[1:mx[0] + 2:2] = a[0:cmx[0] + 1] + 3.0 * a[1:cmx[0] + 2]
    p = np.zeros((mx[0] + 2, mx[1] + 2, nv))
    p[:, 0:mx[1] + 1:2] = (3.0 * b[:, 0:cmx[1] + 1] + b[:, 1:cmx[1] + 2]) / 16.0
    p[:, 1:mx[1] + 2:2] = (b[:, 0:cmx[1] + 1] + 3.0 * b[:, 1:cmx[1] + 2]) / 16.0
    return p


def bilin_p2(a):
    cmx = [a.shape[0] - 4, a.shape[1] - 4]
    mx = [2 * c for c in cmx]
    nv = a.shape[2]
    b = np.zeros((mx[0] + 4, cmx[1] + 4, nv))
    # b(-1:mx+1:2, :) = 3 a(0:cmx+1, :) + a(-1:cmx, :)
    b[0:mx[0] + 3:2] = 3.0 * a[1:cmx[0] + 3] + a[0:cmx[0] + 2]
    # b(0:mx+2:2, :) = 3 a(0:cmx+1, :) + a(1:cmx+2, :)
    b[1:mx[0] + 4:2] = 3.0 * a[1:cmx[0] + 3] + a[2:cmx[0] + 4]
    p = np.zeros((mx[0] + 4, mx[1] + 4, nv))
    p[:, 0:mx[1] + 3:2] = (3.0 * b[:, 1:cmx[1] + 3] + b[:, 0:cmx[1] + 2]) / 16.0
    p[:, 1:mx[1] + 4:2] = (3.0 * b[:, 1:cmx[1] + 3] + b[:, 2:cmx[1] + 4]) / 16.0
    return p


def trilin_p1(a):
    cmx = [n - 2 for n in a.shape[:3]]
    mx = [2 * c for c in cmx]
    nv = a.shape[3]
    b = np.zeros((mx[0] + 2, cmx[1] + 2, cmx[2] + 2, nv))
    b[0:mx[0] + 1:2] = 3.0 * a[0:cmx[0] + 1] + a[1:cmx[0] + 2]
    b[1:mx[0] + 2:2] = a[0:cmx[0] + 1] + 3.0 * a[1:cmx[0] + 2]
    c = np.zeros((mx[0] + 2, mx[1] + 2, cmx[2] + 2, nv))
    c[:, 0:mx[1] + 1:2] = 3.0 * b[:, 0:cmx[1] + 1] + b[:, 1:cmx[1] + 2]
    c[:, 1:mx[1] + 2:2] = b[:, 0:cmx[1] + 1] + 3.0 * b[:, 1:cmx[1] + 2]
    p = np.zeros((mx[0] + 2, mx[1] + 2, mx[2] + 2, nv))
    p[:, :, 0:mx[2] + 1:2] = (3.0 * c[:, :, 0:cmx[2] + 1] + c[:, :, 1:cmx[2] + 2]) / 64.0
    p[:, :, 1:mx[2] + 2:2] = (c[:, :, 0:cmx[2] + 1] + 3.0 * c[:, :, 1:cmx[2] + 2]) / 64.0
    return p


def trilin_p2(a):
    cmx = [n - 4 for n in a.shape[:3]]
    mx = [2 * c for c in cmx]
    nv = a.shape[3]
    b = np.zeros((mx[0] + 4, cmx[1] + 4, cmx[2] + 4, nv))
    b[0:mx[0] + 3:2] = 3.0 * a[1:cmx[0] + 3] + a[0:cmx[0] + 2]
    b[1:mx[0] + 4:2] = 3.0 * a[1:cmx[0] + 3] + a[2:cmx[0] + 4]
    c = np.zeros((mx[0] + 4, mx[1] + 4, cmx[2] + 4, nv))
    c[:, 0:mx[1] + 3:2] = 3.0 * b[:, 1:cmx[1] + 3] + b[:, 0:cmx[1] + 2]
    c[:, 1:mx[1] + 4:2] = 3.0 * b[:, 1:cmx[1] + 3] + b[:, 2:cmx[1] + 4]
    p = np.zeros((mx[0] + 4, mx[1] + 4, mx[2] + 4, nv))
    p[:, :, 0:mx[2] + 3:2] = (3.0 * c[:, :, 1:cmx[2] + 3] + c[:, :, 0:cmx[2] + 2]) / 64.0
    p[:, :, 1:mx[2] + 4:2] = (3.0 * c[:, :, 1:cmx[2] + 3] + c[:, :, 2:cmx[2] + 4]) / 64.0
    return p


def mass_correct(a, p, mbc):
    """The MC forms' correction of the interior cells (same statements for
    P1MC and P2MC): a and p carry mbc ghost layers."""
    nd = a.ndim - 1
    o = mbc - 1  # python index of Fortran 1 is o + 1
    cmx = [n - 2 * mbc for n in a.shape[:nd]]
    ev = [slice(o + 2, o + 2 * c + 1, 2) for c in cmx]   # fine 2:mx:2
    od = [slice(o + 1, o + 2 * c, 2) for c in cmx]       # fine 1:mx-1:2
    ai = tuple(slice(o + 1, o + c + 1) for c in cmx)
    p = p.copy()
    if nd == 2:
        terms = [(ev[0], ev[1]), (od[0], ev[1]), (ev[0], od[1]), (od[0], od[1])]
        s = p[terms[0]] + p[terms[1]] + p[terms[2]] + p[terms[3]]
        cor = a[ai] - 0.25 * s
    else:
        terms = [(ev[0], ev[1], ev[2]), (od[0], ev[1], ev[2]), (ev[0], od[1], ev[2]), (od[0], od[1], ev[2]),
                 (ev[0], ev[1], od[2]), (od[0], ev[1], od[2]), (ev[0], od[1], od[2]), (od[0], od[1], od[2])]
        s = p[terms[0]]
        for t in terms[1:]:
            s = s + p[t]
        cor = a[ai] - 0.125 * s
    for t in terms:
        p[t] = p[t] + cor
    return p


PROL = {(2, 1): bilin_p1, (2, 2): bilin_p2, (3, 1): trilin_p1, (3, 2): trilin_p2}


@pytest.mark.parametrize("nd", [2, 3])
@pytest.mark.parametrize("mbc", [1, 2])
def test_prolong_mc_matches_the_reference_statements(oracle_mod, nd, mbc):
    rng = np.random.default_rng(40 + 10 * nd + mbc)
    cmx = [6, 4, 5][:nd]
    a = rng.uniform(-1, 1, size=[c + 2 * mbc for c in cmx])
    want = mass_correct(a[..., None], PROL[nd, mbc](a[..., None]), mbc)[..., 0]
    got = oracle_mod.prolong_mc(a, mbc)
    assert got.shape == want.shape
    assert np.array_equal(got, want)


def _correct_fine_case(oracle_mod, nd, mbc):
    cfg = CH2 if nd == 2 else CH3
    s = H.Spec(nd)
    if nd == 2:
        s.root_and_below(16, -1, [10] * 6)
        s.child(0, 101, [3, 5], [6, 10])   # touches nothing
        s.child(0, 102, [1, 11], [4, 16])  # at the low-x and high-y faces
    else:
        s.root_and_below(8, -1, [10] * 6)
        s.child(0, 101, [2, 3, 2], [5, 6, 5])
        s.child(0, 102, [1, 5, 5], [4, 8, 8])
    o = oracle_mod.OracleHierarchy(nd, 2, cfg["problem"], cfg["params"], mbc=mbc)
    s.apply(o)
    rng = np.random.default_rng(7 + nd + mbc)
    for p in s.patches:
        for fld in ("q", "qc"):
            o.put(p["id"], fld, rng.uniform(-1, 1, size=o.field_size(p["id"], fld)))
    return s, o


@pytest.mark.parametrize("nd", [2, 3])
@pytest.mark.parametrize("mbc", [1, 2])
def test_correct_fine_matches_the_reference_statements(oracle_mod, nd, mbc):
    """qc(1-mbc:cmx+mbc) = parent%q(mb-mbc:mb+mbc) - qc, then
    q(1-mbc:mx+mbc) += P1/P2(qc), for every patch of the level."""
    s, o = _correct_fine_case(oracle_mod, nd, mbc)
    byid = {p["id"]: p for p in s.patches}
    shape = lambda p, m: [m[d] + 2 * mbc for d in range(nd)] + [2]
    before = {p["id"]: (o.get(p["id"], "q"), o.get(p["id"], "qc")) for p in s.patches}
    o.correct_fine(1)
    for p in s.patches:
        if p["level"] != 1:
            continue
        par = byid[p["parent_id"]]
        pq = before[par["id"]][0].reshape(shape(par, par["mx"]), order="F")
        q = before[p["id"]][0].reshape(shape(p, p["mx"]), order="F")
        cmx = [m // 2 for m in p["mx"][:nd]]
        qc = before[p["id"]][1].reshape(shape(p, cmx), order="F")
        # parent Fortran index f sits at python f + mbc - 1
        win = tuple(slice(p["mbounds"][2 * d] - 1, p["mbounds"][2 * d + 1] + 2 * mbc) for d in range(nd))
        qc_new = pq[win] - qc
        q_new = q + PROL[nd, mbc](qc_new)
        assert np.array_equal(o.get(p["id"], "qc"), qc_new.ravel(order="F"))
        assert np.array_equal(o.get(p["id"], "q"), q_new.ravel(order="F"))


def _inner(a, mx, nd, nv, mbc):
    """q(0:mx+1) of a flat ghosted array with mbc layers"""
    a = a.reshape([m + 2 * mbc for m in mx[:nd]] + [nv], order="F")
    g = mbc - 1
    return a[tuple(slice(g, g + m + 2) for m in mx[:nd])]


class _Pair:
    """the same hierarchy with mbc = 1 and mbc = 2"""

    def __init__(self, oracle_mod, cfg, spec):
        self.h = [oracle_mod.OracleHierarchy(cfg["ndims"], 2, cfg["problem"], cfg["params"], mbc=m) for m in (1, 2)]
        for h in self.h:
            spec.apply(h)
        self.spec, self.nd = spec, cfg["ndims"]

    def put(self, pid, q1):
        """q1 in the one-layer layout goes to q(0:mx+1) of both"""
        p = next(x for x in self.spec.patches if x["id"] == pid)
        self.h[0].put(pid, "q", q1)
        mx = p["mx"][:self.nd]
        full = np.zeros([m + 4 for m in mx] + [2], order="F")
        full[tuple(slice(1, m + 3) for m in mx)] = np.asarray(q1).reshape([m + 2 for m in mx] + [2], order="F")
        self.h[1].put(pid, "q", full.ravel(order="F"))

    def compare(self):
        for p in self.spec.patches:
            a = self.h[0].get(p["id"], "q").reshape([m + 2 for m in p["mx"][:self.nd]] + [2], order="F")
            b = _inner(self.h[1].get(p["id"], "q"), p["mx"], self.nd, 2, 2)
            assert np.array_equal(a, b), p["id"]


CASES = {
    "ch2d-amr-periodic": (CH2, lambda: H.amr2d(periodic=True)),
    "ch2d-amr-neumann": (CH2, lambda: H.amr2d(periodic=False)),
    "ch3d-amr-periodic": (CH3, lambda: H.amr3d(periodic=True)),
}


@pytest.mark.parametrize("case", list(CASES))
def test_two_ghost_layers_give_the_one_layer_solution(oracle_mod, pkg, case):
    initial = pkg.initial
    cfg, mk = CASES[case]
    spec = mk()
    pr = _Pair(oracle_mod, cfg, spec)
    nd = cfg["ndims"]
    for p in spec.patches:
        pr.put(p["id"], initial.ch_spinodal(tuple(p["mx"][:nd]), cfg["params"][1], p["dx"][0], seed=61 + p["id"]))
    fin, mn = spec.finest(), spec.minlevel()
    for step in range(2):
        r = [h.time_step(step == 0, fin, mn, tol=1e-9, maxvcycles=20) for h in pr.h]
        assert r[0][0] == r[1][0] and np.array_equal(r[0][1], r[1][1]), (step, r)
    pr.compare()


def test_regrid_with_two_ghost_layers(oracle_mod):
    """The regrid (tagging on q, InitFields' P2MC, TransferValues) builds
    the one-layer run's mesh with the same interior values."""
    out = []
    for mbc in (1, 2):
        o = oracle_mod.OracleHierarchy(2, 2, "ch", [1e-3, 0.01], mbc=mbc)
        o.build_uniform([32, 32, 1], -4, [2, 2, 2, 2, 10, 10], [0, 0, 0], [1, 1, 1])
        o.commit()
        q = circle()(0, [32, 32], [1.0 / 32] * 2, [0.0, 0.0])
        if mbc == 2:
            full = np.zeros((36, 36, 2), order="F")
            full[1:35, 1:35] = q
            q = full
        o.put(0, "q", np.asarray(q).ravel(order="F"))
        prm = oracle_mod.regrid_params(2, qtolerance=0.05)
        a = oracle_mod.regrid(o, prm)
        b = oracle_mod.regrid(a, prm)
        out.append(b)
    ta, tb = out[0].patch_table(), out[1].patch_table()
    assert ta == tb
    for p in ta:
        qa = out[0].get(p["id"], "q").reshape([m + 2 for m in p["mx"][:2]] + [2], order="F")
        qb = _inner(out[1].get(p["id"], "q"), p["mx"], 2, 2, 2)
        assert np.array_equal(qa, qb), p["id"]
