"""The oracle against a literal numpy transcription of the reference's array
statements (no GPU).

The reference has no tests, so beyond the known-answer properties of
test_oracle_kat.py the oracle's arithmetic is pinned here by a second,
independent restatement of the Fortran source written as numpy array
expressions in the source's own evaluation order (IEEE double, no fused
multiply-add, like the oracle's -ffp-contract=off build):

* CH RelaxGrid2D / RelaxGrid3D (PROBLEM/CH/problem.f90:318-369, :554-614):
  one colour of the red-black update, compared bit for bit;
* CH Operator2D / Operator3D with ULap2D / ULap3D (CH:393-422, :638-669;
  LIBRARY/gridutilities.f90:50-72, :372-399) through Residual
  (afasroutines.f90:817-857): rf bit for bit;
* ErrorAFAS errortype 1 and 2 (afasroutines.f90:113-233) with SquareSum's
  sequential SUM: the norm bit for bit;
* BioGrowth RelaxGrid2D and Operator2D with Growth / Uptake
  (PROBLEM/BioGrowth/problem.f90:255-353, :743-766): bit for bit;
* Interpolate2D, the coarse-fine ghost statements (LIBRARY/boundary.f90:
  143-333) for ipass 0, 1 and 2: bit for bit;
* Interpolate3D (boundary.f90:1018-1550): corners, the 12 edges (with the
  z-face test of edges 1-4 that reads /= 99), the four colour classes of
  each face and the grey face corners, for ipass 0, 1, 2, inside the
  parent and at a physical face: bit for bit;
* the V-cycle's coarse branch in 2D and 3D: RestrictSolution with
  Restriction2D/3D, GetCoarseGhostPoints and CoarseLoadingFunction (the
  child's Residual, then Restriction(rf) + Operator(qc) at the parent's
  spacing): bit for bit;
* SelfPeriodicBC with the quasi-periodic offset qpo and SetPhysicalBC with
  CH UserBC2D / UserBC3D (boundary.f90:478-575, :640-800; CH:770-881) on a
  root patch, one and two ghost layers: bit for bit;
* TransferBC / GhostOverlap between touching siblings after their
  Interpolate2D (boundary.f90:336-480), and TransferPeriodicBC's
  GhostOverlap through every periodic offset (:582-605, :824-954): bit for
  bit;
* AFASVcycle / LevelRelax (afasroutines.f90:495-557) as the reference's
  sequence of those operations on 2D and 3D AMR hierarchies: the oracle's
  V-cycle equals it bit for bit;
* MultigridIterations (afasroutines.f90:48-110) as its sequence of FillDown,
  GetSourceFunction / UpdateSourceFunction, V-cycles and ErrorAFAS: the same
  V-cycle count, residuals and fields bit for bit;
* AfterStepStatistics with CH AfterStep2D, Energy2D and Ff
  (bsamroutines.f90:763-775, :918-963; CH/problem.f90:149-183, :512-547,
  :901-915) on a 2D AMR hierarchy: both integrals bit for bit;
* the regrid's clustering, NewSubGrids with GetSignatures and
  GridFlagRatio (bsamroutines.f90:1408-1662), on 160 random 2D and 3D flag
  fields, fill ratios and minimum sizes: the same boxes in the same order.
"""
import numpy as np
import pytest

CH = dict(dt=1e-3, eps=0.02)
BIO = dict(dt=0.1, eps=0.05, gamma=1.5, lam=2.0, czero=0.5)


def hierarchy(oracle_mod, nd, problem, params, mx, seed):
    o = oracle_mod.OracleHierarchy(nd, 2, problem, params)
    o.build_uniform(list(mx) + [1] * (3 - nd), 0, [10] * 6, [0, 0, 0],
                    [mx[d] / mx[0] if d < nd else 1.0 for d in range(3)])
    o.commit()
    rng = np.random.default_rng(seed)
    fields = {}
    for fld in ("q", "qold", "f"):
        a = rng.uniform(-1, 1, size=o.field_size(0, fld))
        o.put(0, fld, a)
        fields[fld] = a
    gh = [m + 2 for m in mx] + [2]
    return o, {k: v.reshape(gh if k != "f" else list(mx) + [2], order="F") for k, v in fields.items()}


def spacing(o):
    return o.patch_table()[0]["dx"][0]


def interior(nd, mx, di=(0, 0, 0)):
    """slice of the ghosted array for interior cells shifted by di"""
    return tuple(slice(1 + di[d], 1 + di[d] + mx[d]) for d in range(nd))


def ulap(a, nd, mx):
    """ULap2D / ULap3D: neighbours in the source's order minus (4|6) centre"""
    e = np.eye(3, dtype=int)
    r = a[interior(nd, mx, e[0])] + a[interior(nd, mx, -e[0])]
    r = r + a[interior(nd, mx, e[1])]
    r = r + a[interior(nd, mx, -e[1])]
    if nd == 3:
        r = r + a[interior(nd, mx, e[2])]
        r = r + a[interior(nd, mx, -e[2])]
    return r - (4.0 if nd == 2 else 6.0) * a[interior(nd, mx)]


def colour_mask(nd, mx, ipass):
    """cells i = 1 + MODULO(j (+k) + ipass, 2), ..., mx(1), 2"""
    idx = np.indices(mx) + 1
    return (idx.sum(axis=0) + ipass) % 2 == 1


def ch_relax(q, f, nd, mx, h, ipass, dt, eps):
    eps2 = eps * eps
    h2 = h * h
    tmp1, tmp2 = dt / h2, eps2 / h2
    tmp3 = (4.0 if nd == 2 else 6.0) * eps2 / h2
    a12 = (4.0 if nd == 2 else 6.0) * tmp1
    e = np.eye(3, dtype=int)
    q = q.copy()
    c = interior(nd, mx)
    phi, mu = q[c + (0,)], q[c + (1,)]

    def nb(v, order):
        s = None
        for d, sgn in order:
            t = q[interior(nd, mx, sgn * e[d]) + (v,)]
            s = t if s is None else s + t
        return s
    if nd == 2:
        s_mu = nb(1, [(0, -1), (0, 1), (1, -1), (1, 1)])   # q(i-1,j,2)+q(i+1,j,2)+q(i,j-1,2)+q(i,j+1,2)
        s_phi = nb(0, [(0, 1), (0, -1), (1, 1), (1, -1)])  # q(i+1,j,1)+q(i-1,j,1)+q(i,j+1,1)+q(i,j-1,1)
    else:
        s_mu = nb(1, [(0, -1), (0, 1), (1, -1), (1, 1), (2, -1), (2, 1)])
        s_phi = nb(0, [(0, 1), (0, -1), (1, 1), (1, -1), (2, 1), (2, -1)])
    a21 = -3.0 * (phi * phi) - tmp3
    b1 = f[..., 0] + tmp1 * s_mu
    b2 = f[..., 1] - tmp2 * s_phi - 2.0 * ((phi * phi) * phi)
    det = 1.0 - a12 * a21
    new_phi = (b1 - a12 * b2) / det
    new_mu = (b2 - a21 * b1) / det
    m = colour_mask(nd, mx, ipass)
    phi[m] = new_phi[m]
    mu[m] = new_mu[m]
    return q


def ch_residual(q, f, nd, mx, h, dt, eps):
    eps2 = eps * eps
    h2 = h * h
    tmp1, tmp2 = dt / h2, eps2 / h2
    c = interior(nd, mx)
    phi, mu = q[c + (0,)], q[c + (1,)]
    op1 = phi - tmp1 * ulap(q[..., 1], nd, mx)
    op2 = mu - ((phi * phi) * phi) + tmp2 * ulap(q[..., 0], nd, mx)
    return np.stack([f[..., 0] - op1, f[..., 1] - op2], axis=-1)


def error_afas(rf, errortype, nv=2):
    """SQRT(SUM(rf*rf) / (nrvars * cells)) with SUM in element order
    (errortype 1); the largest per-component value (errortype 2)"""
    seq = lambda a: np.cumsum(np.ravel(a * a, order="F"))[-1]
    cells = float(np.prod(rf.shape[:-1]))
    if errortype == 1:
        return float(np.sqrt(seq(rf) / (nv * cells)))
    return float(max(np.sqrt(seq(rf[..., v]) / cells) for v in range(nv)))


@pytest.mark.parametrize("nd,mx", [(2, (16, 12)), (3, (8, 6, 4))])
def test_ch_relax_is_the_reference_statements(oracle_mod, nd, mx):
    o, F = hierarchy(oracle_mod, nd, "ch", [CH["dt"], CH["eps"]], mx, 80 + nd)
    h = spacing(o)
    q = F["q"]
    for ipass in (1, 2):
        o.relax_level_color(0, ipass)
        q = ch_relax(q, F["f"], nd, list(mx), h, ipass, CH["dt"], CH["eps"])
        got = o.get(0, "q").reshape(q.shape, order="F")
        assert np.array_equal(got, q), (ipass, np.max(np.abs(got - q)))


@pytest.mark.parametrize("nd,mx", [(2, (16, 12)), (3, (8, 6, 4))])
@pytest.mark.parametrize("errortype", [1, 2])
def test_ch_residual_and_error_afas_are_the_reference_statements(oracle_mod, nd, mx, errortype):
    o, F = hierarchy(oracle_mod, nd, "ch", [CH["dt"], CH["eps"]], mx, 90 + nd)
    rf = ch_residual(F["q"], F["f"], nd, list(mx), spacing(o), CH["dt"], CH["eps"])
    norm = o.residual_norm(0, errortype)
    got = o.get(0, "rf").reshape(rf.shape, order="F")
    assert np.array_equal(got, rf)
    assert norm == error_afas(rf, errortype)


def bio_relax(q, qold, f, mx, h, ipass, p):
    dt, eps2 = p["dt"], p["eps"] * p["eps"]
    h2 = h * h
    tmp1, tmp3 = dt * eps2 / h2, 1.0 / h2
    growth = lambda x: p["gamma"] * 0.5 * (x + 1.0)
    uptake = lambda x: p["lam"] * 0.5 * (x + 1.0)
    q = q.copy()
    c = interior(2, mx)
    e = np.eye(3, dtype=int)
    sh = lambda v, d, s: q[interior(2, mx, s * e[d]) + (v,)]
    phi, n, po = q[c + (0,)], q[c + (1,)], qold[c + (0,)]
    tmp2 = 4.0 * tmp1 + 1.0 + dt * (phi * phi)
    new_phi = (f[..., 0] + dt * growth(po) * (n - p["czero"])
               + tmp1 * (sh(0, 0, -1) + sh(0, 0, 1) + sh(0, 1, -1) + sh(0, 1, 1))) / tmp2
    m = colour_mask(2, mx, ipass)
    phi[m] = new_phi[m]
    tmp4 = 4.0 * tmp3 + uptake(po)
    new_n = (f[..., 1] + tmp3 * (sh(1, 0, 1) + sh(1, 0, -1) + sh(1, 1, 1) + sh(1, 1, -1))) / tmp4
    n[m] = new_n[m]
    return q


def bio_residual(q, qold, f, mx, h, p):
    dt, eps2 = p["dt"], p["eps"] * p["eps"]
    h2 = h * h
    tmp1, tmp3 = dt * eps2 / h2, 1.0 / h2
    growth = lambda x: p["gamma"] * 0.5 * (x + 1.0)
    uptake = lambda x: p["lam"] * 0.5 * (x + 1.0)
    c = interior(2, mx)
    phi, n, po = q[c + (0,)], q[c + (1,)], qold[c + (0,)]
    op1 = phi - tmp1 * ulap(q[..., 0], 2, mx) + dt * ((phi * phi) * phi) - dt * growth(po) * (n - p["czero"])
    op2 = -tmp3 * ulap(q[..., 1], 2, mx) + uptake(po) * n
    return np.stack([f[..., 0] - op1, f[..., 1] - op2], axis=-1)


def test_biogrowth_relax_and_residual_are_the_reference_statements(oracle_mod):
    mx = [16, 12]
    params = [BIO["dt"], BIO["eps"], BIO["gamma"], BIO["lam"], BIO["czero"]]
    o, F = hierarchy(oracle_mod, 2, "biogrowth", params, mx, 77)
    h = spacing(o)
    rf = bio_residual(F["q"], F["qold"], F["f"], mx, h, BIO)
    assert o.residual_norm(0, 1) == error_afas(rf, 1)
    assert np.array_equal(o.get(0, "rf").reshape(rf.shape, order="F"), rf)
    q = F["q"]
    for ipass in (1, 2):
        o.relax_level_color(0, ipass)
        q = bio_relax(q, F["qold"], F["f"], mx, h, ipass, BIO)
        assert np.array_equal(o.get(0, "q").reshape(q.shape, order="F"), q), ipass


# --- Interpolate2D (LIBRARY/boundary.f90:143-333), constants :54-63 -------
A1, A2, A3 = -1.0 / 5.0, 2.0 / 3.0, 8.0 / 15.0
B1, B2, B3 = 5.0 / 32.0, 15.0 / 16.0, -3.0 / 32.0


def interpolate2d(qf, qc, mx, mb, mthbc, ipass):
    """The C/F ghost statements on qf(0:mx+1,0:my+1,:) from the parent's
    qc(0:,0:,:); Fortran index = python index, a:b:2 inclusive."""
    qf = qf.copy()
    m0, m1 = mx
    (l0, h0), (l1, h1) = mb
    red, black = ipass in (1, 0), ipass in (2, 0)
    s = lambda a, b: slice(a, b + 1, 2)
    r = lambda a, b: slice(a, b + 1)
    if red:
        qf[m0 + 1, m1 + 1] = A1 * qf[m0 - 1, m1 - 1] + A2 * qf[m0, m1] + A3 * qc[h0 + 1, h1 + 1]
        qf[0, 0] = A1 * qf[2, 2] + A2 * qf[1, 1] + A3 * qc[l0 - 1, l1 - 1]
    if black:
        qf[m0 + 1, 0] = A1 * qf[m0 - 1, 2] + A2 * qf[m0, 1] + A3 * qc[h0 + 1, l1 - 1]
        qf[0, m1 + 1] = A1 * qf[2, m1 - 1] + A2 * qf[1, m1] + A3 * qc[l0 - 1, h1 + 1]
    bsum = lambda u, v, w: A3 * (B1 * u + B2 * v + B3 * w)
    if mthbc[0] in (2, 999):
        if red:
            qf[0, s(2, m1 - 2)] = A1 * qf[2, s(4, m1)] + A2 * qf[1, s(3, m1 - 1)] + A3 * qc[l0 - 1, r(l1, h1 - 1)]
            qf[0, m1] = A1 * qf[2, m1] + A2 * qf[1, m1] + bsum(qc[l0 - 1, h1 + 1], qc[l0 - 1, h1], qc[l0 - 1, h1 - 1])
        if black:
            qf[0, s(3, m1 - 1)] = A1 * qf[2, s(1, m1 - 3)] + A2 * qf[1, s(2, m1 - 2)] + A3 * qc[l0 - 1, r(l1 + 1, h1)]
            qf[0, 1] = A1 * qf[2, 1] + A2 * qf[1, 1] + bsum(qc[l0 - 1, l1 - 1], qc[l0 - 1, l1], qc[l0 - 1, l1 + 1])
    if mthbc[1] in (2, 999):
        if red:
            qf[m0 + 1, s(3, m1 - 1)] = (A1 * qf[m0 - 1, s(1, m1 - 3)] + A2 * qf[m0, s(2, m1 - 2)]
                                        + A3 * qc[h0 + 1, r(l1 + 1, h1)])
            qf[m0 + 1, 1] = A1 * qf[m0 - 1, 1] + A2 * qf[m0, 1] + bsum(qc[h0 + 1, l1 - 1], qc[h0 + 1, l1],
                                                                       qc[h0 + 1, l1 + 1])
        if black:
            qf[m0 + 1, s(2, m1 - 2)] = (A1 * qf[m0 - 1, s(4, m1)] + A2 * qf[m0, s(3, m1 - 1)]
                                        + A3 * qc[h0 + 1, r(l1, h1 - 1)])
            qf[m0 + 1, m1] = A1 * qf[m0 - 1, m1] + A2 * qf[m0, m1] + bsum(qc[h0 + 1, h1 + 1], qc[h0 + 1, h1],
                                                                          qc[h0 + 1, h1 - 1])
    if mthbc[2] in (2, 999):
        if red:
            qf[s(2, m0 - 2), 0] = A1 * qf[s(4, m0), 2] + A2 * qf[s(3, m0 - 1), 1] + A3 * qc[r(l0, h0 - 1), l1 - 1]
            qf[m0, 0] = A1 * qf[m0, 2] + A2 * qf[m0, 1] + bsum(qc[h0 + 1, l1 - 1], qc[h0, l1 - 1], qc[h0 - 1, l1 - 1])
        if black:
            qf[s(3, m0 - 1), 0] = A1 * qf[s(1, m0 - 3), 2] + A2 * qf[s(2, m0 - 2), 1] + A3 * qc[r(l0 + 1, h0), l1 - 1]
            qf[1, 0] = A1 * qf[1, 2] + A2 * qf[1, 1] + bsum(qc[l0 - 1, l1 - 1], qc[l0, l1 - 1], qc[l0 + 1, l1 - 1])
    if mthbc[3] in (2, 999):
        if red:
            qf[s(3, m0 - 1), m1 + 1] = (A1 * qf[s(1, m0 - 3), m1 - 1] + A2 * qf[s(2, m0 - 2), m1]
                                        + A3 * qc[r(l0 + 1, h0), h1 + 1])
            qf[1, m1 + 1] = A1 * qf[1, m1 - 1] + A2 * qf[1, m1] + bsum(qc[l0 - 1, h1 + 1], qc[l0, h1 + 1],
                                                                       qc[l0 + 1, h1 + 1])
        if black:
            qf[s(2, m0 - 2), m1 + 1] = (A1 * qf[s(4, m0), m1 - 1] + A2 * qf[s(3, m0 - 1), m1]
                                        + A3 * qc[r(l0, h0 - 1), h1 + 1])
            qf[m0, m1 + 1] = A1 * qf[m0, m1 - 1] + A2 * qf[m0, m1] + bsum(qc[h0 + 1, h1 + 1], qc[h0, h1 + 1],
                                                                          qc[h0 - 1, h1 + 1])
    return qf


@pytest.mark.parametrize("ipass", [0, 1, 2])
def test_cf_interpolation_2d_is_the_reference_statements(oracle_mod, ipass):
    """SetGhost on a child with internal faces only (no siblings, no
    physical or periodic faces) is Interpolate2D alone."""
    from tests import hierarchies as H
    s = H.Spec(2)
    s.root_and_below(16, 0, [10] * 6)
    s.child(0, 101, [5, 4], [10, 11])  # 12 x 16 fine cells, faces internal
    o = oracle_mod.OracleHierarchy(2, 2, "ch", [CH["dt"], CH["eps"]])
    s.apply(o)
    rng = np.random.default_rng(50 + ipass)
    q = {}
    for p in s.patches:
        a = rng.uniform(-1, 1, size=o.field_size(p["id"], "q"))
        o.put(p["id"], "q", a)
        q[p["id"]] = a.reshape([m + 2 for m in p["mx"][:2]] + [2], order="F")
    child = s.patches[-1]
    o.set_ghost(1, ipass)
    mb = [(child["mbounds"][0], child["mbounds"][1]), (child["mbounds"][2], child["mbounds"][3])]
    want = interpolate2d(q[101], q[0], child["mx"][:2], mb, child["mthbc"][:4], ipass)
    got = o.get(101, "q").reshape(want.shape, order="F")
    assert np.array_equal(got, want)


# --- RestrictSolution, GetCoarseGhostPoints, CoarseLoadingFunction --------
# (afasroutines.f90:610-652, :673-736; boundary.f90:957-1015; Restriction2D/
# 3D gridutilities.f90:103-127, :437-468)

def restriction(a, nd):
    """a: interior values (Fortran 1..mx -> python 0..mx-1), variables last;
    2:mx:2 is python 1::2 and 1:mx-1:2 python 0::2"""
    e, o = slice(1, None, 2), slice(0, None, 2)
    if nd == 2:
        return 0.25 * (a[e, e] + a[o, e] + a[e, o] + a[o, o])
    t = [(e, e, e), (o, e, e), (e, o, e), (o, o, e), (e, e, o), (o, e, o), (e, o, o), (o, o, o)]
    s = a[t[0]]
    for x in t[1:]:
        s = s + a[x]
    return 0.125 * s


def ch_operator(q, nd, mx, h, dt, eps):
    eps2 = eps * eps
    h2 = h * h
    tmp1, tmp2 = dt / h2, eps2 / h2
    c = interior(nd, mx)
    phi, mu = q[c + (0,)], q[c + (1,)]
    return np.stack([phi - tmp1 * ulap(q[..., 1], nd, mx),
                     mu - ((phi * phi) * phi) + tmp2 * ulap(q[..., 0], nd, mx)], axis=-1)


@pytest.mark.parametrize("nd", [2, 3])
def test_coarse_branch_is_the_reference_statements(oracle_mod, nd):
    from tests import hierarchies as H
    s = H.Spec(nd)
    if nd == 2:
        s.root_and_below(16, 0, [10] * 6)
        s.child(0, 101, [3, 5], [8, 12])
    else:
        s.root_and_below(8, 0, [10] * 6)
        s.child(0, 101, [2, 3, 2], [5, 6, 7])
    o = oracle_mod.OracleHierarchy(nd, 2, "ch", [CH["dt"], CH["eps"]])
    s.apply(o)
    root, child = s.patches[0], s.patches[-1]
    rng = np.random.default_rng(60 + nd)
    arr = {}
    for p in (root, child):
        for fld in ("q", "qold", "qc", "f"):
            a = rng.uniform(-1, 1, size=o.field_size(p["id"], fld))
            o.put(p["id"], fld, a)
            arr[p["id"], fld] = a
    mx, cmx, pmx = child["mx"][:nd], [m // 2 for m in child["mx"][:nd]], root["mx"][:nd]
    shp = lambda m, g: [x + 2 * g for x in m] + [2]
    q = arr[101, "q"].reshape(shp(mx, 1), order="F")
    qc = arr[101, "qc"].reshape(shp(cmx, 1), order="F")
    pq = arr[0, "q"].reshape(shp(pmx, 1), order="F")
    f = arr[101, "f"].reshape(shp(mx, 0), order="F")
    lo = [child["mbounds"][2 * d] for d in range(nd)]
    under = tuple(slice(lo[d], lo[d] + cmx[d]) for d in range(nd))  # parent cells mb(1):mb(2)
    # RestrictSolution
    o.level_op(1, "restrict")
    r = restriction(q[interior(nd, mx)], nd)
    qc[interior(nd, cmx)] = r
    pq[under] = r
    assert np.array_equal(o.get(101, "qc").reshape(qc.shape, order="F"), qc)
    assert np.array_equal(o.get(0, "q").reshape(pq.shape, order="F"), pq)
    # GetCoarseGhostPoints: every ring cell of qc(0:cmx+1) from parent%q(mb-1+i, ...)
    o.level_op(1, "coarse_ghost")
    idx = np.indices([c + 2 for c in cmx])
    ring = np.zeros(idx.shape[1:], dtype=bool)
    for d in range(nd):
        ring |= (idx[d] == 0) | (idx[d] == cmx[d] + 1)
    for cell in zip(*np.nonzero(ring)):
        qc[cell] = pq[tuple(lo[d] - 1 + cell[d] for d in range(nd))]
    assert np.array_equal(o.get(101, "qc").reshape(qc.shape, order="F"), qc)
    # CoarseLoadingFunction: Residual on the child, then parent%f(mb) =
    # Restriction(rf) + Operator(qc(0:cmx+1)) at the parent's spacing
    o.level_op(1, "coarse_load")
    rf = f - ch_operator(q, nd, mx, child["dx"][0], CH["dt"], CH["eps"])
    pf = arr[0, "f"].reshape(shp(pmx, 0), order="F").copy()
    pf[tuple(slice(lo[d] - 1, lo[d] - 1 + cmx[d]) for d in range(nd))] = (
        restriction(rf, nd) + ch_operator(qc, nd, cmx, root["dx"][0], CH["dt"], CH["eps"]))
    assert np.array_equal(o.get(101, "rf").reshape(rf.shape, order="F"), rf)
    assert np.array_equal(o.get(0, "f").reshape(pf.shape, order="F"), pf)


# --- SelfPeriodicBC and SetPhysicalBC2D/3D with CH UserBC2D/3D -----------
# (boundary.f90:478-575, :640-800; CH/problem.f90:770-881).  A root patch:
# SetGhost(rootlevel) is SelfPeriodicBC then SetPhysicalBC.

def root_ghosts(q, nd, mx, mbc, mthbc, qpo):
    """q indexed from 1-mbc (python = Fortran + mbc - 1), variables last"""
    q = q.copy()
    o = mbc - 1
    F = lambda i: i + o  # Fortran index -> python index
    nv = q.shape[-1]
    ax = lambda d, i: tuple(F(i) if e == d else slice(None) for e in range(nd))
    # SelfPeriodicBC: x with the quasi-periodic offset, then y (then z)
    if mthbc[0] == 2 and mthbc[1] == 2:
        for ibc in range(1, mbc + 1):
            for n in range(nv):
                q[ax(0, mx[0] + ibc) + (n,)] = q[ax(0, ibc) + (n,)] + qpo[n]
                q[ax(0, 1 - ibc) + (n,)] = q[ax(0, mx[0] + 1 - ibc) + (n,)] - qpo[n]
    for d in range(1, nd):
        if mthbc[2 * d] == 2 and mthbc[2 * d + 1] == 2:
            for ibc in range(1, mbc + 1):
                q[ax(d, mx[d] + ibc)] = q[ax(d, ibc)]
                q[ax(d, 1 - ibc)] = q[ax(d, mx[d] + 1 - ibc)]
    # SetPhysicalBC: faces in order, UserBC2D reflects, UserBC3D is 2 - q
    refl = (lambda v: v) if nd == 2 else (lambda v: 2.0 - v)
    for face in range(2 * nd):
        if mthbc[face] != 10:
            continue
        d, hi = face // 2, face % 2
        for ibc in range(1, mbc + 1):
            if hi:
                q[ax(d, mx[d] + ibc)] = refl(q[ax(d, mx[d] - ibc + 1)])
            else:
                q[ax(d, 1 - ibc)] = refl(q[ax(d, ibc)])
    return q


@pytest.mark.parametrize("nd,mthbc", [(2, [10, 10, 10, 10]), (2, [2, 2, 10, 10]), (2, [2, 2, 2, 2]),
                                      (3, [10] * 6), (3, [2, 2, 10, 10, 2, 2]), (3, [2] * 6)])
@pytest.mark.parametrize("mbc", [1, 2])
def test_root_ghosts_are_the_reference_statements(oracle_mod, nd, mthbc, mbc):
    mx = [12, 8, 6][:nd]
    qpo = [0.25, -0.5]
    o = oracle_mod.OracleHierarchy(nd, 2, "ch", [CH["dt"], CH["eps"]], qpo=qpo, mbc=mbc)
    o.build_uniform(mx + [1] * (3 - nd), 0, mthbc + [10] * (6 - 2 * nd), [0, 0, 0],
                    [mx[d] / mx[0] if d < nd else 1.0 for d in range(3)])
    o.commit()
    rng = np.random.default_rng(sum(mthbc) + 7 * mbc + nd)
    a = rng.uniform(-1, 1, size=o.field_size(0, "q"))
    o.put(0, "q", a)
    q = a.reshape([m + 2 * mbc for m in mx] + [2], order="F")
    o.set_ghost(0, 0)
    want = root_ghosts(q, nd, mx, mbc, mthbc, qpo)
    assert np.array_equal(o.get(0, "q").reshape(want.shape, order="F"), want)


# --- TransferBC / GhostOverlap (boundary.f90:336-480) after Interpolate2D --

def ghost_overlap(q1, q2, mg1, mg2, mbc, nd):
    """grid1's ghost cells from grid2's interior and back; q indexed from 0
    (mbc = 1: python = Fortran), mg = [(lo, hi)] per dimension"""
    ovg = [(max(mg1[n][0] - mbc, mg2[n][0] - mbc), min(mg1[n][1] + mbc, mg2[n][1] + mbc)) for n in range(nd)]
    if any(h < l for l, h in ovg):
        return
    ov1 = [(max(ovg[n][0], mg2[n][0]), min(ovg[n][1], mg2[n][1])) for n in range(nd)]
    ov2 = [(max(ovg[n][0], mg1[n][0]), min(ovg[n][1], mg1[n][1])) for n in range(nd)]
    loc = lambda ov, mg: tuple(slice(ov[n][0] - mg[n][0] + 1, ov[n][1] - mg[n][0] + 2) for n in range(nd))
    q1[loc(ov1, mg1)] = q2[loc(ov1, mg2)]
    q2[loc(ov2, mg2)] = q1[loc(ov2, mg1)]


def test_sibling_transfer_after_interpolation_is_the_reference_statements(oracle_mod):
    """Two touching siblings with internal faces: SetGhost(level, 0) is
    Interpolate2D on each, then GhostOverlap of the pair."""
    from tests import hierarchies as H
    s = H.Spec(2)
    s.root_and_below(16, 0, [10] * 6)
    s.child(0, 101, [3, 3], [6, 8])
    s.child(0, 102, [7, 5], [10, 10])
    o = oracle_mod.OracleHierarchy(2, 2, "ch", [CH["dt"], CH["eps"]])
    s.apply(o)
    rng = np.random.default_rng(99)
    q = {}
    for p in s.patches:
        a = rng.uniform(-1, 1, size=o.field_size(p["id"], "q"))
        o.put(p["id"], "q", a)
        q[p["id"]] = a.reshape([m + 2 for m in p["mx"][:2]] + [2], order="F")
    o.set_ghost(1, 0)
    want = {}
    for p in s.patches[1:]:
        mb = [(p["mbounds"][0], p["mbounds"][1]), (p["mbounds"][2], p["mbounds"][3])]
        want[p["id"]] = interpolate2d(q[p["id"]], q[0], p["mx"][:2], mb, p["mthbc"][:4], 0)
    a, b = s.patches[1], s.patches[2]
    mg = lambda p: [(p["mglobal"][0], p["mglobal"][1]), (p["mglobal"][2], p["mglobal"][3])]
    ghost_overlap(want[101], want[102], mg(a), mg(b), 1, 2)
    for pid in (101, 102):
        assert np.array_equal(o.get(pid, "q").reshape(want[pid].shape, order="F"), want[pid]), pid


# --- AFASVcycle / LevelRelax composition (afasroutines.f90:495-557) -------

def afas_vcycle(o, level, minlevel, nsmooth):
    """The reference's recursive V-cycle written with the oracle's single
    operations (each pinned above): LevelRelax, then RestrictSolution,
    SetGhost(level-1, 0), GetCoarseGhostPoints, GetCoarseLevelLoading, the
    coarser cycle, CorrectFine, SetGhost(level, 0), LevelRelax"""
    def level_relax(l):
        for _ in range(nsmooth):
            for rb in (1, 2):
                o.relax_level_color(l, rb)
                o.set_ghost(l, rb)
    level_relax(level)
    if level > minlevel:
        o.level_op(level, "restrict")
        o.set_ghost(level - 1, 0)
        o.level_op(level, "coarse_ghost")
        o.level_op(level, "coarse_load")
        afas_vcycle(o, level - 1, minlevel, nsmooth)
        o.correct_fine(level)
        o.set_ghost(level, 0)
        level_relax(level)


@pytest.mark.parametrize("nd", [2, 3])
def test_vcycle_is_the_reference_composition(oracle_mod, nd):
    """The oracle's V-cycle equals the reference's sequence of operations on
    an AMR hierarchy with levels below the root, bit for bit."""
    from tests import hierarchies as H
    s = H.amr2d(periodic=True) if nd == 2 else H.amr3d(periodic=False)
    params = [1e-3, 0.01] if nd == 2 else [5e-4, 0.02]
    a, b = (oracle_mod.OracleHierarchy(nd, 2, "ch", params) for _ in range(2))
    s.apply(a)
    s.apply(b)
    rng = np.random.default_rng(5 + nd)
    for p in s.patches:
        for fld in ("q", "qold", "f"):
            v = rng.uniform(-1, 1, size=a.field_size(p["id"], fld))
            a.put(p["id"], fld, v)
            b.put(p["id"], fld, v)
    fin, mn = s.finest(), s.minlevel()
    a.vcycle(fin, mn, 2)
    afas_vcycle(b, fin, mn, 2)
    for p in s.patches:
        for fld in ("q", "qc", "f", "rf"):
            assert np.array_equal(a.get(p["id"], fld), b.get(p["id"], fld)), (p["id"], fld)


# --- FillDown and MultigridIterations composition (afasroutines.f90:48-110,
# :236-327, :330-492) ------------------------------------------------------

def fill_down(o, field, finest, minlevel):
    """FillDown: FillDownLevel from the finest level down, SetGhost(level-1,
    0) after each level when the field is the solution"""
    for level in range(finest, minlevel, -1):
        o.level_op(level, "fill_q" if field == "q" else "fill_f")
        if field == "q":
            o.set_ghost(level - 1, 0)


def multigrid_iterations(o, finest, minlevel, nsmooth, maxvcycles, tol):
    fill_down(o, "q", finest, minlevel)
    for level in range(finest, -1, -1):  # finestlevel .. rootlevel
        o.level_op(level, "get_source")
    for level in range(finest, -1, -1):
        o.level_op(level, "update_source")
    fill_down(o, "f", finest, minlevel)
    res = []
    for _ in range(maxvcycles):
        afas_vcycle(o, finest, minlevel, nsmooth)
        fill_down(o, "q", finest, minlevel)
        for level in range(finest, -1, -1):
            o.level_op(level, "update_source")
        fill_down(o, "f", finest, minlevel)
        res.append(o.residual_norm(finest, 1))
        if res[-1] < tol:
            break
    return len(res), res


def test_multigrid_iterations_are_the_reference_composition(oracle_mod, pkg):
    """The oracle's MultigridIterations equals the reference's sequence
    (FillDown, source functions, V-cycles, ErrorAFAS) of pinned operations:
    the same V-cycle count, residuals and fields bit for bit; CH's
    Source2D is (qold_phi, -qold_phi) in ftmp, SourceUpdate2D zero."""
    from tests import hierarchies as H
    s = H.amr2d(periodic=False)
    a, b = (oracle_mod.OracleHierarchy(2, 2, "ch", [1e-3, 0.01]) for _ in range(2))
    s.apply(a)
    s.apply(b)
    for p in s.patches:
        q = pkg.initial.ch_spinodal(tuple(p["mx"][:2]), 0.01, p["dx"][0], seed=40 + p["id"])
        for h in (a, b):
            h.put(p["id"], "q", q)
            h.copy_q_to_qold(s.minlevel(), s.finest())
    fin, mn = s.finest(), s.minlevel()
    na, ra = a.multigrid_iterations(fin, mn, 2, 20, 1e-9)
    nb, rb = multigrid_iterations(b, fin, mn, 2, 20, 1e-9)
    assert na == nb and list(ra[:na]) == rb, (na, nb, ra, rb)
    for p in s.patches:
        for fld in ("q", "qc", "f", "ftmp"):
            assert np.array_equal(a.get(p["id"], fld), b.get(p["id"], fld)), (p["id"], fld)
    # the source statements themselves on the finest level
    for p in s.patches:
        if p["level"] == fin:
            qold = b.get(p["id"], "qold").reshape([m + 2 for m in p["mx"][:2]] + [2], order="F")
            ftmp = b.get(p["id"], "ftmp").reshape(p["mx"][:2] + [2], order="F")
            assert np.array_equal(ftmp[..., 0], qold[1:-1, 1:-1, 0])
            assert np.array_equal(ftmp[..., 1], -qold[1:-1, 1:-1, 0])


# --- Interpolate3D (LIBRARY/boundary.f90:1018-1550) ------------------------
C1, C2, C3, C4 = 9.0 / 16.0, 3.0 / 16.0, 3.0 / 16.0, 1.0 / 16.0


def face_index(mx, mb, d, parity):
    """GetFaceIndex (:1018-1045): ghost, second and first interior cells
    along d, the coarse cell beyond the patch and the one at its edge"""
    if parity == 1:
        return (0, 2, 1, mb[d][0] - 1, mb[d][0])
    return (mx[d] + 1, mx[d] - 1, mx[d], mb[d][1] + 1, mb[d][1])


def interpolate3d(qf, qc, mx, mb, mthbc, ipass):
    """qf(0:mx+1, ...) and qc(0:, ...) indexed as in Fortran; mb[d] =
    (lo, hi); every statement assigns cells no other statement reads, so
    each is applied to the incoming array"""
    qf = qf.copy()
    src = qf.copy()
    s = lambda a, b: slice(a, b + 1, 2)
    r = lambda a, b: slice(a, b + 1)
    ok = lambda face: not (mthbc[face] not in (2, 999) and ipass == 1)

    def at(pos):  # {dim: index or slice} -> index tuple
        return tuple(pos[d] for d in range(3))

    # (1) the 8 corners
    for p1 in (1, 2):
        if not ok(p1 - 1):
            continue
        f1 = face_index(mx, mb, 0, p1)
        for p2 in (1, 2):
            if not ok(p2 + 1):
                continue
            f2 = face_index(mx, mb, 1, p2)
            for p3 in (1, 2):
                if not ok(p3 + 3):
                    continue
                f3 = face_index(mx, mb, 2, p3)
                qf[f1[0], f2[0], f3[0]] = (A1 * src[f1[1], f2[1], f3[1]] + A2 * src[f1[2], f2[2], f3[2]]
                                           + A3 * qc[f1[3], f2[3], f3[3]])

    # (2) the 12 edges: fixed dims (da, db), running along w
    def edge(da, fa, db, fb, w):
        m, (lo, hi) = mx[w], mb[w]

        def P(k, wv):
            pos = {da: fa[k], db: fb[k], w: wv}
            return at(pos)

        def Q(wv):
            return qc[at({da: fa[3], db: fb[3], w: wv})]
        qf[P(0, s(3, m - 1))] = A1 * src[P(1, s(1, m - 3))] + A2 * src[P(2, s(2, m - 2))] + A3 * Q(r(lo + 1, hi))
        qf[P(0, 1)] = A1 * src[P(1, 1)] + A2 * src[P(2, 1)] + A3 * (B1 * Q(lo - 1) + B2 * Q(lo) + B3 * Q(lo + 1))
        qf[P(0, s(2, m - 2))] = A1 * src[P(1, s(4, m))] + A2 * src[P(2, s(3, m - 1))] + A3 * Q(r(lo, hi - 1))
        qf[P(0, m)] = A1 * src[P(1, m)] + A2 * src[P(2, m)] + A3 * (B1 * Q(hi + 1) + B2 * Q(hi) + B3 * Q(hi - 1))

    for p1 in (1, 2):  # edges 1-4 (coordinates 1 and 3 fixed); the z test reads /= 99 (:1106)
        if not ok(p1 - 1):
            continue
        for p3 in (1, 2):
            if mthbc[p3 + 3] != 2 and mthbc[p3 + 3] != 99 and ipass == 1:
                continue
            edge(0, face_index(mx, mb, 0, p1), 2, face_index(mx, mb, 2, p3), 1)
    for p1 in (1, 2):  # edges 5-8 (coordinates 1 and 2 fixed)
        if not ok(p1 - 1):
            continue
        for p2 in (1, 2):
            if not ok(p2 + 1):
                continue
            edge(0, face_index(mx, mb, 0, p1), 1, face_index(mx, mb, 1, p2), 2)
    for p2 in (1, 2):  # edges 9-12 (coordinates 2 and 3 fixed)
        if not ok(p2 + 1):
            continue
        for p3 in (1, 2):
            if not ok(p3 + 3):
                continue
            edge(1, face_index(mx, mb, 1, p2), 2, face_index(mx, mb, 2, p3), 0)

    # (3) the 6 faces, periodic or internal only: normal n, in-face (u, v)
    for n, (ud, vd) in ((0, (1, 2)), (1, (0, 2)), (2, (0, 1))):
        for p in (1, 2):
            if mthbc[2 * n + p - 1] not in (2, 999):
                continue
            fn = face_index(mx, mb, n, p)
            mu, mv = mx[ud], mx[vd]
            (ul, uh), (vl, vh) = mb[ud], mb[vd]

            def F(k, u, v):
                return at({n: fn[k], ud: u, vd: v})

            def Q(u, v):
                return qc[at({n: fn[3], ud: u, vd: v})]

            def put(u, v, du2, dv2, du1, dv1, coarse):
                qf[F(0, u, v)] = A1 * src[F(1, du2, dv2)] + A2 * src[F(2, du1, dv1)] + A3 * coarse

            if ipass == 0 or (p + ipass) % 2 == 0:
                # yellow
                put(s(2, mu - 2), s(2, mv - 2), s(4, mu), s(4, mv), s(3, mu - 1), s(3, mv - 1), Q(r(ul, uh - 1), r(vl, vh - 1)))
                put(mu, s(2, mv - 2), mu, s(4, mv), mu, s(3, mv - 1),
                    B1 * Q(uh + 1, r(vl, vh - 1)) + B2 * Q(uh, r(vl, vh - 1)) + B3 * Q(uh - 1, r(vl, vh - 1)))
                put(s(2, mu - 2), mv, s(4, mu), mv, s(3, mu - 1), mv,
                    B1 * Q(r(ul, uh - 1), vh + 1) + B2 * Q(r(ul, uh - 1), vh) + B3 * Q(r(ul, uh - 1), vh - 1))
                # blue
                put(s(3, mu - 1), s(3, mv - 1), s(1, mu - 3), s(1, mv - 3), s(2, mu - 2), s(2, mv - 2), Q(r(ul + 1, uh), r(vl + 1, vh)))
                put(s(3, mu - 1), 1, s(1, mu - 3), 1, s(2, mu - 2), 1,
                    B1 * Q(r(ul + 1, uh), vl - 1) + B2 * Q(r(ul + 1, uh), vl) + B3 * Q(r(ul + 1, uh), vl + 1))
                put(1, s(3, mv - 1), 1, s(1, mv - 3), 1, s(2, mv - 2),
                    B1 * Q(ul - 1, r(vl + 1, vh)) + B2 * Q(ul, r(vl + 1, vh)) + B3 * Q(ul + 1, r(vl + 1, vh)))
            if ipass == 0 or (p + ipass) % 2 == 1:
                # green
                put(s(3, mu - 1), s(2, mv - 2), s(1, mu - 3), s(4, mv), s(2, mu - 2), s(3, mv - 1), Q(r(ul + 1, uh), r(vl, vh - 1)))
                put(1, s(2, mv - 2), 1, s(4, mv), 1, s(3, mv - 1),
                    B1 * Q(ul - 1, r(vl, vh - 1)) + B2 * Q(ul, r(vl, vh - 1)) + B3 * Q(ul + 1, r(vl, vh - 1)))
                put(s(3, mu - 1), mv, s(1, mu - 3), mv, s(2, mu - 2), mv,
                    B1 * Q(r(ul + 1, uh), vh + 1) + B2 * Q(r(ul + 1, uh), vh) + B3 * Q(r(ul + 1, uh), vh - 1))
                # red
                put(s(2, mu - 2), s(3, mv - 1), s(4, mu), s(1, mv - 3), s(3, mu - 1), s(2, mv - 2), Q(r(ul, uh - 1), r(vl + 1, vh)))
                put(s(2, mu - 2), 1, s(4, mu), 1, s(3, mu - 1), 1,
                    B1 * Q(r(ul, uh - 1), vl - 1) + B2 * Q(r(ul, uh - 1), vl) + B3 * Q(r(ul, uh - 1), vl + 1))
                put(mu, s(3, mv - 1), mu, s(1, mv - 3), mu, s(2, mv - 2),
                    B1 * Q(uh + 1, r(vl + 1, vh)) + B2 * Q(uh, r(vl + 1, vh)) + B3 * Q(uh - 1, r(vl + 1, vh)))
            # grey corner cells of the face, every ipass
            for pu in (1, 2):
                fu = face_index(mx, mb, ud, pu)
                for pv in (1, 2):
                    fv = face_index(mx, mb, vd, pv)
                    put(fu[2], fv[2], fu[2], fv[2], fu[2], fv[2],
                        C1 * Q(fu[4], fv[4]) + C2 * Q(fu[3], fv[4]) + C3 * Q(fu[4], fv[3]) + C4 * Q(fu[3], fv[3]))
    return qf


@pytest.mark.parametrize("ipass", [0, 1, 2])
@pytest.mark.parametrize("where", ["inside", "at-low-x"])
def test_cf_interpolation_3d_is_the_reference_statements(oracle_mod, ipass, where):
    """SetGhost on one 3D child: Interpolate3D (corners, the 12 edges with
    the z-face test of edges 1-4 reading /= 99, the yellow/blue/green/red
    face classes and the grey face corners), then the physical boundary of
    a face the child shares with the root (UserBC3D, 2 - q)."""
    from tests import hierarchies as H
    s = H.Spec(3)
    s.root_and_below(8, 0, [10] * 6)
    if where == "inside":
        s.child(0, 101, [2, 3, 2], [5, 6, 7])
    else:
        s.child(0, 101, [1, 3, 2], [4, 6, 7])
    o = oracle_mod.OracleHierarchy(3, 2, "ch", [CH["dt"], CH["eps"]])
    s.apply(o)
    rng = np.random.default_rng(70 + ipass + (where == "inside"))
    q = {}
    for p in s.patches:
        a = rng.uniform(-1, 1, size=o.field_size(p["id"], "q"))
        o.put(p["id"], "q", a)
        q[p["id"]] = a.reshape([m + 2 for m in p["mx"][:3]] + [2], order="F")
    child = s.patches[-1]
    o.set_ghost(1, ipass)
    mx = child["mx"][:3]
    mb = [(child["mbounds"][2 * d], child["mbounds"][2 * d + 1]) for d in range(3)]
    want = interpolate3d(q[101], q[0], mx, mb, child["mthbc"], ipass)
    want = root_ghosts(want, 3, mx, 1, child["mthbc"], [0.0, 0.0])
    got = o.get(101, "q").reshape(want.shape, order="F")
    bad = np.argwhere(got != want)
    assert bad.size == 0, (len(bad), bad[:6])


# --- AfterStepStatistics with CH AfterStep2D / Energy2D / Ff ---------------
# (bsamroutines.f90:763-775, :918-963; CH/problem.f90:149-183, :512-547,
# :901-915)

def seq_sum(a):
    """Fortran SUM in element order"""
    return np.cumsum(np.ravel(a, order="F"))[-1]


def energy2d(c, h, eps):
    mx, my = c.shape[0] - 2, c.shape[1] - 2
    h2 = h * h
    f1 = c[1:mx + 2, 1:my + 1] - c[0:mx + 1, 1:my + 1]   # f1(0:mx, 1:my)
    f1 = f1 * f1
    f2 = c[1:mx + 1, 1:my + 2] - c[1:mx + 1, 0:my + 1]   # f2(1:mx, 0:my)
    f2 = f2 * f2
    tmp = eps * eps / h2 / 4.0
    ci = c[1:mx + 1, 1:my + 1]
    c2 = ci * ci
    ff = c2 * (c2 - 2.0) / 4.0
    return h2 * (seq_sum(ff) + tmp * seq_sum(f1[1:mx + 1, :] + f1[0:mx, :] + f2[:, 1:my + 1] + f2[:, 0:my]))


def test_after_step_statistics_are_the_reference_statements(oracle_mod, pkg):
    from tests import hierarchies as H
    s = H.amr2d(periodic=True)
    eps = 0.01
    o = oracle_mod.OracleHierarchy(2, 2, "ch", [1e-3, eps])
    s.apply(o)
    q = {}
    for p in s.patches:
        v = pkg.initial.ch_spinodal(tuple(p["mx"][:2]), eps, p["dx"][0], seed=11 + p["id"])
        o.put(p["id"], "q", v)
        q[p["id"]] = o.get(p["id"], "q").reshape([m + 2 for m in p["mx"][:2]] + [2], order="F")[..., 0]
    byid = {p["id"]: p for p in s.patches}
    fin = s.finest()
    i1 = i2 = 0.0
    for level in range(fin, -1, -1):
        # ApplyOnLevel: youngest node first (the reverse of creation order)
        for p in reversed([x for x in s.patches if x["level"] == level]):
            h = p["dx"][0]
            h2, ch = h * h, h * 2.0
            ch2 = ch * ch
            c = q[p["id"]]
            if level == 0:
                i1 = i1 + h2 * seq_sum(c[1:-1, 1:-1])
                i2 = i2 + energy2d(c, h, eps)
            else:
                par = byid[p["parent_id"]]
                lo = [p["mbounds"][0], p["mbounds"][2]]
                hi = [p["mbounds"][1], p["mbounds"][3]]
                pc = q[par["id"]][lo[0] - 1:hi[0] + 2, lo[1] - 1:hi[1] + 2]  # parent%q(mb-1:mb+1)
                i1 = i1 + h2 * seq_sum(c[1:-1, 1:-1]) - ch2 * seq_sum(pc[1:-1, 1:-1])
                i2 = i2 + energy2d(c, h, eps) - energy2d(pc, ch, eps)
    got = o.after_step_stats(fin)
    assert (got[0], got[1]) == (i1, i2), (got, i1, i2)


def test_periodic_transfer_between_patches_is_the_reference_statements(oracle_mod):
    """Two children at opposite faces of a periodic root: Interpolate2D on
    both (their periodic faces included, CASE(2, 999)), then
    TransferPeriodicBC's GhostOverlap of the pair through every periodic
    offset of GetPeriodicOffsets (boundary.f90:582-605, :824-954) with
    both polarities; no quasi-periodic offset in these transfers."""
    from tests import hierarchies as H
    s = H.Spec(2)
    s.root_and_below(16, 0, [2, 2, 2, 2, 10, 10])
    s.child(0, 101, [1, 5], [4, 12])
    s.child(0, 102, [13, 9], [16, 16])
    o = oracle_mod.OracleHierarchy(2, 2, "ch", [CH["dt"], CH["eps"]])
    s.apply(o)
    rng = np.random.default_rng(123)
    q = {}
    for p in s.patches:
        a = rng.uniform(-1, 1, size=o.field_size(p["id"], "q"))
        o.put(p["id"], "q", a)
        q[p["id"]] = a.reshape([m + 2 for m in p["mx"][:2]] + [2], order="F")
    o.set_ghost(1, 0)
    want = {}
    for p in s.patches[1:]:
        mb = [(p["mbounds"][0], p["mbounds"][1]), (p["mbounds"][2], p["mbounds"][3])]
        want[p["id"]] = interpolate2d(q[p["id"]], q[0], p["mx"][:2], mb, p["mthbc"][:4], 0)
    mxmax = [32, 32]  # level 1 of a 16^2 root
    offsets = [(mxmax[0], 0), (0, mxmax[1]), (mxmax[0], mxmax[1]), (-mxmax[0], mxmax[1])]  # indices 1, 2, 4, 5
    a, b = s.patches[1], s.patches[2]
    mg = lambda p, o=(0, 0): [(p["mglobal"][0] + o[0], p["mglobal"][1] + o[0]),
                              (p["mglobal"][2] + o[1], p["mglobal"][3] + o[1])]
    for pol in (-1, 1):
        for off in offsets:
            ghost_overlap(want[101], want[102], mg(a), mg(b, (pol * off[0], pol * off[1])), 1, 2)
    for pid in (101, 102):
        assert np.array_equal(o.get(pid, "q").reshape(want[pid].shape, order="F"), want[pid]), pid


# --- NewSubGrids, GetSignatures, GridFlagRatio (bsamroutines.f90:1408-1662)

def new_sub_grids_ref(flags, desfill, mgp, maxsubgrids=1024, maxsplitpasses=15):
    """The Berger-Rigoutsos variant of NewSubGrids, statement by statement;
    flags[i-1, j-1(, k-1)] is errorflags(i, j(, k)); boxes 1-based"""
    nd = flags.ndim
    mx = flags.shape

    def box_sum(b):
        return int(flags[tuple(slice(b[d][0] - 1, b[d][1]) for d in range(nd))].sum())

    def ratio(b):
        total = 1.0
        for d in range(nd):
            total = total * float(b[d][1] - b[d][0] + 1)
        return float(box_sum(b)) / total

    maxm = max(mx)
    sig = np.zeros((maxm + 2, nd), dtype=np.int64)
    dds = np.zeros((maxm + 2, nd), dtype=np.int64)

    def signatures(b):
        for n in range(nd):
            for i in range(b[n][0], b[n][1] + 1):
                bb = [list(x) for x in b]
                bb[n] = [i, i]
                sig[i, n] = box_sum(bb)

    whole = [[1, mx[d]] for d in range(nd)]
    if ratio(whole) < 1.0e-10:
        return []
    ngrid = 1
    cansplit = [True] * (maxsubgrids + 2)
    msub = [None, [list(x) for x in whole]]
    igrid = 1
    while ngrid < maxsubgrids and igrid <= ngrid:
        npass = 0
        while cansplit[igrid] and npass < maxsplitpasses:
            npass += 1
            signatures(msub[igrid])
            for n in range(nd):  # trim unflagged edges, then whole coarse cells
                i1, i2 = msub[igrid][n]
                while sig[i1, n] == 0 and i1 < msub[igrid][n][1] and i2 - i1 + 1 > mgp:
                    i1 += 1
                while sig[i2, n] == 0 and i2 > msub[igrid][n][0] and i2 - i1 + 1 > mgp:
                    i2 -= 1
                msub[igrid][n] = [i1 - (i1 + 1) % 2, i2 + i2 % 2]
            if ratio(msub[igrid]) < desfill:
                signatures(msub[igrid])
                isplit, havesplit = [0, 0, 0], False
                for n in range(nd):  # a hole
                    i1, i2 = msub[igrid][n]
                    for i in range(i1 + mgp - 1, i2 - mgp + 1, 2):
                        if sig[i, n] == 0 and min(i - i1 + 1, i2 - i) >= mgp:
                            isplit[n], havesplit = i, True
                            break
                    if havesplit:
                        break
                if not havesplit:  # the strongest inflection
                    for n in range(nd):
                        i1, i2 = msub[igrid][n]
                        for i in range(i1 + 1, i2):
                            dds[i, n] = sig[i - 1, n] - 2 * sig[i, n] + sig[i + 1, n]
                    inflect = dist0 = 0
                    for n in range(nd):
                        i1, i2 = msub[igrid][n]
                        for i in range(i1 + mgp, i2 - mgp + 2, 2):
                            dl = abs(int(dds[i, n]) - int(dds[i - 1, n]))
                            if dl > inflect:
                                inflect, isplit, havesplit = dl, [0, 0, 0], True
                                isplit[n] = i - 1
                                dist0 = min(i - i1, i2 - i + 1)
                            elif dl == inflect and inflect > 0:
                                dist1 = min(i - i1, i2 - i + 1)
                                if dist1 > dist0:
                                    isplit, havesplit = [0, 0, 0], True
                                    isplit[n] = i - 1
                                    dist0 = dist1
                if havesplit:
                    for n in range(nd):
                        lo, hi = msub[igrid][n]
                        if isplit[n] > 0 and min(hi - isplit[n], isplit[n] - lo + 1) >= mgp:
                            ngrid += 1
                            cansplit[ngrid] = True
                            new = [list(x) for x in msub[igrid]]
                            new[n] = [isplit[n] + 1, hi]
                            msub.append(new)
                            msub[igrid][n] = [lo, isplit[n]]
                            break
                else:
                    cansplit[igrid] = False
            else:
                cansplit[igrid] = False
        igrid += 1
    return [[tuple(x) for x in msub[g]] for g in range(1, ngrid + 1)]


def random_flags(rng, shape):
    f = np.zeros(shape, dtype=np.int32)
    for _ in range(rng.integers(1, 5)):  # a few blobs and scattered points
        c = [rng.integers(0, n) for n in shape]
        r = [rng.integers(1, max(2, n // 3)) for n in shape]
        idx = np.indices(shape)
        inside = np.ones(shape, dtype=bool)
        for d in range(len(shape)):
            inside &= np.abs(idx[d] - c[d]) <= r[d]
        f[inside] = 1
    f[rng.random(shape) < rng.choice([0.0, 0.01, 0.05])] = 1
    return f


@pytest.mark.parametrize("nd", [2, 3])
def test_new_sub_grids_is_the_reference_algorithm(oracle_mod, nd):
    rng = np.random.default_rng(2000 + nd)
    cases = 120 if nd == 2 else 40
    for c in range(cases):
        shape = tuple(int(2 * rng.integers(4, 25 if nd == 2 else 9)) for _ in range(nd))
        flags = random_flags(rng, shape)
        desfill = float(rng.choice([0.5, 0.7, 0.8, 0.9]))
        mgp = int(rng.choice([4, 6, 8]))
        if min(shape) < mgp:
            continue
        want = new_sub_grids_ref(flags, desfill, mgp)
        got = oracle_mod.new_sub_grids(flags, desfill, mgp)
        assert got == want, (c, shape, desfill, mgp, got, want)
