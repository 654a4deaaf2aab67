"""Known-answer tests that pin the CPU oracle (no GPU).

The reference ships no tests or golden vectors, so the oracle is pinned by
properties that follow from the mathematics of the reference's routines.
"""
import numpy as np
import pytest

from tests import hierarchies as H

EPS, DT = 0.01, 1e-3


def _ch(oracle_mod, nd=2):
    return oracle_mod.OracleHierarchy(nd, 2, "ch", [DT, EPS])


def test_splitmix_known_answer(oracle_mod):
    # splitmix64 seeded with 0: first output 0xE220A8397B1DCDAF (published
    # reference sequence of the generator)
    u = 0xE220A8397B1DCDAF
    expect = 2.0 * ((u >> 11) * 2.0 ** -53) - 1.0
    assert oracle_mod.uniform_pm1(0, 0) == expect


def test_splitmix_matches_numpy_generator(oracle_mod, pkg):
    g = np.arange(0, 5000, 7, dtype=np.uint64)
    a = pkg.initial.splitmix_pm1(1234, g)
    b = np.array([oracle_mod.uniform_pm1(1234, int(x)) for x in g])
    assert np.array_equal(a, b)


def test_uniform_builder_matches_rootinit_initseed(oracle_mod):
    h = _ch(oracle_mod)
    H.uniform(h, 2, 64, -5, [2, 2, 2, 2, 10, 10])
    h.commit()
    t = {p["level"]: p for p in h.patch_table()}
    assert sorted(t) == [-5, -4, -3, -2, -1, 0]
    for l in range(-5, 1):
        m = 64 >> (-l)
        assert t[l]["mx"][:2] == [m, m]
        assert t[l]["mglobal"][:4] == [1, m, 1, m]
        # InitSeed resets the child's mbounds to (1, mx/2); the coarsest keeps (1, mx)
        hi = m // 2 if l > -5 else m
        assert t[l]["mbounds"][:4] == [1, hi, 1, hi]
        assert t[l]["dx"][0] == pytest.approx(1.0 / m)
        assert t[l]["parent_id"] == (-l + 1 if l > -5 else -1)


def _fill_linear(h, spec, fn):
    """q on every patch = fn(x, y) at cell centres, ghosts included."""
    for p in spec.patches:
        mx, dx, xl = p["mx"], p["dx"], p["xlower"]
        i = np.arange(0, mx[0] + 2)
        j = np.arange(0, mx[1] + 2)
        X = xl[0] + (i - 0.5) * dx[0]
        Y = xl[1] + (j - 0.5) * dx[1]
        XX, YY = np.meshgrid(X, Y, indexing="ij")
        q = np.stack([fn(XX, YY), 2.0 * fn(XX, YY) + 1.0], axis=-1)
        h.put(p["id"], "q", q)


def test_cf_interpolation_exact_for_linear_fields(oracle_mod):
    # Interpolate2D (boundary.f90:143-333) is quadratic along the lines it
    # uses, so a linear field is reproduced exactly in every C/F ghost cell;
    # the a-, b- and c-weights each sum to 1.
    spec = H.amr2d(periodic=False)
    h = _ch(oracle_mod)
    spec.apply(h)
    fn = lambda x, y: 0.3 + 1.7 * x - 0.9 * y
    _fill_linear(h, spec, fn)
    for level in (1, 2):
        for ipass in (0, 1, 2):
            h.set_ghost(level, ipass)
    for p in spec.patches:
        if p["level"] < 1:
            continue
        mx, dx, xl = p["mx"], p["dx"], p["xlower"]
        q = h.get(p["id"], "q").reshape(mx[0] + 2, mx[1] + 2, 2, order="F")
        i = np.arange(0, mx[0] + 2)
        j = np.arange(0, mx[1] + 2)
        XX, YY = np.meshgrid(xl[0] + (i - 0.5) * dx[0], xl[1] + (j - 0.5) * dx[1], indexing="ij")
        ghost = np.ones_like(XX, dtype=bool)
        ghost[1:-1, 1:-1] = False
        # faces with a physical BC are reflected, not interpolated: skip them
        for face, sl in ((0, (0, slice(None))), (1, (-1, slice(None))), (2, (slice(None), 0)),
                         (3, (slice(None), -1))):
            if p["mthbc"][face] == 10:
                ghost[sl] = False
        exp = fn(XX, YY)
        assert np.allclose(q[..., 0][ghost], exp[ghost], rtol=0, atol=1e-13)
        assert np.allclose(q[..., 1][ghost], 2.0 * exp[ghost] + 1.0, rtol=0, atol=1e-13)


def test_cf_interpolation_3d_exact_for_linear_fields(oracle_mod):
    # Interpolate3D (boundary.f90:1048-1550): every ghost cell, its two fine
    # cells and its parent value lie on one line, and the a-, b- and
    # c-weights are exact for linear data, so a linear field is reproduced
    # in every interpolated ghost cell (corners, edges, faces, grey cells).
    for periodic in (False, True):
        spec = H.amr3d(periodic=periodic)
        h = _ch(oracle_mod, 3)
        spec.apply(h)
        fn = lambda x, y, z: 0.3 + 1.7 * x - 0.9 * y + 0.6 * z
        for p in spec.patches:
            h.put(p["id"], "q", _linear3(p, fn))
        for level in (1, 2):
            for ipass in (0, 1, 2):
                h.set_ghost(level, ipass)
        checked = 0
        for p in spec.patches:
            if p["level"] < 1:
                continue
            mx = p["mx"]
            q = h.get(p["id"], "q").reshape(mx[0] + 2, mx[1] + 2, mx[2] + 2, 2, order="F")
            exp = _linear3(p, fn)
            ghost = np.ones(q.shape[:3], dtype=bool)
            ghost[1:-1, 1:-1, 1:-1] = False
            # faces with a physical BC are reflected, not interpolated; with
            # periodic roots the images of other patches land in the ring too,
            # and those agree with a linear field only up to the period shift
            for d in range(3):
                for side, idx in ((0, 0), (1, -1)):
                    if p["mthbc"][2 * d + side] != 999:
                        sl = [slice(None)] * 3
                        sl[d] = idx
                        ghost[tuple(sl)] = False
            assert np.allclose(q[..., 0][ghost], exp[..., 0][ghost], rtol=0, atol=1e-13)
            assert np.allclose(q[..., 1][ghost], exp[..., 1][ghost], rtol=0, atol=1e-13)
            checked += int(ghost.sum())
        assert checked > 1000


def _linear3(p, fn):
    mx, dx, xl = p["mx"], p["dx"], p["xlower"]
    ax = [xl[d] + (np.arange(0, mx[d] + 2) - 0.5) * dx[d] for d in range(3)]
    X, Y, Z = np.meshgrid(*ax, indexing="ij")
    return np.stack([fn(X, Y, Z), 2.0 * fn(X, Y, Z) + 1.0], axis=-1)


def test_restriction_of_linear_is_cell_average(oracle_mod):
    spec = H.Spec(2)
    spec.root_and_below(16, -2, [10, 10, 10, 10, 10, 10])
    h = _ch(oracle_mod)
    spec.apply(h)
    fn = lambda x, y: 2.0 + x + 3.0 * y
    _fill_linear(h, spec, fn)
    h.fill_down("q", 0, -2)
    for p in spec.patches:
        mx, dx = p["mx"], p["dx"]
        q = h.get(p["id"], "q").reshape(mx[0] + 2, mx[1] + 2, 2, order="F")[1:-1, 1:-1, 0]
        c = (np.arange(1, mx[0] + 1) - 0.5) * dx[0]
        XX, YY = np.meshgrid(c, c, indexing="ij")
        assert np.allclose(q, fn(XX, YY), rtol=0, atol=1e-13)


def _spinodal(pkg, h, n, minlevel, seed=3, nd=2):
    q = pkg.initial.ch_spinodal((n,) * nd, EPS, 1.0 / n, seed=seed)
    h.put(0, "q", q)
    h.set_ghost(0, 0)
    h.copy_q_to_qold(minlevel, 0)
    return q


def test_vcycle_residual_decreases_and_converges(oracle_mod, pkg):
    h = _ch(oracle_mod)
    H.uniform(h, 2, 64, -5, [2, 2, 2, 2, 10, 10])
    h.commit()
    _spinodal(pkg, h, 64, -5)
    n, res = h.time_step(True, 0, -5, tol=1e-11, maxvcycles=20)
    assert n < 20 and res[-1] < 1e-11
    assert all(b < 0.5 * a for a, b in zip(res, res[1:]))


def test_ch_mass_conserved_with_periodic_bc(oracle_mod, pkg):
    # Operator2D row 1 is phi - dt/h^2 ULap(mu) = phi_old (CH/problem.f90:415,
    # :444): with periodic ghosts the Laplacian sums to zero, so
    # sum(phi) - sum(phi_old) = -sum(rf_1), bounded by the final residual.
    n = 64
    h = _ch(oracle_mod)
    H.uniform(h, 2, n, -5, [2, 2, 2, 2, 10, 10])
    h.commit()
    q0 = _spinodal(pkg, h, n, -5)
    for step in range(3):
        nc, res = h.time_step(step == 0, 0, -5, tol=1e-12, maxvcycles=30)
    q = h.get(0, "q").reshape(n + 2, n + 2, 2, order="F")
    m0 = q0[1:-1, 1:-1, 0].sum()
    m1 = q[1:-1, 1:-1, 0].sum()
    assert abs(m1 - m0) < n * n * 1e-11


def _energy(phi, h):
    # Energy2D, CH/problem.f90:512-547, on a periodic grid
    f1 = (np.roll(phi, -1, 0) - phi) ** 2
    f2 = (np.roll(phi, -1, 1) - phi) ** 2
    ff = phi ** 2 * (phi ** 2 - 2.0) / 4.0
    return h * h * (ff.sum() + EPS ** 2 / h ** 2 / 4.0 * (2 * f1.sum() + 2 * f2.sum()))


def test_ch_energy_decreases(oracle_mod, pkg):
    n = 64
    h = _ch(oracle_mod)
    H.uniform(h, 2, n, -5, [2, 2, 2, 2, 10, 10])
    h.commit()
    q0 = _spinodal(pkg, h, n, -5)
    es = [_energy(q0[1:-1, 1:-1, 0], 1.0 / n)]
    for step in range(4):
        h.time_step(step == 0, 0, -5, tol=1e-12, maxvcycles=30)
        q = h.get(0, "q").reshape(n + 2, n + 2, 2, order="F")
        es.append(_energy(q[1:-1, 1:-1, 0], 1.0 / n))
    assert all(b <= a + 1e-12 for a, b in zip(es, es[1:]))


def test_biogrowth_runs_and_converges(oracle_mod, pkg):
    n = 32
    h = oracle_mod.OracleHierarchy(2, 2, "biogrowth", [0.1, 0.05, 1.5, 2.0, 0.5])
    H.uniform(h, 2, n, -4, [10, 10, 10, 10, 10, 10], length=6.4)
    h.commit()
    q = np.zeros((n + 2, n + 2, 2), order="F")
    x = (np.arange(n) + 0.5) * 6.4 / n
    XX, YY = np.meshgrid(x, x, indexing="ij")
    q[1:-1, 1:-1, 0] = np.where((XX > 2.6) & (XX < 3.8) & (YY > 3.0) & (YY < 3.4), 1.0, -1.0)
    q[1:-1, 1:-1, 1] = 1.0
    h.put(0, "q", q)
    h.set_ghost(0, 0)
    h.copy_q_to_qold(-4, 0)
    nc, res = h.time_step(True, 0, -4, tol=1e-9, maxvcycles=20)
    assert res[-1] < 1e-9 and nc < 20


def test_amr_hierarchy_converges(oracle_mod, pkg):
    spec = H.amr2d(periodic=True)
    h = _ch(oracle_mod)
    spec.apply(h)
    rng = np.random.default_rng(5)
    for p in spec.patches:
        mx = p["mx"]
        q = np.zeros((mx[0] + 2, mx[1] + 2, 2), order="F")
        q[1:-1, 1:-1, 0] = 0.05 * rng.uniform(-1, 1, size=(mx[0], mx[1]))
        h.put(p["id"], "q", q)
    nc, res = h.time_step(True, spec.finest(), spec.minlevel(), tol=1e-9, maxvcycles=30)
    assert res[-1] < res[0] * 1e-3
