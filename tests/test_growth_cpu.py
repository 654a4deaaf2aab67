"""Known answers for the three-variable growth plugin in the oracle (no GPU).

The plugin has no reference counterpart; its equations (phi and n as
BioGrowth's with 2*ndims neighbours, p from -Lap(p)/h^2 = cpress*phi*n) are
pinned by exact solutions.  With phi = -1 everywhere the growth and uptake
rates vanish, so phi = -1 and n = 1 are exact discrete solutions, and p
must equal the direct solution of the discrete Poisson problem with p = 0 on
the faces.
"""
import numpy as np

PARAMS = [0.01, 0.025, 1.5, 2.0, 0.5, 1.0]  # dt, eps, gamma, lambda, czero, cpress


def test_uniform_states_and_pressure_poisson(oracle_mod):
    nd, n = 3, 8
    o = oracle_mod.OracleHierarchy(nd, 3, "growth", PARAMS)
    o.build_uniform([n, n, n], -2, [10] * 6, [0, 0, 0], [1, 1, 1])
    o.commit()
    q = np.zeros((n + 2, n + 2, n + 2, 3), order="F")
    q[..., 0] = -1.0
    q[..., 1] = 1.0
    o.put(0, "q", q)
    nc, res = o.time_step(True, 0, -2, tol=1e-13, maxvcycles=60)
    assert res[-1] < 1e-13
    out = o.get(0, "q").reshape(n + 2, n + 2, n + 2, 3, order="F")[1:-1, 1:-1, 1:-1]
    assert np.array_equal(out[..., 0], np.full((n, n, n), -1.0))
    assert np.array_equal(out[..., 1], np.full((n, n, n), 1.0))
    # -(1/h^2) Lap_h p = cpress * phi * n = -cpress, ghost p = -p (p = 0 on faces)
    h = 1.0 / n
    N = n ** 3
    A = np.zeros((N, N))
    idx = lambda i, j, k: (k * n + j) * n + i
    for k in range(n):
        for j in range(n):
            for i in range(n):
                r = idx(i, j, k)
                A[r, r] = 6.0
                for d in range(3):
                    for s in (-1, 1):
                        c = [i, j, k]
                        c[d] += s
                        if 0 <= c[d] < n:
                            A[r, idx(*c)] -= 1.0
                        else:
                            A[r, r] += 1.0  # ghost = -p
    b = np.full(N, -PARAMS[5] * h * h)
    p = np.linalg.solve(A, b)
    got = out[..., 2].ravel(order="F")
    assert np.allclose(got, p, rtol=0, atol=1e-10), np.max(np.abs(got - p))


def test_seeded_sphere_converges_2d_and_3d(oracle_mod, pkg):
    for nd, n, ml in ((2, 32, -4), (3, 16, -3)):
        o = oracle_mod.OracleHierarchy(nd, 3, "growth", PARAMS)
        mx = [n] * nd + [1] * (3 - nd)
        o.build_uniform(mx, ml, [10] * 6, [0, 0, 0], [1, 1, 1])
        o.commit()
        fn = pkg.initial.growth_sphere(PARAMS[1], seed=3)
        o.put(0, "q", fn(0, [n] * nd, [1.0 / n] * nd, [0.0] * nd))
        for step in range(2):
            nc, res = o.time_step(step == 0, 0, ml, tol=1e-9, maxvcycles=40)
            assert res[-1] < 1e-9 and nc < 40, (nd, step, nc, res)
            assert all(b <= a * 1.0001 for a, b in zip(res, res[1:]))
