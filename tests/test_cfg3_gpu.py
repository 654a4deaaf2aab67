"""The headline configuration, 3D Cahn-Hilliard 256^3 periodic (eps = 0.02,
dt = 5e-4, V(2,2), levels 256^3 .. 2^3, spinodal start phi0 = 0.1 +
0.05 U(-1,1)), pinned against the CPU oracle (needs a GB300).

* The plain FP64 path after a fixed number of V-cycles of the first time
  step (MultigridIterations, afasroutines.f90:48-110, stopped at maxvcycles)
  equals the oracle bit for bit: every operation of a V-cycle is evaluated in
  the reference's order, and the residual norms, whose parallel sum is the
  only reordered arithmetic, do not feed back into the fields.
* The mixed path's error against the FP64 oracle is a tested number: after
  time steps at the configuration's tolerance on a 128^3 box.
* The periodic-box path's exit test uses a double-float residual; on the
  same iterate it agrees with the FP64 ErrorAFAS (bsamg_residual_norm) to
  1e-12 absolute (the residual is ~1e-8 at convergence, its terms are up to
  ~30, and double-float carries ~2^-47 of each term).
"""
import numpy as np
import pytest

from tests.test_parity_gpu import CH3, PERIODIC3, make_pair, uniform_spec

pytestmark = pytest.mark.gpu

EPS, DT, SEED = 0.02, 5e-4, 20240503


def _start(pkg, n):
    return pkg.initial.ch_spinodal((n, n, n), EPS, 1.0 / n, seed=SEED, mean=0.1, amp=0.05)


def test_ch3d_256_two_fp64_vcycles_equal_the_oracle(pkg, ctx, oracle_mod):
    n, minlevel = 256, -7
    spec = uniform_spec(3, n, PERIODIC3)
    g, o = make_pair(pkg, ctx, oracle_mod, CH3, spec)
    q0 = _start(pkg, n)
    for h in (g, o):
        h.put(0, "q", q0)
        h.set_ghost(0, 0)
        h.copy_q_to_qold(minlevel, 0)
    ng, rg = g.time_step(True, 0, minlevel, 2, 2, 1e-8)
    no, ro = o.time_step(True, 0, minlevel, 2, 2, 1e-8)
    assert ng == no == 2, (ng, no)
    np.testing.assert_allclose(rg, ro, rtol=1e-12, atol=0)
    a, b = g.get(0, "q"), o.get(0, "q")
    diff = np.flatnonzero(a != b)
    rel = float(np.max(np.abs(a - b)) / np.max(np.abs(b)))
    print(f"256^3, 2 FP64 V-cycles: residuals {rg} (oracle {ro}); max rel diff {rel:.3e}, "
          f"{diff.size} values differ")
    assert diff.size == 0, (diff[:5], a[diff[:5]], b[diff[:5]])
    for fld in ("qc", "f", "rf"):
        assert np.array_equal(g.get(0, fld), o.get(0, fld)), fld
    g.close()


# the error the mixed path delivers at the configuration's tolerance (1e-8)
# after five steps on the 128^3 box, against the FP64 oracle: 3.0e-9
# measured on a GB300 (V-cycles 8, 5, 5, 5, 5 in both paths), asserted with
# a margin of about three
MIXED_128_BOUND = 1e-8


def test_ch3d_128_mixed_error_vs_oracle(pkg, ctx, oracle_mod):
    n, minlevel, steps, tol = 128, -6, 5, 1e-8
    spec = uniform_spec(3, n, PERIODIC3)
    g, o = make_pair(pkg, ctx, oracle_mod, CH3, spec)
    q0 = _start(pkg, n)
    for h in (g, o):
        h.put(0, "q", q0)
        h.set_ghost(0, 0)
        h.copy_q_to_qold(minlevel, 0)
    vg, vo = [], []
    for s in range(steps):
        ng, rg = g.time_step(s == 0, 0, minlevel, 2, 30, tol, mode="mixed", strict=True)
        no, ro = o.time_step(s == 0, 0, minlevel, 2, 30, tol)
        assert rg[-1] < tol and ro[-1] < tol, (s, rg, ro)
        vg.append(ng)
        vo.append(no)
    a, b = g.get(0, "q"), o.get(0, "q")
    k = a.size // 2
    err = float(np.max(np.abs(a[:k] - b[:k])) / np.max(np.abs(b[:k])))
    print(f"128^3 mixed vs FP64 oracle after {steps} steps at tol {tol:g}: max rel error of phi {err:.3e}; "
          f"V-cycles mixed {vg}, FP64 {vo}")
    assert err <= MIXED_128_BOUND, err
    assert all(x <= y + 2 for x, y in zip(vg, vo)), (vg, vo)
    g.close()


def _fp64_norm_of(pkg, h, n):
    """ErrorAFAS of the hierarchy's current q in FP64 (bsamg_residual_norm),
    with f = the CH source of qold (CH/problem.f90:672-721: f1 = phi_old,
    f2 = -phi_old), the f the step solved for."""
    qold = h.get(0, "qold").reshape((n + 2, n + 2, n + 2, 2), order="F")
    phi = np.asfortranarray(qold[1:-1, 1:-1, 1:-1, 0])
    f = np.stack([phi, -phi], axis=-1)
    h.put(0, "f", np.asfortranarray(f))
    return h.residual_norm(0, 1)


@pytest.mark.parametrize("n", [64, 128])
def test_box_double_float_residual_equals_fp64_norm(pkg, ctx, n):
    minlevel = -int(np.log2(n)) + 1
    h = pkg.Hierarchy(ctx, 3, 2, "ch", [DT, EPS])
    h.build_uniform([n] * 3, minlevel, PERIODIC3, [0, 0, 0], [1, 1, 1])
    h.commit()
    h.seed_spinodal(0, SEED, mean=0.1, amp=0.05)
    # one V-cycle: the true residual of the iterate is far from converged
    n1, r1 = h.time_step(True, 0, minlevel, 2, 1, 1e-8, mode="mixed", strict=False)
    f1 = _fp64_norm_of(pkg, h, n)
    # then a step to the configuration's tolerance
    n2, r2 = h.time_step(False, 0, minlevel, 2, 30, 1e-8, mode="mixed", strict=True)
    f2 = _fp64_norm_of(pkg, h, n)
    print(f"{n}^3: double-float {r1[-1]:.15e} vs FP64 {f1:.15e}; converged {r2[-1]:.15e} vs {f2:.15e}")
    # unconverged, the two evaluations of a difference of O(1/h^2) terms
    # agree to 0.5-1.1e-9 relative depending on the iterate's FP32 roundings
    assert abs(r1[-1] - f1) <= max(1e-12, 3e-9 * f1), (r1, f1)
    assert abs(r2[-1] - f2) <= 1e-12, (r2, f2)
    assert f2 < 1e-8
    h.close()


def test_ch3d_256_one_pass_smoothing_equals_the_sweeps(pkg, ctx):
    """At the headline size the one-pass V(2,2) smoothing of the 256^3 level
    (the default) and the four-row colour sweeps give the same mixed time
    steps bit for bit: iterates and residual histories."""
    out = {}
    for kind in (1, 3):
        h = pkg.Hierarchy(ctx, 3, 2, "ch", [DT, EPS])
        h.build_uniform([256] * 3, -7, PERIODIC3, [0, 0, 0], [1, 1, 1])
        h.commit()
        h.set_box_sweep(kind)
        assert h.smoother_colours(0, "mixed") == (4 if kind == 3 else 1)
        h.seed_spinodal(0, SEED, mean=0.1, amp=0.05)
        hist = [h.time_step(s == 0, 0, -7, 2, 30, 1e-8, mode="mixed", strict=True) for s in range(2)]
        out[kind] = (hist, h.get(0, "q"))
        h.close()
    assert out[1][0] == out[3][0]
    assert np.array_equal(out[1][1], out[3][1])
