"""Error behaviour and ragged shapes through the C ABI (needs a GB300).

The library never aborts: every misuse the reference would STOP on, or that
the C ABI cannot honour, comes back as a negative status (BsamgError in the
Python mirror), and the context stays usable.  Ragged meshes -- extents that
are not powers of two, non-square roots, the smallest even patch -- run the
plain FP64 path bit for bit against the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bad_arguments_return_status_codes(pkg, ctx):
    E = pkg.BsamgError
    with pytest.raises(E):  # RootInit allows mbc = 1 or 2
        pkg.Hierarchy(ctx, 2, 2, "ch", [1e-3, 0.01], mbc=3)
    with pytest.raises(E):  # the growth plugin has three variables
        pkg.Hierarchy(ctx, 3, 2, "growth", [0.01, 0.025, 1.5, 2.0, 0.5, 1.0])
    with pytest.raises(E):  # BioGrowth needs five parameters
        pkg.Hierarchy(ctx, 2, 2, "biogrowth", [0.1, 0.05])
    h = pkg.Hierarchy(ctx, 2, 2, "ch", [1e-3, 0.01])
    with pytest.raises(E):  # odd extent
        h.build_uniform([15, 16, 1], -2, [2] * 6, [0, 0, 0], [1, 1, 1])
    h = pkg.Hierarchy(ctx, 2, 2, "ch", [1e-3, 0.01])
    h.build_uniform([16, 16, 1], -3, [2, 2, 2, 2, 10, 10], [0, 0, 0], [1, 1, 1])
    with pytest.raises(E):  # a patch whose parent does not exist
        h.add_patch(1, 77, 12345, [8, 8, 1], [1, 8, 1, 8, 1, 1], [1, 4, 1, 4, 1, 1], [999] * 4 + [10, 10],
                    [1 / 32, 1 / 32, 0], [0, 0, 0])
        h.commit()
    h = pkg.Hierarchy(ctx, 2, 2, "ch", [1e-3, 0.01])
    h.build_uniform([16, 16, 1], -3, [2, 2, 2, 2, 10, 10], [0, 0, 0], [1, 1, 1])
    h.commit()
    with pytest.raises(E):  # no patch may be added after commit
        h.add_patch(1, 5, 0, [8, 8, 1], [1, 8, 1, 8, 1, 1], [1, 4, 1, 4, 1, 1], [999] * 4 + [10, 10],
                    [1 / 32, 1 / 32, 0], [0, 0, 0])
    with pytest.raises(E):  # wrong array size
        h.put(0, "q", np.zeros(10))
    with pytest.raises(E):  # unknown patch id
        h.get(99, "q")
    with pytest.raises(E):  # finest above the hierarchy
        h.time_step(True, 1, -3)
    with pytest.raises(E):  # minlevel below the hierarchy
        h.time_step(True, 0, -5)
    with pytest.raises(E):  # nsmooth must be positive
        h.multigrid_iterations(0, -3, nsmooth=0)
    with pytest.raises(E):  # errortype 1 or 2
        h.multigrid_iterations(0, -3, errortype=3)
    # the hierarchy and the context still work after the errors
    h.put(0, "q", pkg.initial.ch_spinodal((16, 16), 0.01, 1 / 16, seed=1))
    n, res = h.time_step(True, 0, -3, tol=1e-9, maxvcycles=30)
    assert res[-1] < 1e-9


def test_nonconvergence_is_reported_only_when_asked(pkg, ctx):
    h = pkg.Hierarchy(ctx, 2, 2, "ch", [1e-3, 0.01])
    h.build_uniform([32, 32, 1], -4, [2, 2, 2, 2, 10, 10], [0, 0, 0], [1, 1, 1])
    h.commit()
    h.put(0, "q", pkg.initial.ch_spinodal((32, 32), 0.01, 1 / 32, seed=2))
    n, res = h.time_step(True, 0, -4, tol=1e-30, maxvcycles=2)  # silent stop, as the reference
    assert n == 2 and len(res) == 2
    with pytest.raises(pkg.BsamgError) as ei:
        h.time_step(False, 0, -4, tol=1e-30, maxvcycles=2, strict=True)
    assert ei.value.status == -4  # BSAMG_ERR_NOT_CONVERGED


@pytest.mark.parametrize("nd,mx,length,minlevel", [(2, [6, 10], [0.6, 1.0], -1), (2, [2, 2], [1, 1], 0),
                                                  (3, [6, 4, 10], [0.6, 0.4, 1.0], -1), (3, [2, 2, 2], [1, 1, 1], 0)])
@pytest.mark.parametrize("mthbc", ["periodic", "physical"])
def test_ragged_roots_match_the_oracle(pkg, ctx, oracle_mod, nd, mx, length, minlevel, mthbc):
    th = ([2] * (2 * nd) + [10] * (6 - 2 * nd)) if mthbc == "periodic" else [10] * 6
    cfg = (2e-4, 0.02)
    g = pkg.Hierarchy(ctx, nd, 2, "ch", list(cfg))
    o = oracle_mod.OracleHierarchy(nd, 2, "ch", list(cfg))
    full = mx + [1] * (3 - nd)
    up = length + [1] * (3 - nd)
    for h in (g, o):
        h.build_uniform(full, minlevel, th, [0, 0, 0], up)
        h.commit()
    q = pkg.initial.ch_spinodal(tuple(mx), cfg[1], length[0] / mx[0], seed=7, amp=0.1)
    g.put(0, "q", q)
    o.put(0, "q", q)
    for step in range(2):
        ng, rg = g.time_step(step == 0, 0, minlevel, tol=1e-11, maxvcycles=25)
        no, ro = o.time_step(step == 0, 0, minlevel, tol=1e-11, maxvcycles=25)
        assert ng == no
        np.testing.assert_allclose(rg, ro, rtol=1e-10, atol=1e-300)
    a, b = g.get(0, "q"), o.get(0, "q")
    assert np.max(np.abs(a - b)) <= 1e-12 * max(np.max(np.abs(b)), 1e-300)
