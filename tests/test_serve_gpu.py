"""Serving loop (continuous batching over independent CH requests) on a
GB300: results are the same alone and in a concurrent mix, and admission
waits for memory instead of failing when the HBM budget is tight."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _requests(serve, mode):
    R = serve.Request
    return [R(0, 2, 64, 2, 3, 0.012, 2.5e-4 * 4, seed=11, mode=mode),
            R(1, 2, 32, 0, 4, 0.02, 1e-3 * 16, seed=12, mode=mode),
            R(2, 3, 32, 0, 2, 0.025, 5e-4 * 64, seed=13, mode=mode),
            R(3, 2, 128, 1, 2, 0.015, 1e-3, seed=14, mode=mode),
            R(4, 2, 64, 3, 2, 0.03, 2.5e-4 * 4, seed=15, mode=mode),
            R(5, 3, 64, 0, 2, 0.01, 5e-4 * 16, seed=16, mode=mode),
            R(6, 3, 32, 2, 2, 0.02, 5e-4, seed=17, mode=mode)]


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_same_result_alone_and_in_the_mix(pkg, mode):
    serve = pkg.serve
    alone = _requests(serve, mode)
    ctx = pkg.Context(0)
    srv = serve.Server(ctx, slots=1)
    for r in alone:
        srv.run_request(r)
        assert r.error is None and r.result is not None
    srv.close()
    ctx.close()
    # the mix: seven requests, three slots, all submitted at once, and a budget
    # below their sum (the 64^3 request alone takes about 31 MB) so that
    # admission has to wait for memory
    mixed = _requests(serve, mode)
    ctx = pkg.Context(0, hbm_budget=36 * 2**20)
    stats = {}
    done, wall = serve.serve(ctx, mixed, slots=3, stats=stats)
    ctx.close()
    print(f"{mode}: mix of {len(done)} requests in {wall:.3f} s, {stats['admission_waits']} admission waits")
    assert all(r.error is None for r in done), [r.error for r in done]
    for a, b in zip(alone, mixed):
        assert a.vcycles == b.vcycles
        for pid in a.result:
            assert np.array_equal(a.result[pid], b.result[pid]), (a.rid, pid)


def test_request_larger_than_the_budget_fails_cleanly(pkg):
    serve = pkg.serve
    ctx = pkg.Context(0, hbm_budget=1 * 2**20)
    r = serve.Request(0, 3, 64, 0, 1, 0.02, 5e-4 * 16, seed=1)
    done, _ = serve.serve(ctx, [r], slots=1)
    ctx.close()
    assert done[0].error is not None and "budget" in done[0].error


@pytest.mark.parametrize("nd,n,levels", [(2, 64, 2), (3, 32, 1)])
def test_device_seeded_start_equals_the_host_generator(pkg, ctx, nd, n, levels):
    """bsamg_seed_spinodal (the serving loop's initial data) forms the same
    doubles as initial.ch_spinodal: splitmix64 per cell, the wrapped
    Laplacian and mu in the same operation order."""
    pats, _ = pkg.serve.nested_spec(nd, n, levels)
    h = pkg.Hierarchy(ctx, nd, 2, "ch", [1e-3, 0.017])
    for p in pats:
        h.add_patch(p["level"], p["id"], p["parent_id"], p["mx"], p["mglobal"], p["mbounds"], p["mthbc"], p["dx"],
                    p["xlower"])
    h.commit()
    for p in pats:
        if p["level"] < 0:
            continue
        h.seed_spinodal(p["id"], 99 + p["id"], mean=0.1, amp=0.05)
        want = pkg.initial.ch_spinodal(tuple(p["mx"][:nd]), 0.017, p["dx"][0], seed=99 + p["id"], mean=0.1)
        got = h.get(p["id"], "q").reshape(want.shape, order="F")
        assert np.array_equal(got, want), (p["id"], np.max(np.abs(got - want)))


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
@pytest.mark.parametrize("shape", [(2, 64, 2), (2, 32, 0), (3, 32, 1)])
def test_reused_hierarchy_gives_the_fresh_result(pkg, mode, shape):
    """A request served by an idle hierarchy left by another request of the
    same shape (other eps, dt and seed: bsamg_set_params + bsamg_hier_reset)
    gives bit for bit what it gives on a newly built hierarchy."""
    serve = pkg.serve
    nd, n, lv = shape

    def pair():
        return (serve.Request(0, nd, n, lv, 3, 0.021, 1e-3, seed=31, mode=mode),
                serve.Request(1, nd, n, lv, 2, 0.013, 5e-4, seed=32, mode=mode))
    ctx = pkg.Context(0)
    fresh = serve.Server(ctx, slots=1, reuse=False)
    _, b0 = pair()
    fresh.run_request(b0)
    fresh.close()
    srv = serve.Server(ctx, slots=1, reuse=True)
    a1, b1 = pair()
    srv.run_request(a1)
    srv.run_request(b1)
    assert srv.reused == 1
    srv.close()
    ctx.close()
    assert b0.error is None and b1.error is None
    assert b0.vcycles == b1.vcycles
    for pid in b0.result:
        assert np.array_equal(b0.result[pid], b1.result[pid]), pid
