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
