"""The allocation-free norm entry point (bsamg_ch_residual_norm_noalloc).

It serves callers that cannot let the library call cudaMalloc -- hosts whose
device memory belongs to their own allocator, or serving loops that must not
trigger cudaMalloc's device-wide synchronisation.  The test hands it device
buffers owned by PyTorch's allocator and checks, on two calls in a row, that
it returns the same norm as the hierarchy's own ErrorAFAS entry point
(bsamg_residual_norm), to the 1e-12 relative tolerance of the parity tests.
This file is collected last so that a stop-at-first-failure run has already
run every other test.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DT, EPS = 1e-3, 0.01


@pytest.mark.parametrize("nd,n", [(2, 64), (3, 32)])
def test_noalloc_norm_matches_hierarchy_norm(pkg, ctx, nd, n):
    torch = pytest.importorskip("torch")
    minlevel = -int(np.log2(n)) + 1
    h = pkg.Hierarchy(ctx, nd, 2, "ch", [DT, EPS])
    h.build_uniform([n] * nd + [1] * (3 - nd), minlevel, [2] * (2 * nd) + [10] * (6 - 2 * nd), [0, 0, 0],
                    [1, 1, 1])
    h.commit()
    h.put(0, "q", pkg.initial.ch_spinodal((n,) * nd, EPS, 1.0 / n, seed=99))
    h.set_ghost(0, 0)
    rng = np.random.default_rng(4)
    h.put(0, "f", rng.uniform(-1, 1, size=h.field_size(0, "f")))
    for errortype in (1, 2):
        expect = h.residual_norm(0, errortype)
        q = torch.from_numpy(h.get(0, "q")).cuda()
        f = torch.from_numpy(h.get(0, "f")).cuda()
        out = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
        for call in range(2):
            out.fill_(float("nan"))
            torch.cuda.synchronize()
            pkg.api.ch_residual_norm_noalloc(q.data_ptr(), f.data_ptr(), nd, [n] * nd, 1.0 / n, DT, EPS,
                                              out.data_ptr(), errortype=errortype)
            torch.cuda.synchronize()
            got = float(out.item())
            assert abs(got - expect) <= 1e-12 * abs(expect), (call, errortype, got, expect)
    h.close()


def test_noalloc_rejects_patches_above_the_limit(pkg, ctx):
    limit = pkg.lib().bsamg_ch_residual_norm_noalloc
    import ctypes
    mx = (ctypes.c_int * 3)(512, 512, 128)  # 2^25 cells > BSAMG_NOALLOC_MAX_CELLS
    rc = limit(ctypes.c_void_p(16), ctypes.c_void_p(16), 3, mx, 1.0, 1.0, 1.0, 1, ctypes.c_void_p(16), None)
    assert rc == -1  # BSAMG_ERR_ARG, before anything is launched
    assert b"BSAMG_NOALLOC_MAX_CELLS" in pkg.lib().bsamg_last_error_detail()
