"""The allocation-free norm entry point (bsamg_ch_residual_norm_noalloc).

It serves callers that cannot let the library call cudaMalloc -- hosts whose
device memory belongs to their own allocator, or serving loops that must not
trigger cudaMalloc's device-wide synchronisation.  The test hands it device
buffers owned by PyTorch's allocator and checks, on two calls in a row, that
it returns exactly the norm of the hierarchy's own ErrorAFAS entry point
(bsamg_residual_norm): both use the same per-block partials and the same
final reduction.  The sizes cover one-stage final sums (2D 64^2, 3D 32^3),
the two-stage sum above 2048 blocks (3D 128^3) and a patch at the size limit
that fills the whole fixed scratch array (3D 256^3); one case runs on a
non-default stream.  This file is collected last so that a
stop-at-first-failure run has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DT, EPS = 1e-3, 0.01


def _check(pkg, ctx, nd, n, use_stream):
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
    q = torch.from_numpy(h.get(0, "q")).cuda()
    f = torch.from_numpy(h.get(0, "f")).cuda()
    out = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
    stream = torch.cuda.Stream() if use_stream else None
    for errortype in (1, 2):
        expect = h.residual_norm(0, errortype)
        for call in range(2):
            out.fill_(float("nan"))
            torch.cuda.synchronize()
            pkg.api.ch_residual_norm_noalloc(q.data_ptr(), f.data_ptr(), nd, [n] * nd, 1.0 / n, DT, EPS,
                                              out.data_ptr(), errortype=errortype,
                                              stream=stream.cuda_stream if stream is not None else None)
            torch.cuda.synchronize()
            got = float(out.item())
            assert got == expect, (nd, n, call, errortype, got, expect)
    h.close()


@pytest.mark.parametrize("nd,n,use_stream", [(2, 64, False), (3, 32, False), (3, 128, True), (3, 256, False)])
def test_noalloc_norm_equals_hierarchy_norm(pkg, ctx, nd, n, use_stream):
    _check(pkg, ctx, nd, n, use_stream)


def test_noalloc_rejects_patches_above_the_limit(pkg, ctx):
    limit = pkg.lib().bsamg_ch_residual_norm_noalloc
    mx = (ctypes.c_int * 3)(512, 512, 128)  # 2^25 cells > BSAMG_NOALLOC_MAX_CELLS
    rc = limit(ctypes.c_void_p(16), ctypes.c_void_p(16), 3, mx, 1.0, 1.0, 1.0, 1, ctypes.c_void_p(16), None)
    assert rc == -1  # BSAMG_ERR_ARG, before anything is launched
    assert b"BSAMG_NOALLOC_MAX_CELLS" in pkg.lib().bsamg_last_error_detail()
