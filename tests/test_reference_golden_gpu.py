"""The CUDA library against the reference itself (needs a GB300).

The fixtures tests/golden/ref_*.npz are the reference's own Fortran run on
these configurations (tests/golden/make_reference_golden.py).  The plain FP64
path runs the same steps through the C ABI (regrid before every step on the
adaptive cases): every node's q after every step must equal the reference's
bit for bit and the V-cycle counts must be the same; the residual norms are
a parallel sum here and the reference's sequential SUM there, so they agree
to 1e-12 relative.
"""
import numpy as np
import pytest

from tests.golden import make_reference_golden as G
from tests.test_reference_golden_cpu import FIXTURES, compare_frame, load, params_of

pytestmark = pytest.mark.gpu


def library_nodes(h, finest):
    out = []
    tab = h.patch_table()
    for level in range(finest + 1):
        for p in reversed([x for x in tab if x["level"] == level]):
            mg = np.array(p["mglobal"], dtype=np.int64).reshape(3, 2)
            out.append((p["level"], mg, h.get(p["id"], "q"), p["mx"]))
    return out


@pytest.mark.parametrize("name", FIXTURES)
def test_library_equals_the_reference(pkg, ctx, name):
    meta, frames = load(name)
    c = G.CASES[name]
    nd, n, L, mbc = c["nd"], c["n"], c["length"], c["mbc"]
    minlevel = -int(round(np.log2(n))) + 1
    prob, params = params_of(c)
    h = pkg.Hierarchy(ctx, nd, 2, prob, params, mbc=mbc)
    mthbc = [c["mthbc"]] * (2 * nd) + [10] * (6 - 2 * nd)
    h.build_uniform([n] * nd + [1] * (3 - nd), minlevel, mthbc, [0, 0, 0], [L] * nd + [1] * (3 - nd))
    h.commit()
    fn = G.qinit_fn(c)
    q0 = np.asarray(fn(0, [n] * nd, [L / n] * nd, [0.0] * nd))
    if mbc == 2:
        q2 = np.zeros((n + 4,) * nd + (2,), order="F")
        q2[(slice(2, -2),) * nd] = q0[(slice(1, -1),) * nd]
        q0 = q2
    h.put(0, "q", q0)
    h.set_ghost(0, 0)
    h.copy_q_to_qold(minlevel, 0)
    finest = 0
    for step in range(1, c["steps"] + 1):
        if c["maxlevel"] > 0:
            prm = pkg.regrid_params(c["maxlevel"], tagging="ch", initial=step == 1, qtolerance=c["qtol"],
                                    first_id=1000 * step)
            old = h
            h = h.regrid(prm, fn if step == 1 else None)
            old.close()
            finest = max(p["level"] for p in h.patch_table())
        nv, res = h.time_step(step == 1, finest, minlevel, 2, 20, c["tol"])
        ref_nodes, ref_res = frames[step]
        assert nv == len(ref_res), (name, step, nv, ref_res)
        np.testing.assert_allclose(res, ref_res, rtol=1e-12, atol=0)
        compare_frame(ref_nodes, library_nodes(h, finest), nd, 2, mbc, (name, "step", step))
    h.close()
