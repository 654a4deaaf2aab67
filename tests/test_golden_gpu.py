"""The CUDA library against the committed regression fixtures (needs a
GB300): one V-cycle bit for bit, one time step to 1e-12 relative with the
same V-cycle count (the step's norm is a parallel reduction)."""
import os

import numpy as np
import pytest

from tests.golden import make_golden as mg

pytestmark = pytest.mark.gpu
HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("name", sorted(mg.CASES))
def test_library_reproduces_the_fixture(pkg, ctx, name):
    z = np.load(os.path.join(HERE, name + ".npz"))
    nd, nv, prob, params, n, mn, mthbc = mg.CASES[name]
    g = pkg.Hierarchy(ctx, nd, nv, prob, params)
    g.build_uniform([n] * nd + [1] * (3 - nd), mn, mthbc, [0, 0, 0], [1, 1, 1])
    g.commit()
    for fld in ("q", "qold", "f"):
        g.put(0, fld, z[fld])
    g.set_ghost(0, 0)
    g.vcycle(0, mn, 2)
    assert np.array_equal(g.get(0, "q"), z["q_vcycle"])
    ncyc, res = g.time_step(False, 0, mn, tol=1e-10, maxvcycles=12)
    assert ncyc == int(z["ncycles"])
    np.testing.assert_allclose(res, z["residuals"], rtol=1e-10, atol=0)
    b = z["q_step"]
    assert np.max(np.abs(g.get(0, "q") - b)) <= 1e-12 * np.max(np.abs(b))
