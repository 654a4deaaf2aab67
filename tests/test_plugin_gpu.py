"""A plugin added without touching the library solves its problem on the
GPU (needs a GB300).  The test-only heat plugin (tests/plugins/heat.cu: one
implicit Euler step of two uncoupled heat equations) is linked into a build
of its own; on a periodic box its discrete solution is known in closed form
through the FFT, (1 + c dt/h^2 sum_d (2 - 2 cos theta_d)) u^ = u_old^, and
both the plain FP64 path and the mixed path converge to it."""
import pytest

from tests.plugin_build import run_with_heat

pytestmark = pytest.mark.gpu

SCRIPT = r"""
import numpy as np
import __graft_entry__ as ge
pkg = ge.load_package()
ctx = pkg.Context(0)
out = []
for nd, n in ((2, 64), (3, 32)):
    dt, kappa = 1e-3 if nd == 2 else 5e-3, 0.5
    minlevel = -int(np.log2(n)) + 1
    rng = np.random.default_rng(nd)
    u0 = rng.uniform(-1, 1, size=(n,) * nd + (2,))
    h = 1.0 / n
    th = [2 * np.pi * np.fft.fftfreq(n)] * nd
    lam = sum(np.meshgrid(*[2 - 2 * np.cos(t) for t in th], indexing="ij"))
    want = [np.real(np.fft.ifftn(np.fft.fftn(u0[..., v]) / (1 + c * dt / h**2 * lam)))
            for v, c in ((0, 1.0), (1, kappa))]
    for mode in ("fp64", "mixed"):
        g = pkg.Hierarchy(ctx, nd, 2, "heat", [dt, kappa])
        g.build_uniform([n] * nd + [1] * (3 - nd), minlevel, [2] * (2 * nd) + [10] * (6 - 2 * nd), [0, 0, 0],
                        [1, 1, 1])
        g.commit()
        q = np.zeros((n + 2,) * nd + (2,))
        q[(slice(1, -1),) * nd] = u0
        g.put(0, "q", np.asfortranarray(q))
        g.set_ghost(0, 0)
        g.copy_q_to_qold(minlevel, 0)
        nv, res = g.time_step(True, 0, minlevel, 2, 40, 1e-12, mode=mode, strict=True)
        got = g.get(0, "q").reshape((n + 2,) * nd + (2,), order="F")[(slice(1, -1),) * nd]
        err = max(float(np.max(np.abs(got[..., v] - want[v]))) for v in range(2))
        out.append((nd, mode, nv, res[-1], err))
        g.close()
ctx.close()
for r in out:
    print(*r)
"""


def test_heat_plugin_reaches_the_fft_solution():
    rows = [line.split() for line in run_with_heat(SCRIPT).strip().splitlines()]
    assert len(rows) == 4, rows
    for nd, mode, nv, res, err in rows:
        print(f"heat {nd}D {mode}: {nv} V-cycles, residual {float(res):.2e}, max error vs FFT {float(err):.2e}")
        assert float(res) < 1e-12
        assert float(err) < 1e-10, (nd, mode, err)
