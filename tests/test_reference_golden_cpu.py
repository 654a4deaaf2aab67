"""The oracle against the reference itself (no GPU).

tests/golden/ref_*.npz hold what the BSAM 1.2 reference's own Fortran
source computes (run by oracle/fortran_exec.py; see
tests/golden/make_reference_golden.py): every node's q after the initial
regrid and after every time step, and the residual history of every
MultigridIterations, for 2D and 3D CH (periodic, Neumann, Dirichlet, two
ghost layers), 2D BioGrowth, and 2D and 3D CH on adaptive meshes regridded
before every step (the reference's CH tagging, Berger-Rigoutsos clustering
and InitFields).  The oracle runs the same configuration through its own
entry points; meshes, fields and residuals must be identical bit for bit.
"""
import glob
import json
import os

import numpy as np
import pytest

from tests.golden import make_reference_golden as G

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIXTURES = sorted(os.path.basename(p)[4:-4] for p in glob.glob(os.path.join(HERE, "ref_*.npz")))


def load(name):
    d = np.load(os.path.join(HERE, f"ref_{name}.npz"))
    meta = json.loads(str(d["meta"]))
    frames = []
    k = 0
    while f"s{k}_n" in d:
        nodes = []
        for j in range(int(d[f"s{k}_n"])):
            nodes.append((int(d[f"s{k}_n{j}_level"]), d[f"s{k}_n{j}_mglobal"], d[f"s{k}_n{j}_q"]))
        frames.append((nodes, d[f"s{k}_res"]))
        k += 1
    return meta, frames


def params_of(c):
    p = c["pdata"]
    if c["problem"] == "CH":
        return "ch", [c["dt"], p["eps"]]
    return "biogrowth", [c["dt"], p["eps"], p["gamma"], p["lambda_"], p["czero"]]


def oracle_nodes(o, nd, finest):
    """(level, mglobal, q) of the levels 0..finest in visiting order: the
    table is in creation order, and a level is visited youngest first"""
    out = []
    tab = o.patch_table()
    for level in range(finest + 1):
        for p in reversed([x for x in tab if x["level"] == level]):
            mg = np.array(p["mglobal"], dtype=np.int64).reshape(3, 2)
            out.append((p["level"], mg, o.get(p["id"], "q"), p["mx"]))
    return out


def compare_frame(ref_nodes, ora_nodes, nd, nv, mbc, where):
    assert len(ref_nodes) == len(ora_nodes), (where, len(ref_nodes), len(ora_nodes))
    by_key = {(lev, tuple(mg[:nd].ravel())): q for lev, mg, q, _ in ora_nodes}
    for lev, mg, q in ref_nodes:
        key = (lev, tuple(np.asarray(mg)[:nd].ravel()))
        assert key in by_key, (where, key)
        want = np.asarray(q)
        got = by_key[key]
        got = got.reshape(want.shape, order="F")
        bad = np.argwhere(got != want)
        assert bad.size == 0, (where, key, bad[:5], got[tuple(bad[0])], want[tuple(bad[0])])
    # and the same visiting order
    assert [(l, tuple(np.asarray(m)[:nd].ravel())) for l, m, _ in ref_nodes] == \
           [(l, tuple(m[:nd].ravel())) for l, m, _, _ in ora_nodes], where


def _start(oracle_mod, c):
    nd, n, L, mbc = c["nd"], c["n"], c["length"], c["mbc"]
    minlevel = -int(round(np.log2(n))) + 1
    prob, params = params_of(c)
    o = oracle_mod.OracleHierarchy(nd, 2, prob, params, mbc=mbc)
    mthbc = [c["mthbc"]] * (2 * nd) + [10] * (6 - 2 * nd)
    o.build_uniform([n] * nd + [1] * (3 - nd), minlevel, mthbc, [0, 0, 0], [L] * nd + [1] * (3 - nd))
    o.commit()
    fn = G.qinit_fn(c)
    q0 = np.asarray(fn(0, [n] * nd, [L / n] * nd, [0.0] * nd))
    if mbc == 2:  # the same interior in arrays with two ghost layers
        q2 = np.zeros((n + 4,) * nd + (2,), order="F")
        q2[(slice(2, -2),) * nd] = q0[(slice(1, -1),) * nd]
        q0 = q2
    o.put(0, "q", q0)
    # Initialq, SetGhost(rootlevel, 0), CopyQToQold (bsamroutines.f90:133-146)
    o.set_ghost(0, 0)
    o.copy_q_to_qold(minlevel, 0)
    return o, fn, minlevel


def _regrid(oracle_mod, o, c, fn, step):
    prm = oracle_mod.regrid_params(c["maxlevel"], tagging="ch", initial=step == 1, qtolerance=c["qtol"],
                                   first_id=1000 * step)
    o = oracle_mod.regrid(o, prm, fn if step == 1 else None)
    return o, max(p["level"] for p in o.patch_table())


@pytest.mark.parametrize("name", FIXTURES)
def test_oracle_equals_the_reference(oracle_mod, name):
    meta, frames = load(name)
    c = G.CASES[name]
    assert meta["steps"] == c["steps"]
    nd, mbc = c["nd"], c["mbc"]
    amr = c["maxlevel"] > 0
    # frame 0, the state the reference writes after the first regrid,
    # FillDown and CopyQToQold (TakeTimeSteps, bsamroutines.f90:657-705)
    o, fn, minlevel = _start(oracle_mod, c)
    finest = 0
    if amr:
        o, finest = _regrid(oracle_mod, o, c, fn, 1)
    else:
        o.set_ghost(0, 0)
    o.fill_down("q", finest, minlevel)
    compare_frame(frames[0][0], oracle_nodes(o, nd, finest), nd, 2, mbc, (name, "frame 0"))
    # the time steps: regrid (AMR) and bsamg-style time step
    o, fn, minlevel = _start(oracle_mod, c)
    for step in range(1, c["steps"] + 1):
        if amr:
            o, finest = _regrid(oracle_mod, o, c, fn, step)
        nv, res = o.time_step(step == 1, finest, minlevel, 2, 20, c["tol"])
        ref_nodes, ref_res = frames[step]
        assert np.array_equal(np.array(res), ref_res), (name, step, res, ref_res)
        compare_frame(ref_nodes, oracle_nodes(o, nd, finest), nd, 2, mbc, (name, "step", step))
