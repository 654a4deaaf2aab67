"""Writes tests/golden/ref_*.npz: outputs of the BSAM 1.2 reference itself.

The reference is Fortran and no Fortran compiler exists on the machines this
repository is built on, so its unmodified source (LIBRARY/*.f90 and the
problem plugin PROBLEM/<name>/*.f90) is run by oracle/fortran_exec.py, an
interpreter for the Fortran subset it is written in.  The whole program runs
as the reference runs it (BSAMDriver -> BSAMSolver: namelist input files,
RootInit, InitSeed, SetProb, TakeTimeSteps with its regrid, CopyQToQold and
MultigridIterations) with three harness hooks and nothing else replaced:

* the plugin's QInit2D/3D fills the patch from the seeded generators in
  bsam1.2_gb300/initial.py (the reference's own QInit draws from the
  compiler's random-number generator);
* WriteQ (called after every time step when outframes = timeiterations)
  records every node's level, mglobal and q instead of writing a file;
* WriteUniformMeshQ does nothing.

The residual history is the reference's own `PRINT *, 'it =', itmg,
' residual =', residual` output of MultigridIterations.  Run from the
repository root with the reference checked out at /root/reference:

    python tests/golden/make_reference_golden.py [case ...]
"""
import importlib.util
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("BSAM_REFERENCE", "/root/reference")
sys.path.insert(0, ROOT)

from oracle import fortran_exec as F  # noqa: E402

_spec = importlib.util.spec_from_file_location("bsam_initial", os.path.join(ROOT, "bsam1.2_gb300", "initial.py"))
initial = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(initial)

LIB = ["nodeinfodef", "treeops", "gridutilities", "bsamstorage", "boundary", "bsaminputoutput", "afasroutines",
       "bsamroutines", "bsamdriver"]

# case: problem, ndims, root cells per side, domain length, boundary codes,
# maxlevel, mbc, time steps, rundata values, problemdata values, initial
# condition
CASES = {
    "ch2d_periodic_32": dict(problem="CH", nd=2, n=32, length=1.0, mthbc=2, maxlevel=0, mbc=1, steps=3,
                             dt=1e-3, tol=1e-9, pdata=dict(alpha=1.0, eps=0.01), init=("spinodal", 7, 0.0, 0.05)),
    "ch2d_neumann_32": dict(problem="CH", nd=2, n=32, length=1.0, mthbc=10, maxlevel=0, mbc=1, steps=3,
                            dt=1e-3, tol=1e-9, pdata=dict(alpha=1.0, eps=0.01), init=("spinodal", 8, 0.0, 0.05)),
    "ch2d_periodic_16_mbc2": dict(problem="CH", nd=2, n=16, length=1.0, mthbc=2, maxlevel=0, mbc=2, steps=2,
                                  dt=1e-3, tol=1e-9, pdata=dict(alpha=1.0, eps=0.01),
                                  init=("spinodal", 9, 0.0, 0.05)),
    "ch3d_periodic_16": dict(problem="CH", nd=3, n=16, length=1.0, mthbc=2, maxlevel=0, mbc=1, steps=2,
                             dt=5e-4, tol=1e-8, pdata=dict(alpha=1.0, eps=0.02), init=("spinodal", 10, 0.1, 0.05)),
    "ch3d_dirichlet_8": dict(problem="CH", nd=3, n=8, length=1.0, mthbc=10, maxlevel=0, mbc=1, steps=2,
                             dt=5e-4, tol=1e-8, pdata=dict(alpha=1.0, eps=0.05), init=("spinodal", 11, 0.1, 0.05)),
    "bio2d_neumann_32": dict(problem="BioGrowth", nd=2, n=32, length=6.4, mthbc=10, maxlevel=0, mbc=1, steps=2,
                             dt=0.1, tol=1e-9, pdata=dict(czero=0.5, gamma=1.5, lambda_=2.0, eps=0.05),
                             init=("bio", 12)),
    "ch2d_amr_32": dict(problem="CH", nd=2, n=32, length=1.0, mthbc=2, maxlevel=2, mbc=1, steps=3,
                        dt=1e-3, tol=1e-9, pdata=dict(alpha=1.0, eps=0.03), qtol=0.05,
                        init=("circle", 13, 0.25, 0.01)),
    "ch2d_amr_neumann_32": dict(problem="CH", nd=2, n=32, length=1.0, mthbc=10, maxlevel=2, mbc=1, steps=2,
                                dt=1e-3, tol=1e-9, pdata=dict(alpha=1.0, eps=0.03), qtol=0.05,
                                init=("circle", 14, 0.3, 0.01)),
    "ch3d_amr_16": dict(problem="CH", nd=3, n=16, length=1.0, mthbc=2, maxlevel=1, mbc=1, steps=2,
                        dt=5e-4, tol=1e-8, pdata=dict(alpha=1.0, eps=0.05), qtol=0.05,
                        init=("circle", 15, 0.3, 0.01)),
}


def qinit_fn(c):
    """fn(level, mx, dx, xlower) -> ghosted Fortran-layout q of a patch"""
    kind = c["init"][0]
    nd, n = c["nd"], c["n"]
    eps = c["pdata"]["eps"]
    if kind == "spinodal":
        _, seed, mean, amp = c["init"]
        q0 = initial.ch_spinodal((n,) * nd, eps, c["length"] / n, seed=seed, mean=mean, amp=amp)
        return lambda level, mx, dx, xl: q0
    if kind == "bio":
        seed = c["init"][1]
        q = np.zeros((n + 2,) * nd + (2,), order="F")
        q[(slice(1, -1),) * nd + (0,)] = initial.splitmix_pm1(seed, initial.global_index((n,) * nd)).reshape(
            (n,) * nd, order="F") * 0.9
        q[(slice(1, -1),) * nd + (1,)] = 1.0
        return lambda level, mx, dx, xl: q
    _, seed, radius, noise = c["init"]
    return initial.ch_circle_patch(eps, seed, radius=radius, noise=noise, length=c["length"])


def _nml(group, items):
    lines = [f"&{group}"]
    for k, v in items:
        if isinstance(v, bool):
            s = ".true." if v else ".false."
        elif isinstance(v, float):
            s = repr(v).replace("e", "d") if "e" in repr(v) else repr(v) + "d0"
        else:
            s = str(v)
        lines.append(f"{k} = {s}")
    return "\n".join(lines) + "/\n"


def input_files(c):
    nd, n, L = c["nd"], c["n"], c["length"]
    minlevel = -int(round(np.log2(n))) + 1
    run = [("restart", False), ("restartframe", 0), ("syncelliptic", False), ("outframes", c["steps"]),
           ("outputuniformmesh", False), ("getafterstepstats", False), ("timeiterations", c["steps"]),
           ("maxvcycles", 20), ("nsmoothingpasses", 2), ("omega", 1.0), ("qerrortol", c["tol"]),
           ("dt", c["dt"])]
    grid = [("ndims", nd), ("maxlevel", c["maxlevel"]), ("minlevel", minlevel)]
    for l in range(c["maxlevel"] + 1):
        grid += [(f"qtolerance({l})", c.get("qtol", 1e-2)), (f"ibuffer({l})", 1),
                 (f"minimumgridpoints({l})", 4), (f"desiredfillratios({l})", 0.9), (f"errflagopt({l})", 10)]
    for d in range(3):
        m = n if d < nd else 1
        grid += [(f"mx({d + 1})", m), (f"mglobal({d + 1},1)", 1), (f"mglobal({d + 1},2)", m),
                 (f"xlower({d + 1})", 0.0), (f"xupper({d + 1})", L if d < nd else 1.0)]
    grid += [("mbc", c["mbc"])]
    for face in range(6):
        grid += [(f"mthbc({face + 1})", c["mthbc"] if face < 2 * nd else 10)]
    grid += [("qpo(1)", 0.0), ("qpo(2)", 0.0), ("nrvars", 2), ("maux", 0)]
    pd = [(k.rstrip("_"), v) for k, v in c["pdata"].items()]
    return {"rundata.dat": _nml("rundata", run), "griddata.dat": _nml("griddata", grid),
            "problemdata.dat": _nml("problemdata", pd)}


def run_reference(name):
    c = CASES[name]
    prob = c["problem"]
    paths = [os.path.join(REF, "LIBRARY", "nodeinfodef.f90"), os.path.join(REF, "PROBLEM", prob, "problemdef.f90")]
    for m in LIB[1:]:
        if m == "bsamstorage":
            paths.append(os.path.join(REF, "PROBLEM", prob, "problem.f90"))
        paths.append(os.path.join(REF, "LIBRARY", m + ".f90"))
    I = F.Interp(paths, files=input_files(c))
    fn = qinit_fn(c)
    nd = c["nd"]

    def qinit(I, p, actuals, fc):
        f = I.bind(p, actuals, fc)
        q = f["q"]
        mx = [int(v) for v in f["mx"].a[:nd]]
        h = f["h"].get()
        xl = [float(v) for v in f["xlower"].a[:nd]]
        full = np.asarray(fn(None, mx, [h] * nd, xl))
        q.a[...] = full[(slice(1, -1),) * nd].reshape(q.a.shape, order="F")
    I.proc(f"qinit{nd}d").hook = qinit

    snaps = []
    ndi = I.modules["nodeinfodef"]
    ap = I.proc("applyonlevel")
    funcparam = ndi.find_type("funcparam")

    def writeq(I, p, actuals, fc):
        f = I.bind(p, actuals, fc)
        nodes = []

        def record(info, dummy):
            q = info.c["q"]
            nodes.append((int(info.c["level"]), info.c["mglobal"].a.copy(), q.a.copy(), q.lb))
            return 0
        for level in range(0, int(ndi.vars["finestlevel"]) + 1):
            I.call_proc(ap, [F.Actual(None, (lambda f, l=level: l), None, None),
                             F.Actual(None, None, (lambda f: F.PyProc(record)), None),
                             F.Actual(None, (lambda f: I.new_dt(funcparam, None, "funcparam")), None, None)], {})
        snaps.append((f["nframe"].get(), f["time"].get(), nodes, len(I.printed)))
    I.proc("writeq").hook = writeq
    I.proc("writeuniformmeshq").hook = lambda *a: None
    t = time.time()
    I.run_program()
    secs = time.time() - t
    # residual histories per step: the prints between consecutive snapshots
    out = {"meta": json.dumps(dict(c, name=name, seconds=secs))}
    for k, (nframe, tm, nodes, nprint) in enumerate(snaps):
        lo = snaps[k - 1][3] if k > 0 else 0
        res = [v[3] for v in I.printed[lo:nprint] if v and isinstance(v[0], str) and v[0].strip() == "it ="]
        out[f"s{k}_time"] = np.array(tm)
        out[f"s{k}_res"] = np.array(res, dtype=np.float64)
        out[f"s{k}_n"] = np.array(len(nodes))
        for j, (lev, mg, q, lb) in enumerate(nodes):
            out[f"s{k}_n{j}_level"] = np.array(lev)
            out[f"s{k}_n{j}_mglobal"] = mg
            out[f"s{k}_n{j}_q"] = q
    return out, secs


def main(names):
    for name in names or list(CASES):
        out, secs = run_reference(name)
        path = os.path.join(HERE, f"ref_{name}.npz")
        np.savez_compressed(path, **out)
        nsteps = sum(1 for k in out if k.endswith("_res"))
        print(f"{name}: {secs:.1f} s, {nsteps} frames, {os.path.getsize(path)} bytes")


if __name__ == "__main__":
    main(sys.argv[1:])
