"""Python host mirror of the BSAM 1.2 multigrid interface over libbsamg.so.

The methods follow the reference routines they stand for (see the citations
in include/bsamg.h): a Hierarchy is the set of nodes the Fortran host visits
with ApplyOnLevel, and multigrid_iterations / time_step are
MultigridIterations and one TakeTimeSteps step.  All work runs in the CUDA
library; there is no CPU path here, and a missing library is an error.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# BSAMG_LIBRARY names another build of the library (one linked with extra
# problem plugins, bsam1.2_gb300/build.py build(extra_plugins=...))
LIB_PATH = os.environ.get("BSAMG_LIBRARY") or os.path.join(HERE, "libbsamg.so")

FIELD = {"q": 0, "qold": 1, "qc": 2, "f": 3, "rf": 4, "ftmp": 5}
MODE = {"fp64": 0, "mixed": 1}

_lib = None


class BsamgError(RuntimeError):
    def __init__(self, status, what):
        L = lib()
        msg = L.bsamg_strerror(status).decode()
        detail = L.bsamg_last_error_detail().decode()
        super().__init__(f"{what}: {msg} ({status}){': ' + detail if detail else ''}")
        self.status = status


class RegridParams(ctypes.Structure):
    """bsamg_regrid_params (include/bsamg.h)."""
    _fields_ = [("maxlevel", ctypes.c_int), ("tagging", ctypes.c_int), ("initial", ctypes.c_int),
                ("maxside", ctypes.c_int), ("first_id", ctypes.c_int), ("ibuffer", ctypes.c_int * 11),
                ("minimumgridpoints", ctypes.c_int * 11), ("qtolerance", ctypes.c_double * 11),
                ("desiredfillratio", ctypes.c_double * 11)]


TAGGING = {"ch": 0, "gradient": 1}
# bsamg_qinit_fn: (user, level, mx[3], dx[3], xlower[3], q)
QINIT = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                         ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                         ctypes.POINTER(ctypes.c_double))


def regrid_params(maxlevel, tagging="ch", initial=False, maxside=0, first_id=1000, ibuffer=1,
                  minimumgridpoints=4, qtolerance=1e-2, desiredfillratio=0.9):
    """bsamg_regrid_params; scalars apply to every level, lists per level
    (the griddata namelist entries of the reference)."""
    r = RegridParams()
    r.maxlevel, r.tagging, r.initial, r.maxside, r.first_id = (maxlevel, TAGGING[tagging], int(initial), maxside,
                                                              first_id)
    per = lambda x, l: x[l] if isinstance(x, (list, tuple)) else x
    for l in range(11):
        r.ibuffer[l] = per(ibuffer, l)
        r.minimumgridpoints[l] = per(minimumgridpoints, l)
        r.qtolerance[l] = per(qtolerance, l)
        r.desiredfillratio[l] = per(desiredfillratio, l)
    return r


def embed_ghosted(a, mx, nrvars, mbc):
    """A Fortran-ordered array q(1-g:mx+g, ..., nrvars) with g = 1 or mbc as
    the hierarchy's ghosted layout q(1-mbc:mx+mbc, ...): an array with one
    ghost layer goes to q(0:mx+1), the second layer left zero."""
    nd = len(mx)
    a = np.asarray(a, dtype=np.float64).ravel(order="F")
    full = int(np.prod([v + 2 * mbc for v in mx])) * nrvars
    one = int(np.prod([v + 2 for v in mx])) * nrvars
    if a.size == full:
        return a
    if a.size != one:
        raise ValueError(f"qinit returned {a.size} values for a patch of {full}")
    out = np.zeros([v + 2 * mbc for v in mx] + [nrvars], order="F")
    g = mbc - 1
    out[tuple(slice(g, g + v + 2) for v in mx) + (slice(None),)] = a.reshape([v + 2 for v in mx] + [nrvars], order="F")
    return out.ravel(order="F")


def qinit_callback(fn, ndims, nrvars, mbc=1):
    """bsamg_qinit_fn around fn(level, mx, dx, xlower) -> the new patch's
    ghosted Fortran-layout array (only its interior is used), with mbc or
    one ghost layer."""
    def cb(user, level, mx, dx, xl, q):
        m = [mx[d] for d in range(ndims)]
        a = embed_ghosted(fn(level, m, [dx[d] for d in range(ndims)], [xl[d] for d in range(ndims)]), m, nrvars, mbc)
        ctypes.memmove(q, a.ctypes.data, a.size * 8)
    return QINIT(cb)


def lib():
    """Load libbsamg.so (built by __graft_entry__.build()); fail loudly if absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"libbsamg.so is not built ({LIB_PATH}); run __graft_entry__.build()")
    L = ctypes.CDLL(LIB_PATH)
    I, D, P, SZ = ctypes.c_int, ctypes.c_double, ctypes.c_void_p, ctypes.c_size_t
    IP, DP = ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)
    sig = {
        "bsamg_init": ([I, SZ, ctypes.POINTER(P)], I),
        "bsamg_finalize": ([P], I),
        "bsamg_ctx_usage": ([P, ctypes.POINTER(SZ), ctypes.POINTER(SZ)], I),
        "bsamg_ctx_set_blocking_wait": ([P, I], I),
        "bsamg_hier_create": ([P, I, I, I, I, DP, I, DP, ctypes.POINTER(P)], I),
        "bsamg_hier_destroy": ([P], I),
        "bsamg_patch_add": ([P, I, I, I, IP, IP, IP, IP, DP, DP], I),
        "bsamg_build_uniform": ([P, IP, I, IP, DP, DP], I),
        "bsamg_commit": ([P], I),
        "bsamg_num_patches": ([P, IP], I),
        "bsamg_level_range": ([P, IP, IP], I),
        "bsamg_patch_info": ([P, I, IP, DP], I),
        "bsamg_regrid": ([P, ctypes.POINTER(RegridParams), QINIT, P, ctypes.POINTER(P)], I),
        "bsamg_field_size": ([P, I, I], SZ),
        "bsamg_put_field": ([P, I, I, DP, SZ], I),
        "bsamg_get_field": ([P, I, I, DP, SZ], I),
        "bsamg_put_field_section": ([P, I, I, DP, IP, IP], I),
        "bsamg_get_field_section": ([P, I, I, DP, IP, IP], I),
        "bsamg_relax_level_color": ([P, I, I], I),
        "bsamg_set_ghost": ([P, I, I], I),
        "bsamg_level_relax": ([P, I, I], I),
        "bsamg_fill_down": ([P, I, I, I], I),
        "bsamg_copy_q_to_qold": ([P, I, I], I),
        "bsamg_vcycle": ([P, I, I, I], I),
        "bsamg_residual_norm": ([P, I, I, DP], I),
        "bsamg_multigrid_iterations": ([P, I, I, I, I, D, I, I, I, I, IP, DP], I),
        "bsamg_time_step": ([P, I, I, I, I, I, D, I, I, I, I, IP, DP], I),
        "bsamg_sync": ([P], I),
        "bsamg_stream": ([P, ctypes.POINTER(P)], I),
        "bsamg_launch_count": ([P, ctypes.POINTER(ctypes.c_longlong)], I),
        "bsamg_set_tail_cells": ([P, ctypes.c_longlong], I),
        "bsamg_set_box_sweep": ([P, I], I),
        "bsamg_set_solve": ([P, I, I, I, I, ctypes.c_longlong], I),
        "bsamg_get_solve": ([P, IP, IP, IP, IP, ctypes.POINTER(ctypes.c_longlong)], I),
        "bsamg_solve_trace": ([P, I], I),
        "bsamg_regrid_timing": ([P, DP, I], I),
        "bsamg_ctx_set_autotune": ([P, I], I),
        "bsamg_tune_save": ([P, ctypes.c_char_p], I),
        "bsamg_tune_load": ([P, ctypes.c_char_p], I),
        "bsamg_tune_count": ([P, IP], I),
        "bsamg_solve_info": ([P, ctypes.POINTER(ctypes.c_longlong), I], I),
        "bsamg_solve_trace_read": ([P, I, IP, IP, ctypes.POINTER(ctypes.c_longlong), IP], I),
        "bsamg_graph_stats": ([P, IP, IP], I),
        "bsamg_set_params": ([P, DP, I], I),
        "bsamg_hier_reset": ([P], I),
        "bsamg_mark": ([P, I], I),
        "bsamg_elapsed_ms": ([P, I, I, DP], I),
        "bsamg_time_smoother": ([P, I, I, I, DP], I),
        "bsamg_smoother_colours": ([P, I, I, IP], I),
        "bsamg_ch_residual_norm_noalloc": ([P, P, I, IP, D, D, D, I, P, P], I),
        "bsamg_host_register": ([P, SZ], I),
        "bsamg_host_unregister": ([P], I),
        "bsamg_after_step_stats": ([P, I, DP, ctypes.POINTER(ctypes.c_longlong)], I),
        "bsamg_write_q": ([P, ctypes.c_char_p, D, I], I),
        "bsamg_write_uniform_q": ([P, ctypes.c_char_p, D, I], I),
        "bsamg_read_q": ([P, ctypes.c_char_p, I, DP, ctypes.POINTER(P)], I),
        "bsamg_format_f25_12": ([D, ctypes.c_char_p], I),
        "bsamg_seed_spinodal": ([P, I, ctypes.c_ulonglong, D, D], I),
        "bsamg_format_stats_line": ([D, DP, ctypes.c_longlong, ctypes.c_char_p, SZ], I),
        "bsamg_problem_kind": ([ctypes.c_char_p, IP], I),
        "bsamg_problem_info": ([I, IP, IP, IP], I),
        "bsamg_strerror": ([I], ctypes.c_char_p),
        "bsamg_last_error_detail": ([], ctypes.c_char_p),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


def problem_kind(problem):
    """The kind of a registered problem plugin, by name ("ch", "biogrowth",
    "growth", or any plugin linked into the library) or kind."""
    if isinstance(problem, int):
        return problem
    k = ctypes.c_int()
    _ck(lib().bsamg_problem_kind(problem.encode(), ctypes.byref(k)), f"bsamg_problem_kind({problem!r})")
    return k.value


def problem_info(problem):
    """(nrvars, minimum parameter count, has a mixed-precision form) of a plugin."""
    nv, npar, mixed = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    _ck(lib().bsamg_problem_info(problem_kind(problem), ctypes.byref(nv), ctypes.byref(npar), ctypes.byref(mixed)),
        "bsamg_problem_info")
    return nv.value, npar.value, bool(mixed.value)


def exported_symbols():
    """Names of the C-ABI entry points the Python mirror binds."""
    lib()
    return [n for n in dir(_lib) if n.startswith("bsamg_")]


def _ck(rc, what):
    if rc != 0:
        raise BsamgError(rc, what)


def _ia(x, n):
    return (ctypes.c_int * n)(*[int(v) for v in x])


def _da(x, n):
    return (ctypes.c_double * n)(*[float(v) for v in x])


class Context:
    """One GPU and an HBM budget (bytes, 0 = unlimited)."""

    def __init__(self, device=0, hbm_budget=0):
        h = ctypes.c_void_p()
        _ck(lib().bsamg_init(device, hbm_budget, ctypes.byref(h)), "bsamg_init")
        self.h = h

    def usage(self):
        u, b = ctypes.c_size_t(), ctypes.c_size_t()
        _ck(lib().bsamg_ctx_usage(self.h, ctypes.byref(u), ctypes.byref(b)), "bsamg_ctx_usage")
        return u.value, b.value

    def set_blocking_wait(self, on=True):
        """Host waits sleep instead of spinning (bsamg_ctx_set_blocking_wait)."""
        _ck(lib().bsamg_ctx_set_blocking_wait(self.h, int(bool(on))), "bsamg_ctx_set_blocking_wait")

    def set_autotune(self, on=True):
        """The one-launch solve's autotuner on or off (bsamg_ctx_set_autotune)."""
        _ck(lib().bsamg_ctx_set_autotune(self.h, int(bool(on))), "bsamg_ctx_set_autotune")

    def tune_save(self, path):
        """Write the autotuner's choices as JSON (bsamg_tune_save)."""
        _ck(lib().bsamg_tune_save(self.h, str(path).encode()), "bsamg_tune_save")

    def tune_load(self, path):
        """Add the choices of a file written by tune_save (bsamg_tune_load)."""
        _ck(lib().bsamg_tune_load(self.h, str(path).encode()), "bsamg_tune_load")

    def tune_count(self):
        """Size classes the autotuner has a choice for (bsamg_tune_count)."""
        n = ctypes.c_int()
        _ck(lib().bsamg_tune_count(self.h, ctypes.byref(n)), "bsamg_tune_count")
        return n.value

    def close(self):
        if getattr(self, "h", None):
            lib().bsamg_finalize(self.h)
            self.h = None

    def __del__(self):
        self.close()


class Hierarchy:
    """A device-resident patch hierarchy (nodes of one mesh)."""

    def __init__(self, ctx, ndims, nrvars, problem, params, qpo=None, mbc=1):
        self.ctx = ctx
        self.ndims, self.nrvars, self.mbc = ndims, nrvars, mbc
        h = ctypes.c_void_p()
        p = _da(params, len(params))
        q = _da(qpo if qpo is not None else [0.0] * nrvars, nrvars)
        _ck(lib().bsamg_hier_create(ctx.h, ndims, nrvars, mbc, problem_kind(problem), p, len(params), q,
                                    ctypes.byref(h)), "bsamg_hier_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().bsamg_hier_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def add_patch(self, level, id, parent_id, mx, mglobal, mbounds, mthbc, dx, xlower):
        _ck(lib().bsamg_patch_add(self.h, level, id, parent_id, _ia(mx, 3), _ia(mglobal, 6),
                                  _ia(mbounds, 6), _ia(mthbc, 6), _da(dx, 3), _da(xlower, 3)),
            "bsamg_patch_add")

    def build_uniform(self, mx, minlevel, mthbc, xlower, xupper):
        _ck(lib().bsamg_build_uniform(self.h, _ia(mx, 3), minlevel, _ia(mthbc, 6), _da(xlower, 3),
                                      _da(xupper, 3)), "bsamg_build_uniform")

    def level_range(self):
        """(minlevel, finest level) of the committed hierarchy (bsamg_level_range)."""
        a, b = ctypes.c_int(), ctypes.c_int()
        _ck(lib().bsamg_level_range(self.h, ctypes.byref(a), ctypes.byref(b)), "bsamg_level_range")
        return a.value, b.value

    def patch_table(self):
        """Geometry of every patch in visiting order (bsamg_patch_info)."""
        L = lib()
        n = ctypes.c_int()
        _ck(L.bsamg_num_patches(self.h, ctypes.byref(n)), "bsamg_num_patches")
        out = []
        for i in range(n.value):
            a = (ctypes.c_int * 24)()
            d = (ctypes.c_double * 6)()
            _ck(L.bsamg_patch_info(self.h, i, a, d), "bsamg_patch_info")
            a = list(a)
            out.append(dict(level=a[0], id=a[1], parent_id=a[2], mx=a[3:6], mglobal=a[6:12], mbounds=a[12:18],
                            mthbc=a[18:24], dx=list(d)[0:3], xlower=list(d)[3:6]))
        return out

    def regrid(self, params, qinit=None):
        """AMR regrid (bsamg_regrid): a new Hierarchy on the same context;
        this one is unchanged."""
        cb = qinit_callback(qinit, self.ndims, self.nrvars, self.mbc) if qinit is not None else QINIT()
        h = ctypes.c_void_p()
        _ck(lib().bsamg_regrid(self.h, ctypes.byref(params), cb, None, ctypes.byref(h)), "bsamg_regrid")
        new = Hierarchy.__new__(Hierarchy)
        new.ctx, new.ndims, new.nrvars, new.mbc, new.h = self.ctx, self.ndims, self.nrvars, self.mbc, h
        return new

    def after_step_stats(self, finest):
        """AfterStepStatistics + GetMeshSize (bsamg_after_step_stats):
        (integral of phi, CH 2D energy, composite mesh size)."""
        r = (ctypes.c_double * 2)()
        m = ctypes.c_longlong()
        _ck(lib().bsamg_after_step_stats(self.h, finest, r, ctypes.byref(m)), "bsamg_after_step_stats")
        return r[0], r[1], m.value

    def write_q(self, path, time, finest):
        """WriteQ: the text frame file of levels 0..finest (bsamg_write_q)."""
        _ck(lib().bsamg_write_q(self.h, os.fsencode(path), time, finest), "bsamg_write_q")

    def write_uniform_q(self, path, time, finest):
        """WriteUniformMeshQ: the composite on one uniform grid (bsamg_write_uniform_q)."""
        _ck(lib().bsamg_write_uniform_q(self.h, os.fsencode(path), time, finest), "bsamg_write_uniform_q")

    def read_q(self, path, first_id=1000):
        """ReadQ: restart from a frame file, with this hierarchy as the root
        grid (bsamg_read_q); returns (new Hierarchy, frame time)."""
        h = ctypes.c_void_p()
        t = ctypes.c_double()
        _ck(lib().bsamg_read_q(self.h, os.fsencode(path), first_id, ctypes.byref(t), ctypes.byref(h)),
            "bsamg_read_q")
        new = Hierarchy.__new__(Hierarchy)
        new.ctx, new.ndims, new.nrvars, new.mbc, new.h = self.ctx, self.ndims, self.nrvars, self.mbc, h
        return new, t.value

    def seed_spinodal(self, pid, seed, mean=0.0, amp=0.05):
        """The seeded spinodal start of patch pid, generated on the device
        (bsamg_seed_spinodal; the same values as initial.ch_spinodal)."""
        _ck(lib().bsamg_seed_spinodal(self.h, pid, seed, mean, amp), "bsamg_seed_spinodal")

    def put_section(self, pid, field, lo, hi, arr):
        """Write the box section lo..hi (Fortran bounds, variable last) of a
        field from arr (bsamg_put_field_section)."""
        a = np.ascontiguousarray(np.asarray(arr, dtype=np.float64).ravel(order="F"))
        _ck(lib().bsamg_put_field_section(self.h, pid, FIELD[field], a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                          _ia(lo, 4), _ia(hi, 4)), "bsamg_put_field_section")

    def get_section(self, pid, field, lo, hi):
        """The box section lo..hi of a field, Fortran-ordered with shape
        hi - lo + 1 (bsamg_get_field_section)."""
        shape = tuple(int(h) - int(l) + 1 for l, h in zip(lo, hi))
        a = np.empty(int(np.prod(shape)), dtype=np.float64)
        _ck(lib().bsamg_get_field_section(self.h, pid, FIELD[field], a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                          _ia(lo, 4), _ia(hi, 4)), "bsamg_get_field_section")
        return a.reshape(shape, order="F")

    def commit(self):
        _ck(lib().bsamg_commit(self.h), "bsamg_commit")

    def field_size(self, pid, field):
        return lib().bsamg_field_size(self.h, pid, FIELD[field])

    def put(self, pid, field, arr):
        a = np.ascontiguousarray(np.asarray(arr, dtype=np.float64).ravel(order="F"))
        _ck(lib().bsamg_put_field(self.h, pid, FIELD[field],
                                  a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), a.size),
            "bsamg_put_field")

    def put_flat(self, pid, field, flat):
        """put from an already Fortran-ordered contiguous float64 buffer (no copy)"""
        _ck(lib().bsamg_put_field(self.h, pid, FIELD[field],
                                  flat.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), flat.size),
            "bsamg_put_field")

    def get(self, pid, field, out=None):
        n = self.field_size(pid, field)
        a = out if out is not None else np.empty(n, dtype=np.float64)
        _ck(lib().bsamg_get_field(self.h, pid, FIELD[field],
                                  a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), n),
            "bsamg_get_field")
        return a

    def relax_level_color(self, level, ipass):
        _ck(lib().bsamg_relax_level_color(self.h, level, ipass), "bsamg_relax_level_color")

    def set_ghost(self, level, ipass):
        _ck(lib().bsamg_set_ghost(self.h, level, ipass), "bsamg_set_ghost")

    def level_relax(self, level, nsmooth):
        _ck(lib().bsamg_level_relax(self.h, level, nsmooth), "bsamg_level_relax")

    def fill_down(self, field, finest, minlevel):
        _ck(lib().bsamg_fill_down(self.h, {"f": 1, "q": 2}[field], finest, minlevel), "bsamg_fill_down")

    def copy_q_to_qold(self, minlevel, finest):
        _ck(lib().bsamg_copy_q_to_qold(self.h, minlevel, finest), "bsamg_copy_q_to_qold")

    def vcycle(self, level, minlevel, nsmooth):
        _ck(lib().bsamg_vcycle(self.h, level, minlevel, nsmooth), "bsamg_vcycle")

    def residual_norm(self, level, errortype=1):
        r = ctypes.c_double()
        _ck(lib().bsamg_residual_norm(self.h, level, errortype, ctypes.byref(r)), "bsamg_residual_norm")
        return r.value

    def multigrid_iterations(self, finest, minlevel, nsmooth=2, maxvcycles=20, tol=1e-9,
                             updateauxfreq=1, errortype=1, mode="fp64", strict=False):
        n = ctypes.c_int()
        res = (ctypes.c_double * maxvcycles)()
        _ck(lib().bsamg_multigrid_iterations(self.h, finest, minlevel, nsmooth, maxvcycles, tol,
                                             updateauxfreq, errortype, MODE[mode], int(strict),
                                             ctypes.byref(n), res), "bsamg_multigrid_iterations")
        return n.value, list(res)[: n.value]

    def time_step(self, first, finest, minlevel, nsmooth=2, maxvcycles=20, tol=1e-9,
                  updateauxfreq=1, errortype=1, mode="fp64", strict=False):
        n = ctypes.c_int()
        res = (ctypes.c_double * maxvcycles)()
        _ck(lib().bsamg_time_step(self.h, int(bool(first)), finest, minlevel, nsmooth, maxvcycles,
                                  tol, updateauxfreq, errortype, MODE[mode], int(strict),
                                  ctypes.byref(n), res), "bsamg_time_step")
        return n.value, list(res)[: n.value]

    def sync(self):
        _ck(lib().bsamg_sync(self.h), "bsamg_sync")

    def stream(self):
        s = ctypes.c_void_p()
        _ck(lib().bsamg_stream(self.h, ctypes.byref(s)), "bsamg_stream")
        return s.value

    def mark(self, slot):
        _ck(lib().bsamg_mark(self.h, slot), "bsamg_mark")

    def elapsed_ms(self, a, b):
        ms = ctypes.c_double()
        _ck(lib().bsamg_elapsed_ms(self.h, a, b, ctypes.byref(ms)), "bsamg_elapsed_ms")
        return ms.value

    def time_smoother(self, level, mode="fp64", reps=20):
        ms = ctypes.c_double()
        _ck(lib().bsamg_time_smoother(self.h, level, MODE[mode], reps, ctypes.byref(ms)),
            "bsamg_time_smoother")
        return ms.value

    def smoother_colours(self, level, mode="fp64"):
        n = ctypes.c_int()
        _ck(lib().bsamg_smoother_colours(self.h, level, MODE[mode], ctypes.byref(n)), "bsamg_smoother_colours")
        return n.value

    def set_params(self, params):
        """New plugin parameters for a committed hierarchy (bsamg_set_params)."""
        _ck(lib().bsamg_set_params(self.h, _da(params, len(params)), len(params)), "bsamg_set_params")

    def reset(self):
        """Every field back to zero, as after commit (bsamg_hier_reset)."""
        _ck(lib().bsamg_hier_reset(self.h), "bsamg_hier_reset")

    def set_box_sweep(self, kind):
        """Colour sweep of 3D periodic-box levels: 0 two rows a thread, 1
        four, 2 rows staged by bulk copies, 3 (default) one-pass V(2,2)
        smoothing where it applies (bsamg_set_box_sweep)."""
        _ck(lib().bsamg_set_box_sweep(self.h, int(kind)), "bsamg_set_box_sweep")

    def set_tail_cells(self, cells):
        """Largest cumulative coarse-level size the mixed V-cycle runs inside
        one thread block (bsamg_set_tail_cells; 0 disables)."""
        _ck(lib().bsamg_set_tail_cells(self.h, cells), "bsamg_set_tail_cells")

    def set_solve(self, mode=1, ctas=16, threads=512, tile=64, solo_cells=8192):
        """How a mixed-mode solve of an adaptive hierarchy runs
        (bsamg_set_solve): mode 1 as one launch of a cluster of `ctas` CTAs
        of `threads` threads, work lists in tiles of `tile` units, the levels
        holding at most `solo_cells` cells together run by one CTA; mode 0 as
        separate launches from captured graphs.  Both give the same iterates."""
        _ck(lib().bsamg_set_solve(self.h, int(mode), int(ctas), int(threads), int(tile), int(solo_cells)),
            "bsamg_set_solve")

    def get_solve(self):
        """(mode, ctas, threads, tile, solo_cells) of bsamg_set_solve."""
        m, c, t, g, s = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_longlong()
        _ck(lib().bsamg_get_solve(self.h, ctypes.byref(m), ctypes.byref(c), ctypes.byref(t), ctypes.byref(g),
                                  ctypes.byref(s)), "bsamg_get_solve")
        return m.value, c.value, t.value, g.value, s.value

    def solve_info(self):
        """dict of the last one-launch solve program (bsamg_solve_info)."""
        v = (ctypes.c_longlong * 11)()
        _ck(lib().bsamg_solve_info(self.h, v, 11), "bsamg_solve_info")
        keys = ("phases", "body", "dsm_levels", "data_bytes", "image_bytes", "ctas", "threads", "too_large",
                "build_us", "run_us", "readback_us")
        return dict(zip(keys, list(v)))

    def regrid_timing(self):
        """Host ms of the regrid that made this hierarchy (bsamg_regrid_timing):
        download, host model, create + commit, upload, ghost compilation, rest of commit, and the
        model's parts (ghost fill, tagging, edge-tag inflation, clustering, new patches, transfer)."""
        v = (ctypes.c_double * 12)()
        _ck(lib().bsamg_regrid_timing(self.h, v, 12), "bsamg_regrid_timing")
        return dict(zip(("download", "model", "commit", "upload", "ghost_compile", "commit_rest", "m_ghost",
                         "m_tag", "m_inflate", "m_cluster", "m_new", "m_transfer"), list(v)))

    def solve_trace(self, enable=True):
        """Record per-phase clocks of the next one-launch solves (bsamg_solve_trace)."""
        _ck(lib().bsamg_solve_trace(self.h, int(bool(enable))), "bsamg_solve_trace")

    def solve_trace_read(self):
        """[(op, n, cycles)] per phase of the last traced solve (bsamg_solve_trace_read)."""
        cnt = ctypes.c_int()
        _ck(lib().bsamg_solve_trace_read(self.h, 0, None, None, None, ctypes.byref(cnt)), "bsamg_solve_trace_read")
        k = cnt.value
        op, n, cy = (ctypes.c_int * max(k, 1))(), (ctypes.c_int * max(k, 1))(), (ctypes.c_longlong * max(k, 1))()
        _ck(lib().bsamg_solve_trace_read(self.h, k, op, n, cy, ctypes.byref(cnt)), "bsamg_solve_trace_read")
        return [(op[x], n[x], cy[x]) for x in range(k)]

    def graph_stats(self):
        """(graphs instantiated, graphs inherited and updated in place)."""
        a, b = ctypes.c_int(), ctypes.c_int()
        _ck(lib().bsamg_graph_stats(self.h, ctypes.byref(a), ctypes.byref(b)), "bsamg_graph_stats")
        return a.value, b.value

    def launch_count(self):
        n = ctypes.c_longlong()
        _ck(lib().bsamg_launch_count(self.h, ctypes.byref(n)), "bsamg_launch_count")
        return n.value


def format_f25(x):
    """One F25.12 field as the frame files hold it."""
    b = ctypes.create_string_buffer(26)
    _ck(lib().bsamg_format_f25_12(float(x), b), "bsamg_format_f25_12")
    return b.value.decode()


def format_stats_line(time, integral, meshsize):
    """One OUT/stats.dat record (newline included)."""
    b = ctypes.create_string_buffer(128)
    _ck(lib().bsamg_format_stats_line(time, _da(integral, 2), meshsize, b, 128), "bsamg_format_stats_line")
    return b.value.decode()


def pin(arr):
    """Page-lock a numpy array's memory (for fast put/get); returns arr."""
    _ck(lib().bsamg_host_register(arr.ctypes.data_as(ctypes.c_void_p), arr.nbytes), "bsamg_host_register")
    return arr


def unpin(arr):
    _ck(lib().bsamg_host_unregister(arr.ctypes.data_as(ctypes.c_void_p)), "bsamg_host_unregister")


def ch_residual_norm_noalloc(q_dev, f_dev, ndims, mx, h, dt, eps, norm_out_dev, errortype=1, stream=None):
    """Allocation-free ErrorAFAS of one CH patch on caller-owned device buffers
    (raw device addresses as ints); writes the norm to the device double at
    norm_out_dev.  See bsamg_ch_residual_norm_noalloc in include/bsamg.h."""
    _ck(lib().bsamg_ch_residual_norm_noalloc(ctypes.c_void_p(q_dev), ctypes.c_void_p(f_dev), ndims,
                                              _ia(list(mx) + [1] * (3 - len(mx)), 3), h, dt, eps, errortype,
                                              ctypes.c_void_p(norm_out_dev), ctypes.c_void_p(stream)),
        "bsamg_ch_residual_norm_noalloc")
