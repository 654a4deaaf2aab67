"""ctypes view of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py
import this module.  The method names mirror the CUDA library's Python host
class (bsam1.2_gb300.Hierarchy) so a parity test can drive both the same way.
"""
import ctypes
import os

import numpy as np

from .build import build_oracle  # noqa: F401  (package-relative when imported as oracle.*)

FIELD = {"q": 0, "qold": 1, "qc": 2, "f": 3, "rf": 4, "ftmp": 5}
PROBLEM = {"ch": 1, "biogrowth": 2, "growth": 3}

_lib = None


class RegridParams(ctypes.Structure):
    """bsamo_regrid_params (the same layout as bsamg_regrid_params)."""
    _fields_ = [("maxlevel", ctypes.c_int), ("tagging", ctypes.c_int), ("initial", ctypes.c_int),
                ("maxside", ctypes.c_int), ("first_id", ctypes.c_int), ("ibuffer", ctypes.c_int * 11),
                ("minimumgridpoints", ctypes.c_int * 11), ("qtolerance", ctypes.c_double * 11),
                ("desiredfillratio", ctypes.c_double * 11)]


TAGGING = {"ch": 0, "gradient": 1}
QINIT = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                         ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                         ctypes.POINTER(ctypes.c_double))


def regrid_params(maxlevel, tagging="ch", initial=False, maxside=0, first_id=1000, ibuffer=1,
                  minimumgridpoints=4, qtolerance=1e-2, desiredfillratio=0.9):
    """RegridParams with one value for every level (lists are taken per level)."""
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


def make_qinit(fn, ndims, nrvars, mbc=1):
    """C callback around fn(level, mx, dx, xlower) -> ghosted Fortran-layout
    array of the new patch (only its interior is used), with mbc ghost
    layers or one (then placed at q(0:mx+1), the second layer zero)."""
    def cb(user, level, mx, dx, xl, q):
        m = [mx[d] for d in range(ndims)]
        a = np.asarray(fn(level, m, [dx[d] for d in range(3)][:ndims], [xl[d] for d in range(3)][:ndims]),
                       dtype=np.float64).ravel(order="F")
        full = int(np.prod([v + 2 * mbc for v in m])) * nrvars
        if a.size != full:
            assert a.size == int(np.prod([v + 2 for v in m])) * nrvars, (a.size, full)
            out = np.zeros([v + 2 * mbc for v in m] + [nrvars], order="F")
            g = mbc - 1
            out[tuple(slice(g, g + v + 2) for v in m) + (slice(None),)] = a.reshape([v + 2 for v in m] + [nrvars],
                                                                                   order="F")
            a = out.ravel(order="F")
        ctypes.memmove(q, a.ctypes.data, full * 8)
    return QINIT(cb)


def lib():
    global _lib
    if _lib is None:
        path = build_oracle()
        L = ctypes.CDLL(path)
        I, D, P = ctypes.c_int, ctypes.c_double, ctypes.c_void_p
        IP = ctypes.POINTER(ctypes.c_int)
        DP = ctypes.POINTER(ctypes.c_double)
        L.bsamo_create.argtypes = [I, I, I, I, DP, I, DP, ctypes.POINTER(P)]
        L.bsamo_destroy.argtypes = [P]
        L.bsamo_patch_add.argtypes = [P, I, I, I, IP, IP, IP, IP, DP, DP]
        L.bsamo_build_uniform.argtypes = [P, IP, I, IP, DP, DP]
        L.bsamo_commit.argtypes = [P]
        L.bsamo_num_patches.argtypes = [P]
        L.bsamo_patch_info.argtypes = [P, I, IP, DP]
        L.bsamo_field_size.argtypes = [P, I, I]
        L.bsamo_field_size.restype = ctypes.c_size_t
        L.bsamo_put_field.argtypes = [P, I, I, DP, ctypes.c_size_t]
        L.bsamo_get_field.argtypes = [P, I, I, DP, ctypes.c_size_t]
        L.bsamo_relax_level_color.argtypes = [P, I, I]
        L.bsamo_set_ghost.argtypes = [P, I, I]
        L.bsamo_level_relax.argtypes = [P, I, I]
        L.bsamo_fill_down.argtypes = [P, I, I, I]
        L.bsamo_copy_q_to_qold.argtypes = [P, I, I]
        L.bsamo_vcycle.argtypes = [P, I, I, I]
        L.bsamo_correct_fine.argtypes = [P, I]
        L.bsamo_level_op.argtypes = [P, I, I]
        L.bsamo_new_sub_grids.argtypes = [I, IP, IP, D, I, IP, I]
        L.bsamo_prolong_mc.argtypes = [I, I, DP, IP, DP]
        L.bsamo_residual_norm.argtypes = [P, I, I, DP]
        L.bsamo_multigrid_iterations.argtypes = [P, I, I, I, I, D, I, I, IP, DP]
        L.bsamo_time_step.argtypes = [P, I, I, I, I, I, D, I, I, IP, DP]
        L.bsamo_regrid.argtypes = [P, ctypes.POINTER(RegridParams), QINIT, P, ctypes.POINTER(P)]
        L.bsamo_after_step_stats.argtypes = [P, I, DP, ctypes.POINTER(ctypes.c_longlong)]
        L.bsamo_write_q.argtypes = [P, ctypes.c_char_p, D, I]
        L.bsamo_write_uniform_q.argtypes = [P, ctypes.c_char_p, D, I]
        L.bsamo_read_q.argtypes = [P, ctypes.c_char_p, I, DP, ctypes.POINTER(P)]
        L.bsamo_format_f25_12.argtypes = [D, ctypes.c_char_p]
        L.bsamo_format_f25_12.restype = None
        L.bsamo_format_stats_line.argtypes = [D, DP, ctypes.c_longlong, ctypes.c_char_p, ctypes.c_size_t]
        L.bsamo_uniform_pm1.argtypes = [ctypes.c_ulonglong, ctypes.c_ulonglong]
        L.bsamo_uniform_pm1.restype = D
        _lib = L
    return _lib


def _ia(x, n):
    a = (ctypes.c_int * n)(*[int(v) for v in x])
    return a


def _da(x, n):
    return (ctypes.c_double * n)(*[float(v) for v in x])


def _check(rc, what):
    if rc != 0:
        raise RuntimeError(f"oracle {what} failed with status {rc}")


class OracleHierarchy:
    """A patch hierarchy held by the CPU oracle."""

    def __init__(self, ndims, nrvars, problem, params, qpo=None, mbc=1):
        L = lib()
        self.ndims, self.nrvars, self.mbc = ndims, nrvars, mbc
        h = ctypes.c_void_p()
        p = _da(params, len(params))
        q = _da(qpo if qpo is not None else [0.0] * nrvars, nrvars)
        _check(L.bsamo_create(ndims, nrvars, mbc, PROBLEM[problem], p, len(params), q,
                              ctypes.byref(h)), "create")
        self.h = h
        self.patches = []

    def __del__(self):
        if getattr(self, "h", None):
            lib().bsamo_destroy(self.h)
            self.h = None

    def add_patch(self, level, id, parent_id, mx, mglobal, mbounds, mthbc, dx, xlower):
        _check(lib().bsamo_patch_add(self.h, level, id, parent_id, _ia(mx, 3), _ia(mglobal, 6),
                                     _ia(mbounds, 6), _ia(mthbc, 6), _da(dx, 3),
                                     _da(xlower, 3)), "patch_add")

    def build_uniform(self, mx, minlevel, mthbc, xlower, xupper):
        _check(lib().bsamo_build_uniform(self.h, _ia(mx, 3), minlevel, _ia(mthbc, 6),
                                         _da(xlower, 3), _da(xupper, 3)), "build_uniform")

    def commit(self):
        _check(lib().bsamo_commit(self.h), "commit")

    def patch_table(self):
        L = lib()
        out = []
        for n in range(L.bsamo_num_patches(self.h)):
            a = (ctypes.c_int * 28)()
            d = (ctypes.c_double * 6)()
            _check(L.bsamo_patch_info(self.h, n, a, d), "patch_info")
            a = list(a)
            out.append(dict(level=a[0], id=a[1], parent_id=a[2], mx=a[3:6], mglobal=a[6:12],
                            mbounds=a[12:18], mthbc=a[18:24], dx=list(d)[0:3],
                            xlower=list(d)[3:6]))
        return out

    def level_range(self):
        """(minlevel, finest level), as the library's bsamg_level_range."""
        levels = [p["level"] for p in self.patch_table()]
        return min(levels), max(levels)

    def field_size(self, pid, field):
        return lib().bsamo_field_size(self.h, pid, FIELD[field])

    def put(self, pid, field, arr):
        a = np.ascontiguousarray(np.asarray(arr, dtype=np.float64).ravel(order="F"))
        _check(lib().bsamo_put_field(self.h, pid, FIELD[field],
                                     a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), a.size),
               "put_field")

    def get(self, pid, field):
        n = self.field_size(pid, field)
        a = np.empty(n, dtype=np.float64)
        _check(lib().bsamo_get_field(self.h, pid, FIELD[field],
                                     a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), n),
               "get_field")
        return a

    def relax_level_color(self, level, ipass):
        _check(lib().bsamo_relax_level_color(self.h, level, ipass), "relax")

    def set_ghost(self, level, ipass):
        _check(lib().bsamo_set_ghost(self.h, level, ipass), "set_ghost")

    def level_relax(self, level, nsmooth):
        _check(lib().bsamo_level_relax(self.h, level, nsmooth), "level_relax")

    def fill_down(self, field, finest, minlevel):
        _check(lib().bsamo_fill_down(self.h, {"f": 1, "q": 2}[field], finest, minlevel), "fill_down")

    def copy_q_to_qold(self, minlevel, finest):
        _check(lib().bsamo_copy_q_to_qold(self.h, minlevel, finest), "copy_q_to_qold")

    def vcycle(self, level, minlevel, nsmooth):
        _check(lib().bsamo_vcycle(self.h, level, minlevel, nsmooth), "vcycle")

    def correct_fine(self, level):
        _check(lib().bsamo_correct_fine(self.h, level), "correct_fine")

    def level_op(self, level, which):
        """a per-patch operation on every patch of a level: "restrict",
        "coarse_ghost", "coarse_load", "get_source", "update_source",
        "fill_f", "fill_q" (FillDownLevel of f or q)"""
        code = {"restrict": 1, "coarse_ghost": 2, "coarse_load": 3, "get_source": 4, "update_source": 5,
                "fill_f": 6, "fill_q": 7}[which]
        _check(lib().bsamo_level_op(self.h, level, code), "level_op")

    def residual_norm(self, level, errortype=1):
        r = ctypes.c_double()
        _check(lib().bsamo_residual_norm(self.h, level, errortype, ctypes.byref(r)), "resid")
        return r.value

    def multigrid_iterations(self, finest, minlevel, nsmooth=2, maxvcycles=20, tol=1e-9,
                             updateauxfreq=1, errortype=1):
        n = ctypes.c_int()
        res = (ctypes.c_double * maxvcycles)()
        _check(lib().bsamo_multigrid_iterations(self.h, finest, minlevel, nsmooth, maxvcycles,
                                                tol, updateauxfreq, errortype, ctypes.byref(n),
                                                res), "multigrid_iterations")
        return n.value, list(res)[: n.value]

    def time_step(self, first, finest, minlevel, nsmooth=2, maxvcycles=20, tol=1e-9,
                  updateauxfreq=1, errortype=1):
        n = ctypes.c_int()
        res = (ctypes.c_double * maxvcycles)()
        _check(lib().bsamo_time_step(self.h, int(bool(first)), finest, minlevel, nsmooth,
                                     maxvcycles, tol, updateauxfreq, errortype, ctypes.byref(n),
                                     res), "time_step")
        return n.value, list(res)[: n.value]

    def after_step_stats(self, finest):
        """(integral of phi, CH 2D energy, composite mesh size)."""
        r = (ctypes.c_double * 2)()
        m = ctypes.c_longlong()
        _check(lib().bsamo_after_step_stats(self.h, finest, r, ctypes.byref(m)), "after_step_stats")
        return r[0], r[1], m.value

    def write_q(self, path, time, finest):
        _check(lib().bsamo_write_q(self.h, os.fsencode(path), time, finest), "write_q")

    def write_uniform_q(self, path, time, finest):
        _check(lib().bsamo_write_uniform_q(self.h, os.fsencode(path), time, finest), "write_uniform_q")


def read_q(root, path, first_id=1000):
    """Restart from a frame file (bsamo_read_q); returns (hierarchy, time)."""
    h = ctypes.c_void_p()
    t = ctypes.c_double()
    _check(lib().bsamo_read_q(root.h, os.fsencode(path), first_id, ctypes.byref(t), ctypes.byref(h)), "read_q")
    return _wrap(h, root.ndims, root.nrvars, root.mbc), t.value


def format_f25(x):
    b = ctypes.create_string_buffer(26)
    lib().bsamo_format_f25_12(float(x), b)
    return b.value.decode()


def format_stats_line(time, integral, meshsize):
    b = ctypes.create_string_buffer(128)
    _check(lib().bsamo_format_stats_line(time, _da(integral, 2), meshsize, b, 128), "format_stats_line")
    return b.value.decode()


def _wrap(h, ndims, nrvars, mbc=1):
    o = OracleHierarchy.__new__(OracleHierarchy)
    o.h, o.ndims, o.nrvars, o.mbc, o.patches = h, ndims, nrvars, mbc, []
    return o


def regrid(old, params, qinit=None):
    """AMR regrid of an oracle hierarchy (bsamo_regrid); returns a new one."""
    cb = make_qinit(qinit, old.ndims, old.nrvars, old.mbc) if qinit is not None else QINIT()
    h = ctypes.c_void_p()
    _check(lib().bsamo_regrid(old.h, ctypes.byref(params), cb, None, ctypes.byref(h)), "regrid")
    return _wrap(h, old.ndims, old.nrvars, old.mbc)


def new_sub_grids(flags, desfill, mgp):
    """NewSubGrids on one patch's flags (a 2D or 3D int array): the boxes
    [(lo, hi) per dimension] in the order the oracle makes them"""
    f = np.asfortranarray(np.asarray(flags, dtype=np.int32))
    nd = f.ndim
    mx = list(f.shape) + [1] * (3 - nd)
    cap = 4096
    out = (ctypes.c_int * (6 * cap))()
    n = lib().bsamo_new_sub_grids(nd, (ctypes.c_int * 3)(*mx), f.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                  desfill, mgp, out, cap)
    _check(0 if n >= 0 else n, "new_sub_grids")
    return [[(out[6 * g + 2 * d], out[6 * g + 2 * d + 1]) for d in range(nd)] for g in range(n)]


def prolong_mc(a, mbc):
    """P1MC / P2MC of one variable (bsamo_prolong_mc): a is the coarse
    block with mbc ghost layers (Fortran order), the result the fine block."""
    a = np.asarray(a, dtype=np.float64)
    nd = a.ndim
    cmx = [n - 2 * mbc for n in a.shape] + [1] * (3 - nd)
    out = np.zeros([2 * c + 2 * mbc for c in cmx[:nd]], order="F")
    src = np.asfortranarray(a)
    _check(lib().bsamo_prolong_mc(nd, mbc, src.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                  (ctypes.c_int * 3)(*cmx), out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))),
           "prolong_mc")
    return out


def uniform_pm1(seed, gidx):
    return lib().bsamo_uniform_pm1(seed, gidx)
