"""The schedule of the one-pass V(2,2) smoothing (box.cu k_bx_smooth),
emulated on the CPU with the kernel's own index arithmetic.

The kernel streams z-planes through a ring of shared-memory slots and lets
four stages (colour half-sweeps 0, 1, 0, 1) lag one plane apart, with one
barrier per plane; each thread keeps the same four cells of one row in every
stage, carries the in-plane values of its last pass and forwards a stage's
results as the next stage's z+1 values in registers.  This test runs that
schedule thread by thread and checks, on boxes with wrapped halos, several
tiles and z ranges shorter than the halo:

* the result equals four plain half-sweeps of the same arithmetic (in FP64,
  so any difference would be a wrong operand, not rounding);
* every shared-memory access falls inside its slot, every output cell is
  written exactly once;
* between two barriers no location written by one thread is read or written
  by another, no thread reads a location before it was written in an
  earlier pass or by itself, and no slot is read while its bulk copy is in
  flight -- the conditions under which one barrier per plane is enough.
"""
import numpy as np
import pytest

NS = 4          # stages (half-sweeps) per pass
NSL = NS + 3    # slots of the plane ring
CPT = 4         # consecutive cells of a colour row per thread
CF = (0.3, 0.02, 0.1, 1.2)  # c0, c1, tmp3, a12


def newton(pb, xv, s0, s1, g0, g1):
    c0, c1, tmp3, a12 = CF
    w = pb + xv
    a21 = -3.0 * w * w - tmp3
    b1 = g0 + c0 * s1
    b2 = g1 - c1 * s0 - xv * xv * (3.0 * pb + 2.0 * xv)
    rdet = 1.0 / (1.0 - a12 * a21)
    return (b1 - a12 * b2) * rdet, (b2 - a21 * b1) * rdet


def four_sweeps(e, g, pb, fresh):
    """colour-split arrays e[2v+c][z][y][h]; the half-sweeps of relax_at"""
    e = e.copy()
    _, n2, n1, hh = e.shape
    z, y, h = np.meshgrid(np.arange(n2), np.arange(n1), np.arange(hh), indexing="ij")
    for s in range(1, NS + 1):
        c, o = (s - 1) & 1, 1 - ((s - 1) & 1)
        first = (s if s <= 2 else 0) if fresh else 0
        bb = (c + y + z + 1) & 1
        xm = np.where(bb == 1, h, (h - 1) % hh)
        xp = np.where(bb == 1, (h + 1) % hh, h)
        s0 = np.zeros(z.shape)
        s1 = np.zeros(z.shape)
        xv = np.zeros(z.shape)
        if first != 1:
            for v, acc in ((0, s0), (1, s1)):
                a = e[2 * v + o]
                t = a[z, y, xm] + a[z, y, xp] + a[z, (y - 1) % n1, h] + a[z, (y + 1) % n1, h]
                acc[...] = t + (a[(z - 1) % n2, y, h] + a[(z + 1) % n2, y, h])
            if first == 0:
                xv = e[c][z, y, h]
        r0, r1 = newton(pb[c], xv, s0, s1, g[c], g[2 + c])
        e[c], e[2 + c] = r0, r1
    return e


class Smem:
    """the ring with per-location write stamps and per-pass access logs"""

    def __init__(self, n):
        self.val = np.full(n, np.nan)
        self.w_it = np.full(n, -1, dtype=np.int64)
        self.w_th = np.full(n, -2, dtype=np.int64)
        self.log = []  # (locations, thread, is_write) of the current pass

    def read(self, loc, th, it, lo, hi):
        loc = np.asarray(loc)
        assert loc.min() >= lo and loc.max() < hi, "shared-memory read outside its slot"
        ok = (self.w_it[loc] < it) | (self.w_th[loc] == th)
        assert ok.all(), "read of a location another thread writes in the same pass"
        assert not np.isnan(self.val[loc]).any(), "read of a location never written"
        self.log.append((loc, th, False))
        return self.val[loc]

    def write(self, loc, v, th, it, lo, hi):
        loc = np.asarray(loc)
        assert loc.min() >= lo and loc.max() < hi, "shared-memory write outside its slot"
        self.val[loc] = v
        self.w_it[loc] = it
        self.w_th[loc] = th
        self.log.append((loc, th, True))

    def barrier(self):
        """no location written by one thread is accessed by another in the pass"""
        writers, readers = {}, {}
        for loc, th, wr in self.log:
            d = writers if wr else readers
            for x in np.atleast_1d(loc).tolist():
                d.setdefault(x, set()).add(th)
        for x, ws in writers.items():
            assert len(ws) == 1, "two threads write one location in a pass"
            assert readers.get(x, set()) <= ws, "a location read by one thread and written by another in a pass"
        self.log = []


def one_pass(e_in, g, pb, fresh, TY, nz, HH):
    """k_bx_smooth's schedule, thread by thread; returns the output e"""
    _, n2, n1, hh = e_in.shape
    assert hh == HH
    R = TY + 2 * NS
    AR = R * HH
    SL = 4 * AR
    W = HH // CPT
    NT = 2 * W * R  # as on the device, RK = NT / W rows between a thread's segments, even and >= R
    RK = NT // W
    assert RK % 2 == 0 and RK >= R
    out = np.full(e_in.shape, np.nan)
    written = np.zeros(e_in.shape, dtype=np.int64)
    ytiles = n1 // TY
    wrap = lambda v, n: v + n if v < 0 else (v - n if v >= n else v)
    for blk in range(ytiles * nz):
        y0 = (blk % ytiles) * TY
        zc = blk // ytiles
        z0, z1 = zc * n2 // nz, (zc + 1) * n2 // nz
        P = z1 - z0 + 2 * NS
        sm = Smem(NSL * SL)
        inflight = {}  # slot -> iteration during which its copy may land
        cz = {}        # (thread, stage) -> carried values of the other colour, two variables
        v = {}         # (thread, stage) -> pb, g0, g1 of the next pass

        def issue(j, k, it):
            if fresh or j >= P:
                return
            zw = wrap(z0 - NS + j, n2)
            for a in range(4):
                for r in range(R):
                    yy = wrap(y0 - NS + r, n1)
                    loc = k * SL + a * AR + r * HH + np.arange(HH)
                    sm.val[loc] = e_in[a, zw, yy, :]
                    sm.w_it[loc] = it  # lands before the wait at pass j; read only after it
                    sm.w_th[loc] = -1
            inflight[k] = j - 1  # the pass before that wait must not read the slot

        def load(s, j, th):
            if j < s or j > P - 1 - s:
                return
            rb, li = th // W, th % W
            r = rb
            if not (s <= r <= R - 1 - s):
                return
            c = (s - 1) & 1
            zw = wrap(z0 - NS + j, n2)
            yy = wrap(y0 - NS + r, n1)
            hs = CPT * li + np.arange(CPT)
            v[(th, s)] = (pb[c, zw, yy, hs], g[c, zw, yy, hs], g[2 + c, zw, yy, hs])

        issue(0, 0, -1)
        issue(1, 1, -1)
        for i in range(P):
            si = i % NSL
            slot = lambda d: (si - d) % NSL
            fw = {}
            for th in range(NT):
                for s in range(1, NS + 1):
                    j = i - s
                    if s <= j <= P - 1 - s:
                        c, o = (s - 1) & 1, 1 - ((s - 1) & 1)
                        first = (s if s <= 2 else 0) if fresh else 0
                        rb, li = th // W, th % W
                        r = rb
                        hc = CPT * li
                        if s <= r <= R - 1 - s:
                            z = z0 - NS + j
                            bb = (c + y0 - NS + rb + z + 1) & 1
                            S, Sm, Sp = slot(s) * SL, slot(s + 1) * SL, slot(s - 1) * SL
                            for k_ in (slot(s), slot(s + 1), slot(s - 1)):
                                assert inflight.get(k_) != i, "a slot read while its copy is in flight"
                            lim = lambda base: (base, base + SL)
                            s0 = np.zeros(CPT)
                            s1 = np.zeros(CPT)
                            xv = np.zeros(CPT)
                            if first != 1:
                                for var in range(2):
                                    ao = (2 * var + o) * AR + r * HH
                                    cells = ao + hc + np.arange(CPT)
                                    if j > s:
                                        a = cz[(th, s)][var]
                                    else:
                                        a = sm.read(S + cells, th, i, *lim(S))
                                    if s == 1:
                                        zp = sm.read(Sp + cells, th, i, *lim(Sp))
                                    else:
                                        zp = fw[(th, s - 1)][var]
                                    cz.setdefault((th, s), [None, None])[var] = zp
                                    zm = sm.read(Sm + cells, th, i, *lim(Sm))
                                    ym = sm.read(S + cells - HH, th, i, *lim(S))
                                    yp = sm.read(S + cells + HH, th, i, *lim(S))
                                    edge = sm.read(S + ao + ((hc + CPT) % HH if bb else (hc - 1) % HH), th, i, *lim(S))
                                    t = np.empty(CPT)
                                    for q in range(CPT):
                                        lft = a[q] if bb else (a[q - 1] if q else edge)
                                        rgt = (a[q + 1] if q + 1 < CPT else edge) if bb else a[q]
                                        t[q] = lft + rgt + ym[q] + yp[q]
                                        t[q] = t[q] + (zm[q] + zp[q])
                                    (s0 if var == 0 else s1)[:] = t
                                if first == 0:
                                    xv = sm.read(S + c * AR + r * HH + hc + np.arange(CPT), th, i, *lim(S))
                            pbv, g0, g1 = v[(th, s)]
                            r0, r1 = newton(pbv, xv, s0, s1, g0, g1)
                            fw[(th, s)] = (r0, r1)
                            sm.write(S + c * AR + r * HH + hc + np.arange(CPT), r0, th, i, *lim(S))
                            sm.write(S + (2 + c) * AR + r * HH + hc + np.arange(CPT), r1, th, i, *lim(S))
                    load(s, i + 1 - s, th)
            sm.barrier()
            inflight = {k: t for k, t in inflight.items() if t > i}
            issue(i + 2, slot(NSL - 2), i)
            j = i - NS
            if NS <= j <= P - 1 - NS:
                zz = z0 - NS + j
                base = slot(NS) * SL + NS * HH
                for a in range(4):
                    for rr in range(TY):
                        loc = base + a * AR + rr * HH + np.arange(HH)
                        vals = sm.val[loc]
                        assert not np.isnan(vals).any()
                        out[a, zz, y0 + rr, :] = vals
                        written[a, zz, y0 + rr, :] += 1
                sm.log = []  # the write-back reads final rows; the next writes to them come after later barriers
    assert (written == 1).all(), "every output cell written exactly once"
    return out


@pytest.mark.parametrize("shape,TY,nz", [((8, 16, 8), 8, 1), ((8, 24, 12), 8, 2), ((8, 16, 20), 8, 3)])
@pytest.mark.parametrize("fresh", [False, True])
def test_one_pass_schedule_equals_four_sweeps(shape, TY, nz, fresh):
    n2, n1, hh = shape
    rng = np.random.default_rng(n2 * 100 + n1 + hh)
    e = rng.standard_normal((4, n2, n1, hh)) * 1e-2
    g = rng.standard_normal((4, n2, n1, hh)) * 1e-3
    pb = rng.standard_normal((2, n2, n1, hh)) * 0.5
    want = four_sweeps(e, g, pb, fresh)
    got = one_pass(e, g, pb, fresh, TY, nz, hh)
    assert np.array_equal(want, got)
