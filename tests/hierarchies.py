"""Patch hierarchies shared by the tests (the same list feeds the oracle and
the CUDA library).

AMR patches are derived from (parent, mbounds) with the reference's
MakeNewGrid rules (LIBRARY/bsamroutines.f90:1663-1784): mx = 2*(extent),
mglobal = 2*(parent mglobal + mbounds) - (1, 0), internal boundaries (999)
except where the patch touches a parent face with a physical or periodic
code, which it inherits.
"""
import math

INTERNAL = 999


def uniform(h, ndims, n, minlevel, mthbc, length=1.0):
    mx = [n] * ndims + [1] * (3 - ndims)
    h.build_uniform(mx, minlevel, mthbc, [0, 0, 0], [length if d < ndims else 1 for d in range(3)])


class Spec:
    """Host-side patch list with the reference's child rules."""

    def __init__(self, ndims):
        self.ndims = ndims
        self.patches = []  # dicts in insertion order

    def root_and_below(self, n, minlevel, mthbc, length=1.0):
        nd = self.ndims
        mx = [n] * nd + [1] * (3 - nd)
        dx = length / n
        mb_hi = [n // 2 if minlevel < 0 else n] * nd + [1] * (3 - nd)
        self._add(0, 0, 1 if minlevel < 0 else -1, mx, [1, n] * nd + [1, 1] * (3 - nd),
                  sum(([1, m] for m in mb_hi), []), mthbc, [dx] * nd + [0] * (3 - nd), [0.0] * 3)
        cur, d = n, dx
        for l in range(-1, minlevel - 1, -1):
            cur //= 2
            d *= 2
            hi = cur // 2 if l > minlevel else cur
            self._add(l, -l, -l + 1 if l > minlevel else -1, [cur] * nd + [1] * (3 - nd),
                      [1, cur] * nd + [1, 1] * (3 - nd), [1, hi] * nd + [1, 1] * (3 - nd), mthbc,
                      [d] * nd + [0] * (3 - nd), [0.0] * 3)

    def child(self, pid, cid, lo, hi):
        """child of patch pid covering parent cells lo..hi (1-based, inclusive)"""
        par = next(p for p in self.patches if p["id"] == pid)
        nd = self.ndims
        mx, mg, mb, thbc, xl = [1, 1, 1], [1, 1, 1, 1, 1, 1], [1, 1, 1, 1, 1, 1], [10] * 6, [0.0] * 3
        for d in range(nd):
            mx[d] = 2 * (hi[d] - lo[d] + 1)
            mb[2 * d], mb[2 * d + 1] = lo[d], hi[d]
            g0 = par["mglobal"][2 * d] + lo[d] - 1
            g1 = g0 + hi[d] - lo[d]
            mg[2 * d], mg[2 * d + 1] = (g0 - 1) * 2 + 1, g1 * 2
            xl[d] = (lo[d] - 1) * par["dx"][d] + par["xlower"][d]
        for d in range(nd):
            for s in range(2):
                thbc[2 * d + s] = INTERNAL
            if par["mthbc"][2 * d] < INTERNAL and lo[d] == 1:
                thbc[2 * d] = par["mthbc"][2 * d]
            if par["mthbc"][2 * d + 1] < INTERNAL and hi[d] == par["mx"][d]:
                thbc[2 * d + 1] = par["mthbc"][2 * d + 1]
        dx = [par["dx"][d] / 2 if d < nd else 0.0 for d in range(3)]
        self._add(par["level"] + 1, cid, pid, mx, mg, mb, thbc, dx, xl)

    def _add(self, level, id, parent, mx, mg, mb, thbc, dx, xl):
        self.patches.append(dict(level=level, id=id, parent_id=parent, mx=list(mx), mglobal=list(mg),
                                 mbounds=list(mb), mthbc=list(thbc), dx=list(dx), xlower=list(xl)))

    def apply(self, h):
        for p in self.patches:
            h.add_patch(p["level"], p["id"], p["parent_id"], p["mx"], p["mglobal"], p["mbounds"],
                        p["mthbc"], p["dx"], p["xlower"])
        h.commit()

    def finest(self):
        return max(p["level"] for p in self.patches)

    def minlevel(self):
        return min(p["level"] for p in self.patches)


def amr2d(periodic=True, n=32):
    """root n^2 + below-root levels + two refined levels with siblings that
    touch each other, the periodic boundary and each other's periodic images."""
    s = Spec(2)
    mthbc = [2, 2, 2, 2, 10, 10] if periodic else [10, 10, 10, 10, 10, 10]
    s.root_and_below(n, -int(math.log2(n)) + 1, mthbc)
    s.child(0, 101, [5, 5], [12, 10])      # 16 x 12
    s.child(0, 102, [13, 5], [20, 8])      # 16 x 8, sibling touching 101
    s.child(0, 103, [1, 20], [4, 27])      # touches the left boundary
    s.child(0, 104, [29, 20], [32, 27])    # touches the right boundary (image of 103)
    s.child(101, 201, [3, 3], [10, 8])     # level 2 inside 101
    s.child(101, 202, [11, 3], [14, 10])   # sibling of 201
    return s


def amr3d(periodic=True, n=16):
    """root n^3 + below-root levels + two refined levels in 3D: siblings that
    touch each other, the boundary, each other's periodic images, and a
    level-2 pair inside one level-1 patch."""
    s = Spec(3)
    mthbc = [2] * 6 if periodic else [10] * 6
    s.root_and_below(n, -int(math.log2(n)) + 1, mthbc)
    s.child(0, 101, [3, 3, 3], [8, 6, 7])        # 12 x 8 x 10
    s.child(0, 102, [9, 3, 3], [12, 6, 6])       # 8 x 8 x 8, touches 101 at x
    s.child(0, 103, [1, 10, 4], [4, 13, 7])      # touches the low-x boundary
    s.child(0, 104, [13, 10, 4], [16, 13, 7])    # touches the high-x boundary (image of 103)
    s.child(101, 201, [3, 3, 3], [6, 6, 6])      # level 2 inside 101
    s.child(101, 202, [7, 3, 2], [10, 6, 8])     # sibling of 201, 8 x 8 x 14
    return s
