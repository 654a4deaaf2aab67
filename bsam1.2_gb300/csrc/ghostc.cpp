// Ghost-program compiler.
//
// SetGhost (LIBRARY/boundary.f90:67-97) fills the ghost ring of every patch
// of a level by a fixed sequence of writers: coarse-fine interpolation
// (colour-selective), sibling copies (ApplyOnLevelPairs(TransferBC)),
// self-periodic copies, periodic-image copies, then the plugin's physical
// boundary condition.  Later writers overwrite earlier ones, and some writers
// read ghost cells written earlier in the same sequence (for example the
// bottom-face boundary condition reads the left-face ghost column).
//
// Instead of walking patch pairs on every call (the reference's O(P^2) pair
// loops), the host emits the whole write sequence once per (level, ipass)
// after a regrid, removes writes that are overwritten before anything reads
// them, and groups the rest into stages such that no two operations of a
// stage touch the same cell in a conflicting way.  Executing the stages in
// order on the device gives exactly the state the sequential sequence gives.
#include <algorithm>
#include <cstdint>
#include <iterator>
#include <memory>
#include <unordered_map>

#include "hier.h"

namespace bsamg {

namespace {

struct Em {
  GhostOp op;
  int64_t dst;
  int64_t src[2];
  int nsrc;
};

struct Emitter {
  const Hier& H;
  std::vector<Em> out;
  const std::vector<int>& org;  // per patch: offset of cell (0,0,0) in its q plane
  Emitter(const Hier& h, const std::vector<int>& o) : H(h), org(o) {}

  // offset of Fortran cell (i,j,k) from cell (0,0,0) of a q plane (the
  // device tables address q from that cell; negative in the second ghost
  // layer when mbc = 2)
  int cell(int p, int i, int j, int k) const {
    const HostPatch& P = H.patches[p];
    if (H.ndims == 2) return j * P.qn[0] + i;
    return (k * P.qn[1] + j) * P.qn[0] + i;
  }
  // (patch, cell) key; the cell counted from the array's start (>= 0)
  int64_t key(int p, int c) const {
    return ((int64_t)p << 32) | (uint32_t)(c + org[p]);
  }

  void copy(int type, int dp, int dc, int sp, int sc) {
    Em e{};
    e.op.type = type;
    e.op.dp = dp;
    e.op.dcell = dc;
    e.op.sp = sp;
    e.op.s0 = sc;
    e.dst = key(dp, dc);
    e.src[0] = key(sp, sc);
    e.nsrc = 1;
    out.push_back(e);
  }
  void bc(int dp, int dc, int sc, int mask) {
    Em e{};
    e.op.type = kGBC;
    e.op.dp = dp;
    e.op.dcell = dc;
    e.op.sp = dp;
    e.op.s0 = sc;
    e.op.mask = mask;
    e.dst = key(dp, dc);
    e.src[0] = key(dp, sc);
    e.nsrc = 1;
    out.push_back(e);
  }
  // a1*f(s0) + a2*f(s1) + a3*(coarse combination)
  void cf(int type, int dp, int dc, int s0, int s1, int cp, int c0, int c1 = 0, int c2 = 0, int c3 = 0) {
    Em e{};
    e.op.type = type;
    e.op.dp = dp;
    e.op.dcell = dc;
    e.op.sp = cp;
    e.op.s0 = s0;
    e.op.s1 = s1;
    e.op.c0 = c0;
    e.op.c1 = c1;
    e.op.c2 = c2;
    e.op.c3 = c3;
    e.dst = key(dp, dc);
    e.src[0] = key(dp, s0);
    e.src[1] = key(dp, s1);
    e.nsrc = 2;  // parent cells live on another level: never written here
    out.push_back(e);
  }

  // Interpolate2D, boundary.f90:143-333 (same statement order)
  void interpolate2d(int f, int ipass) {
    const HostPatch& F = H.patches[f];
    int c = F.parent;
    int mx1 = F.mx[0], mx2 = F.mx[1];
    int mb11 = F.mbounds[0][0], mb12 = F.mbounds[0][1];
    int mb21 = F.mbounds[1][0], mb22 = F.mbounds[1][1];
    const int* m = F.mthbc;
    auto fq = [&](int i, int j) { return cell(f, i, j, 0); };
    auto cq = [&](int i, int j) { return cell(c, i, j, 0); };
    if (ipass == 1 || ipass == 0) {
      cf(kGCfA, f, fq(mx1 + 1, mx2 + 1), fq(mx1 - 1, mx2 - 1), fq(mx1, mx2), c, cq(mb12 + 1, mb22 + 1));
      cf(kGCfA, f, fq(0, 0), fq(2, 2), fq(1, 1), c, cq(mb11 - 1, mb21 - 1));
    }
    if (ipass == 2 || ipass == 0) {
      cf(kGCfA, f, fq(mx1 + 1, 0), fq(mx1 - 1, 2), fq(mx1, 1), c, cq(mb12 + 1, mb21 - 1));
      cf(kGCfA, f, fq(0, mx2 + 1), fq(2, mx2 - 1), fq(1, mx2), c, cq(mb11 - 1, mb22 + 1));
    }
    if (m[0] == 2 || m[0] == kInternalBC) {
      if (ipass == 1 || ipass == 0) {
        for (int j = 2, n = 0; j <= mx2 - 2; j += 2, n++)
          cf(kGCfA, f, fq(0, j), fq(2, j + 2), fq(1, j + 1), c, cq(mb11 - 1, mb21 + n));
        cf(kGCfAB, f, fq(0, mx2), fq(2, mx2), fq(1, mx2), c, cq(mb11 - 1, mb22 + 1), cq(mb11 - 1, mb22),
           cq(mb11 - 1, mb22 - 1));
      }
      if (ipass == 2 || ipass == 0) {
        for (int j = 3, n = 0; j <= mx2 - 1; j += 2, n++)
          cf(kGCfA, f, fq(0, j), fq(2, j - 2), fq(1, j - 1), c, cq(mb11 - 1, mb21 + 1 + n));
        cf(kGCfAB, f, fq(0, 1), fq(2, 1), fq(1, 1), c, cq(mb11 - 1, mb21 - 1), cq(mb11 - 1, mb21),
           cq(mb11 - 1, mb21 + 1));
      }
    }
    if (m[1] == 2 || m[1] == kInternalBC) {
      if (ipass == 1 || ipass == 0) {
        for (int j = 3, n = 0; j <= mx2 - 1; j += 2, n++)
          cf(kGCfA, f, fq(mx1 + 1, j), fq(mx1 - 1, j - 2), fq(mx1, j - 1), c, cq(mb12 + 1, mb21 + 1 + n));
        cf(kGCfAB, f, fq(mx1 + 1, 1), fq(mx1 - 1, 1), fq(mx1, 1), c, cq(mb12 + 1, mb21 - 1), cq(mb12 + 1, mb21),
           cq(mb12 + 1, mb21 + 1));
      }
      if (ipass == 2 || ipass == 0) {
        for (int j = 2, n = 0; j <= mx2 - 2; j += 2, n++)
          cf(kGCfA, f, fq(mx1 + 1, j), fq(mx1 - 1, j + 2), fq(mx1, j + 1), c, cq(mb12 + 1, mb21 + n));
        cf(kGCfAB, f, fq(mx1 + 1, mx2), fq(mx1 - 1, mx2), fq(mx1, mx2), c, cq(mb12 + 1, mb22 + 1),
           cq(mb12 + 1, mb22), cq(mb12 + 1, mb22 - 1));
      }
    }
    if (m[2] == 2 || m[2] == kInternalBC) {
      if (ipass == 1 || ipass == 0) {
        for (int i = 2, n = 0; i <= mx1 - 2; i += 2, n++)
          cf(kGCfA, f, fq(i, 0), fq(i + 2, 2), fq(i + 1, 1), c, cq(mb11 + n, mb21 - 1));
        cf(kGCfAB, f, fq(mx1, 0), fq(mx1, 2), fq(mx1, 1), c, cq(mb12 + 1, mb21 - 1), cq(mb12, mb21 - 1),
           cq(mb12 - 1, mb21 - 1));
      }
      if (ipass == 2 || ipass == 0) {
        for (int i = 3, n = 0; i <= mx1 - 1; i += 2, n++)
          cf(kGCfA, f, fq(i, 0), fq(i - 2, 2), fq(i - 1, 1), c, cq(mb11 + 1 + n, mb21 - 1));
        cf(kGCfAB, f, fq(1, 0), fq(1, 2), fq(1, 1), c, cq(mb11 - 1, mb21 - 1), cq(mb11, mb21 - 1),
           cq(mb11 + 1, mb21 - 1));
      }
    }
    if (m[3] == 2 || m[3] == kInternalBC) {
      if (ipass == 1 || ipass == 0) {
        for (int i = 3, n = 0; i <= mx1 - 1; i += 2, n++)
          cf(kGCfA, f, fq(i, mx2 + 1), fq(i - 2, mx2 - 1), fq(i - 1, mx2), c, cq(mb11 + 1 + n, mb22 + 1));
        cf(kGCfAB, f, fq(1, mx2 + 1), fq(1, mx2 - 1), fq(1, mx2), c, cq(mb11 - 1, mb22 + 1), cq(mb11, mb22 + 1),
           cq(mb11 + 1, mb22 + 1));
      }
      if (ipass == 2 || ipass == 0) {
        for (int i = 2, n = 0; i <= mx1 - 2; i += 2, n++)
          cf(kGCfA, f, fq(i, mx2 + 1), fq(i + 2, mx2 - 1), fq(i + 1, mx2), c, cq(mb11 + n, mb22 + 1));
        cf(kGCfAB, f, fq(mx1, mx2 + 1), fq(mx1, mx2 - 1), fq(mx1, mx2), c, cq(mb12 + 1, mb22 + 1),
           cq(mb12, mb22 + 1), cq(mb12 - 1, mb22 + 1));
      }
    }
  }

  // GetFaceIndex, boundary.f90:1018-1045: [0] ghost index, [1] second fine
  // cell, [2] first fine cell, [3] parent cell beyond the patch, [4] parent
  // cell at the patch edge, for the low (parity 1) or high (2) side of d.
  void face_index(const HostPatch& F, int d, int parity, int fi[5]) const {
    if (parity == 1) {
      fi[0] = 0, fi[1] = 2, fi[2] = 1, fi[3] = F.mbounds[d][0] - 1, fi[4] = F.mbounds[d][0];
    } else {
      fi[0] = F.mx[d] + 1, fi[1] = F.mx[d] - 1, fi[2] = F.mx[d], fi[3] = F.mbounds[d][1] + 1,
      fi[4] = F.mbounds[d][1];
    }
  }
  // one 3D interpolated ghost cell; kind 0: kGCfA, 1: kGCfAB, 2: kGCfAC
  void cf3(int f, int c, int kind, const int* g, const int* s1, const int* s2, const int (*cc)[3]) {
    static const int types[3] = {kGCfA, kGCfAB, kGCfAC};
    int nc = kind == 0 ? 1 : kind == 1 ? 3 : 4;
    int co[4] = {0, 0, 0, 0};
    for (int x = 0; x < nc; x++) co[x] = cell(c, cc[x][0], cc[x][1], cc[x][2]);
    cf(types[kind], f, cell(f, g[0], g[1], g[2]), cell(f, s1[0], s1[1], s1[2]), cell(f, s2[0], s2[1], s2[2]), c,
       co[0], co[1], co[2], co[3]);
  }
  // an edge: dimensions d1, d2 fixed by the face indices fa, fb; t runs
  // (the four statements of each edge group, boundary.f90:1107-1126)
  void cf3_edge(int f, int c, int d1, const int* fa, int d2, const int* fb, int t) {
    const HostPatch& F = H.patches[f];
    int mx = F.mx[t], lo = F.mbounds[t][0], hi = F.mbounds[t][1];
    int g[3], s1[3], s2[3], cc[4][3];
    g[d1] = fa[0], s1[d1] = fa[1], s2[d1] = fa[2];
    g[d2] = fb[0], s1[d2] = fb[1], s2[d2] = fb[2];
    for (int x = 0; x < 4; x++) cc[x][d1] = fa[3], cc[x][d2] = fb[3];
    for (int i = 3, n = 0; i <= mx - 1; i += 2, n++) {
      g[t] = i, s1[t] = i - 2, s2[t] = i - 1, cc[0][t] = lo + 1 + n;
      cf3(f, c, 0, g, s1, s2, cc);
    }
    g[t] = s1[t] = s2[t] = 1;
    cc[0][t] = lo - 1, cc[1][t] = lo, cc[2][t] = lo + 1;
    cf3(f, c, 1, g, s1, s2, cc);
    for (int i = 2, n = 0; i <= mx - 2; i += 2, n++) {
      g[t] = i, s1[t] = i + 2, s2[t] = i + 1, cc[0][t] = lo + n;
      cf3(f, c, 0, g, s1, s2, cc);
    }
    g[t] = s1[t] = s2[t] = mx;
    cc[0][t] = hi + 1, cc[1][t] = hi, cc[2][t] = hi - 1;
    cf3(f, c, 1, g, s1, s2, cc);
  }
  // one colour class of a face with normal n (index fn) and tangential
  // dimensions t1 < t2.  cls 0 yellow (t1, t2 even), 1 blue (odd, odd),
  // 2 green (odd, even), 3 red (even, odd); each is its strided bulk and its
  // two edge rows, where the parent value is a b-combination along the
  // dimension that sits at its end (boundary.f90:1236-1320 and analogues).
  void cf3_face_class(int f, int c, int n, const int* fn, int t1, int t2, int cls) {
    const HostPatch& F = H.patches[f];
    int m1 = F.mx[t1], m2 = F.mx[t2];
    int l1 = F.mbounds[t1][0], h1 = F.mbounds[t1][1], l2 = F.mbounds[t2][0], h2 = F.mbounds[t2][1];
    int g[3], s1[3], s2[3], cc[4][3];
    g[n] = fn[0], s1[n] = fn[1], s2[n] = fn[2];
    for (int x = 0; x < 4; x++) cc[x][n] = fn[3];
    bool e1 = cls == 0 || cls == 3, e2 = cls == 0 || cls == 2;
    int a1lo = e1 ? 2 : 3, a1hi = e1 ? m1 - 2 : m1 - 1, a2lo = e2 ? 2 : 3, a2hi = e2 ? m2 - 2 : m2 - 1;
    int d1 = e1 ? 1 : -1, d2 = e2 ? 1 : -1;
    auto par1 = [&](int i) { return e1 ? l1 + i / 2 - 1 : l1 + (i - 1) / 2; };
    auto par2 = [&](int j) { return e2 ? l2 + j / 2 - 1 : l2 + (j - 1) / 2; };
    for (int j = a2lo; j <= a2hi; j += 2)
      for (int i = a1lo; i <= a1hi; i += 2) {
        g[t1] = i, g[t2] = j;
        s1[t1] = i + 2 * d1, s1[t2] = j + 2 * d2;
        s2[t1] = i + d1, s2[t2] = j + d2;
        cc[0][t1] = par1(i), cc[0][t2] = par2(j);
        cf3(f, c, 0, g, s1, s2, cc);
      }
    for (int j = a2lo; j <= a2hi; j += 2) {
      int i = e1 ? m1 : 1;
      g[t1] = s1[t1] = s2[t1] = i;
      g[t2] = j, s1[t2] = j + 2 * d2, s2[t2] = j + d2;
      for (int x = 0; x < 3; x++) cc[x][t2] = par2(j);
      if (e1) cc[0][t1] = h1 + 1, cc[1][t1] = h1, cc[2][t1] = h1 - 1;
      else cc[0][t1] = l1 - 1, cc[1][t1] = l1, cc[2][t1] = l1 + 1;
      cf3(f, c, 1, g, s1, s2, cc);
    }
    for (int i = a1lo; i <= a1hi; i += 2) {
      int j = e2 ? m2 : 1;
      g[t2] = s1[t2] = s2[t2] = j;
      g[t1] = i, s1[t1] = i + 2 * d1, s2[t1] = i + d1;
      for (int x = 0; x < 3; x++) cc[x][t1] = par1(i);
      if (e2) cc[0][t2] = h2 + 1, cc[1][t2] = h2, cc[2][t2] = h2 - 1;
      else cc[0][t2] = l2 - 1, cc[1][t2] = l2, cc[2][t2] = l2 + 1;
      cf3(f, c, 1, g, s1, s2, cc);
    }
  }
  // the four grey corner cells of a face, written on every pass
  // (boundary.f90:1322-1333 and analogues)
  void cf3_face_grey(int f, int c, int n, const int* fn, int t1, int t2) {
    const HostPatch& F = H.patches[f];
    for (int p1 = 1; p1 <= 2; p1++) {
      int fa[5];
      face_index(F, t1, p1, fa);
      for (int p2 = 1; p2 <= 2; p2++) {
        int fb[5];
        face_index(F, t2, p2, fb);
        int g[3], s1[3], s2[3], cc[4][3];
        g[n] = fn[0], s1[n] = fn[1], s2[n] = fn[2];
        g[t1] = s1[t1] = s2[t1] = fa[2];
        g[t2] = s1[t2] = s2[t2] = fb[2];
        for (int x = 0; x < 4; x++) cc[x][n] = fn[3];
        cc[0][t1] = fa[4], cc[0][t2] = fb[4];
        cc[1][t1] = fa[3], cc[1][t2] = fb[4];
        cc[2][t1] = fa[4], cc[2][t2] = fb[3];
        cc[3][t1] = fa[3], cc[3][t2] = fb[3];
        cf3(f, c, 2, g, s1, s2, cc);
      }
    }
  }

  // Interpolate3D, boundary.f90:1048-1550: corners, the twelve edges, then
  // the six faces.  Corners and edges skip non-interface faces on pass 1
  // only; the face-5/6 test of edges 1-4 compares with 99 where every other
  // test compares with 999 (boundary.f90:1104), kept as the reference has it.
  void interpolate3d(int f, int ipass) {
    const HostPatch& F = H.patches[f];
    int c = F.parent;
    const int* m = F.mthbc;
    auto iface = [](int v) { return v == 2 || v == 999; };
    int fa[5], fb[5], fc[5];
    for (int p1 = 1; p1 <= 2; p1++) {
      if (!iface(m[p1 - 1]) && ipass == 1) continue;
      face_index(F, 0, p1, fa);
      for (int p2 = 1; p2 <= 2; p2++) {
        if (!iface(m[p2 + 1]) && ipass == 1) continue;
        face_index(F, 1, p2, fb);
        for (int p3 = 1; p3 <= 2; p3++) {
          if (!iface(m[p3 + 3]) && ipass == 1) continue;
          face_index(F, 2, p3, fc);
          int g[3] = {fa[0], fb[0], fc[0]}, s1[3] = {fa[1], fb[1], fc[1]}, s2[3] = {fa[2], fb[2], fc[2]};
          int cc[4][3] = {{fa[3], fb[3], fc[3]}};
          cf3(f, c, 0, g, s1, s2, cc);
        }
      }
    }
    for (int p1 = 1; p1 <= 2; p1++) {  // edges 1-4
      if (!iface(m[p1 - 1]) && ipass == 1) continue;
      face_index(F, 0, p1, fa);
      for (int p3 = 1; p3 <= 2; p3++) {
        if (m[p3 + 3] != 2 && m[p3 + 3] != 99 && ipass == 1) continue;
        face_index(F, 2, p3, fc);
        cf3_edge(f, c, 0, fa, 2, fc, 1);
      }
    }
    for (int p1 = 1; p1 <= 2; p1++) {  // edges 5-8
      if (!iface(m[p1 - 1]) && ipass == 1) continue;
      face_index(F, 0, p1, fa);
      for (int p2 = 1; p2 <= 2; p2++) {
        if (!iface(m[p2 + 1]) && ipass == 1) continue;
        face_index(F, 1, p2, fb);
        cf3_edge(f, c, 0, fa, 1, fb, 2);
      }
    }
    for (int p2 = 1; p2 <= 2; p2++) {  // edges 9-12
      if (!iface(m[p2 + 1]) && ipass == 1) continue;
      face_index(F, 1, p2, fb);
      for (int p3 = 1; p3 <= 2; p3++) {
        if (!iface(m[p3 + 3]) && ipass == 1) continue;
        face_index(F, 2, p3, fc);
        cf3_edge(f, c, 1, fb, 2, fc, 0);
      }
    }
    static const int T[3][2] = {{1, 2}, {0, 2}, {0, 1}};
    for (int n = 0; n < 3; n++)
      for (int par = 1; par <= 2; par++) {
        if (!iface(m[2 * n + par - 1])) continue;
        int fn[5];
        face_index(F, n, par, fn);
        if (ipass == 0 || (par + ipass) % 2 == 0) {
          cf3_face_class(f, c, n, fn, T[n][0], T[n][1], 0);
          cf3_face_class(f, c, n, fn, T[n][0], T[n][1], 1);
        }
        if (ipass == 0 || (par + ipass) % 2 == 1) {
          cf3_face_class(f, c, n, fn, T[n][0], T[n][1], 2);
          cf3_face_class(f, c, n, fn, T[n][0], T[n][1], 3);
        }
        cf3_face_grey(f, c, n, fn, T[n][0], T[n][1]);
      }
  }

  // GhostOverlap, boundary.f90:359-431 (the landscape part is mesh-build
  // only).  Ghost cells of g1 that lie in the interior of g2 (shifted by
  // off) take g2's values, then the converse.
  void ghost_overlap(int g1, int g2, const int* off) {
    const HostPatch& A = H.patches[g1];
    const HostPatch& B = H.patches[g2];
    int nd = H.ndims, mbc = H.mbc;
    int mg1[3][2], mg2[3][2], ovg[3][2], ovg1[3][2], ovg2[3][2];
    for (int n = 0; n < 3; n++)
      for (int s = 0; s < 2; s++) mg1[n][s] = mg2[n][s] = ovg[n][s] = ovg1[n][s] = ovg2[n][s] = 1;
    for (int n = 0; n < nd; n++) {
      mg1[n][0] = A.mglobal[n][0];
      mg1[n][1] = A.mglobal[n][1];
      mg2[n][0] = B.mglobal[n][0] + (off ? off[n] : 0);
      mg2[n][1] = B.mglobal[n][1] + (off ? off[n] : 0);
    }
    for (int n = 0; n < nd; n++) {
      ovg[n][0] = std::max(mg1[n][0] - mbc, mg2[n][0] - mbc);
      ovg[n][1] = std::min(mg1[n][1] + mbc, mg2[n][1] + mbc);
    }
    for (int n = 0; n < nd; n++)
      if (ovg[n][1] - ovg[n][0] < 0) return;
    for (int n = 0; n < nd; n++) {
      ovg1[n][0] = std::max(ovg[n][0], mg2[n][0]);
      ovg1[n][1] = std::min(ovg[n][1], mg2[n][1]);
      ovg2[n][0] = std::max(ovg[n][0], mg1[n][0]);
      ovg2[n][1] = std::min(ovg[n][1], mg1[n][1]);
    }
    auto xfer = [&](int dst, int src, int ov[3][2], int mgd[3][2], int mgs[3][2]) {
      int lo[3], ls[3], ext[3];
      for (int n = 0; n < 3; n++) {
        if (n < nd) {
          lo[n] = ov[n][0] - mgd[n][0] + 1;
          ls[n] = ov[n][0] - mgs[n][0] + 1;
          ext[n] = ov[n][1] - ov[n][0];
        } else {
          lo[n] = ls[n] = 1;
          ext[n] = 0;
        }
      }
      for (int k = 0; k <= ext[2]; k++)
        for (int j = 0; j <= ext[1]; j++)
          for (int i = 0; i <= ext[0]; i++)
            copy(kGCopy, dst, cell(dst, lo[0] + i, lo[1] + j, nd == 3 ? lo[2] + k : 0), src,
                 cell(src, ls[0] + i, ls[1] + j, nd == 3 ? ls[2] + k : 0));
    };
    xfer(g1, g2, ovg1, mg1, mg2);
    xfer(g2, g1, ovg2, mg2, mg1);
  }

  // SelfPeriodicBC, boundary.f90:480-577
  void self_periodic(int p) {
    const HostPatch& P = H.patches[p];
    int nd = H.ndims, mbc = H.mbc;
    int lo[3], hi[3];
    for (int d = 0; d < 3; d++) {
      lo[d] = d < nd ? 1 - mbc : 1;
      hi[d] = d < nd ? P.mx[d] + mbc : 1;
    }
    auto cl = [&](int i, int j, int k) { return cell(p, i, j, nd == 3 ? k : 0); };
    if (P.mthbc[0] == 2 && P.mthbc[1] == 2)
      for (int ibc = 1; ibc <= mbc; ibc++) {
        for (int k = lo[2]; k <= hi[2]; k++)
          for (int j = lo[1]; j <= hi[1]; j++) copy(kGCopyAdd, p, cl(P.mx[0] + ibc, j, k), p, cl(ibc, j, k));
        for (int k = lo[2]; k <= hi[2]; k++)
          for (int j = lo[1]; j <= hi[1]; j++)
            copy(kGCopySub, p, cl(1 - ibc, j, k), p, cl(P.mx[0] + 1 - ibc, j, k));
      }
    if (P.mthbc[2] == 2 && P.mthbc[3] == 2)
      for (int ibc = 1; ibc <= mbc; ibc++) {
        for (int k = lo[2]; k <= hi[2]; k++)
          for (int i = lo[0]; i <= hi[0]; i++) copy(kGCopy, p, cl(i, P.mx[1] + ibc, k), p, cl(i, ibc, k));
        for (int k = lo[2]; k <= hi[2]; k++)
          for (int i = lo[0]; i <= hi[0]; i++) copy(kGCopy, p, cl(i, 1 - ibc, k), p, cl(i, P.mx[1] + 1 - ibc, k));
      }
    if (nd == 3 && P.mthbc[4] == 2 && P.mthbc[5] == 2)
      for (int ibc = 1; ibc <= mbc; ibc++) {
        for (int j = lo[1]; j <= hi[1]; j++)
          for (int i = lo[0]; i <= hi[0]; i++) copy(kGCopy, p, cl(i, j, P.mx[2] + ibc), p, cl(i, j, ibc));
        for (int j = lo[1]; j <= hi[1]; j++)
          for (int i = lo[0]; i <= hi[0]; i++) copy(kGCopy, p, cl(i, j, 1 - ibc), p, cl(i, j, P.mx[2] + 1 - ibc));
      }
  }

  // Dirichlet masks of the plugin's UserBC2D/3D (CH/problem.f90:770-881,
  // BioGrowth/problem.f90:623-736; the plugin files state theirs): bits 0-7
  // the variables set to 2 - q, bits 8-15 those set to -q, the others
  // reflected.
  int bc_mask() const { return find_plugin(H.problem)->bc_mask(H.ndims); }

  // SetPhysicalBC2D/3D (boundary.f90:614-802) -> UserBC on each face with
  // mthbc = 10, faces in order 1..2*ndims.
  void physical_bc(int p) {
    const HostPatch& P = H.patches[p];
    int nd = H.ndims, mbc = H.mbc, ll = 1 - mbc;
    int ul[3];
    for (int d = 0; d < 3; d++) ul[d] = P.mx[d] + mbc;
    int kl = nd == 3 ? ll : 0, ku = nd == 3 ? ul[2] : 0;
    int mask = bc_mask();
    for (int face = 1; face <= 2 * nd; face++) {
      if (P.mthbc[face - 1] != 10) continue;
      int d = (face - 1) / 2, hi = (face - 1) % 2;
      for (int ibc = 1; ibc <= mbc; ibc++) {
        int gd = hi ? P.mx[d] + ibc : 1 - ibc;
        int gs = hi ? P.mx[d] - ibc + 1 : ibc;
        if (d == 0) {
          for (int k = kl; k <= ku; k++)
            for (int j = ll; j <= ul[1]; j++) bc(p, cell(p, gd, j, k), cell(p, gs, j, k), mask);
        } else if (d == 1) {
          for (int k = kl; k <= ku; k++)
            for (int i = ll; i <= ul[0]; i++) bc(p, cell(p, i, gd, k), cell(p, i, gs, k), mask);
        } else {
          for (int j = ll; j <= ul[1]; j++)
            for (int i = ll; i <= ul[0]; i++) bc(p, cell(p, i, j, gd), cell(p, i, j, gs), mask);
        }
      }
    }
  }

  // GetPeriodicOffsets, boundary.f90:875-954
  void periodic_offsets(int level, int poff[13][3]) const {
    const int* mm = H.mxmax[level];
    for (int o = 0; o < H.nperoff; o++) {
      int a = 0, b = 0, c = 0;
      switch (H.peroffidx[o]) {
        case 1: a = mm[0]; break;
        case 2: b = mm[1]; break;
        case 3: c = mm[2]; break;
        case 4: a = mm[0]; b = mm[1]; break;
        case 5: a = -mm[0]; b = mm[1]; break;
        case 6: b = mm[1]; c = mm[2]; break;
        case 7: b = mm[1]; c = -mm[2]; break;
        case 8: a = mm[0]; c = mm[2]; break;
        case 9: a = -mm[0]; c = mm[2]; break;
        case 10: a = mm[0]; b = mm[1]; c = mm[2]; break;
        case 11: a = mm[0]; b = mm[1]; c = -mm[2]; break;
        case 12: a = -mm[0]; b = mm[1]; c = mm[2]; break;
        case 13: a = mm[0]; b = -mm[1]; c = mm[2]; break;
      }
      poff[o][0] = a;
      poff[o][1] = b;
      poff[o][2] = c;
    }
  }
};

}  // namespace

namespace {

// The writer sequence of SetGhost(level, ipass), in the reference's order,
// as five segments of per-patch items: coarse-fine interpolation of patch a
// (levels > 0), its sibling overlaps with the patches after it (levels >
// 0), its self-periodic copies, its periodic-image overlaps with the patches
// after it (periodic levels > 0), its physical boundary condition.  Item
// (segment, a) appends exactly what the reference's loops append at that
// point, so concatenating the items in (segment, a) order is the sequence;
// the items are independent, so they are emitted in parallel.
struct LevelEmit {
  const Hier& H;
  int level, ipass, n;
  const std::vector<int>& ps;
  std::vector<int> org;
  int poff[13][3] = {};
  std::vector<char> edge;
  LevelEmit(const Hier& h, int l, int ip) : H(h), level(l), ipass(ip), ps(h.L(l).patches), org(h.patches.size()) {
    n = (int)ps.size();
    for (size_t p = 0; p < h.patches.size(); p++) org[p] = (int)origin_of(h, h.patches[p].qn);
    if (H.periodic && level > 0) {
      Emitter E(H, org);
      E.periodic_offsets(level, poff);
      // Only patches within 2*mbc of the domain edge can meet another
      // patch's periodic image (for offset +N in dimension d the ghost boxes
      // meet only if (N - hi_a) + (lo_b - 1) <= 2*mbc); other pairs emit
      // nothing, so skipping them leaves the operation sequence unchanged.
      edge.assign(n, 0);
      for (int a = 0; a < n; a++) {
        const HostPatch& P = H.patches[ps[a]];
        for (int d = 0; d < H.ndims; d++)
          if (P.mglobal[d][0] - 1 <= 2 * H.mbc || H.mxmax[level][d] - P.mglobal[d][1] <= 2 * H.mbc) edge[a] = 1;
      }
    }
  }
  int items() const { return 5 * n; }
  void item(int x, std::vector<Em>& out) const {
    Emitter E(H, org);
    E.out.swap(out);
    const int seg = x / n, a = x % n;
    switch (seg) {
      case 0:
        if (level > 0) {
          if (H.ndims == 2) E.interpolate2d(ps[a], ipass);
          else E.interpolate3d(ps[a], ipass);
        }
        break;
      case 1:
        if (level > 0)
          for (int b = a + 1; b < n; b++) E.ghost_overlap(ps[a], ps[b], nullptr);
        break;
      case 2:
        if (H.periodic) E.self_periodic(ps[a]);
        break;
      case 3:
        if (H.periodic && level > 0 && edge[a])
          for (int b = a + 1; b < n; b++)
            if (edge[b])
              for (int pol = -1; pol <= 1; pol += 2)
                for (int o = 0; o < H.nperoff; o++) {
                  int off[3] = {pol * poff[o][0], pol * poff[o][1], pol * poff[o][2]};
                  E.ghost_overlap(ps[a], ps[b], off);
                }
        break;
      default:
        E.physical_bc(ps[a]);
        break;
    }
    E.out.swap(out);
  }
};

std::vector<Em> concat(std::vector<std::vector<Em>>& parts) {
  size_t m = 0;
  for (auto& v : parts) m += v.size();
  std::vector<Em> all;
  all.reserve(m);
  for (auto& v : parts) {
    all.insert(all.end(), v.begin(), v.end());
    std::vector<Em>().swap(v);
  }
  return all;
}

// the sequence of one (level, ipass), its items emitted in parallel
std::vector<Em> emit_set_ghost(const Hier& H, int level, int ipass) {
  LevelEmit L(H, level, ipass);
  std::vector<std::vector<Em>> parts(L.items());
  parallel_for(L.items(), [&](int x) { L.item(x, parts[x]); });
  return concat(parts);
}

// Dead writes and stages of one emitted sequence (see the file comment).
std::vector<GhostOp> stage_ops(const Hier& H, std::vector<Em>& ops, std::vector<int>& stage_off);

}  // namespace

std::vector<GhostOp> set_ghost_sequence(const Hier& H, int level, int ipass) {
  std::vector<Em> em = emit_set_ghost(H, level, ipass);
  std::vector<GhostOp> res(em.size());
  for (size_t x = 0; x < em.size(); x++) res[x] = em[x].op;
  return res;
}

std::vector<GhostOp> compile_set_ghost(const Hier& H, int level, int ipass, std::vector<int>& stage_off) {
  std::vector<Em> em = emit_set_ghost(H, level, ipass);
  return stage_ops(H, em, stage_off);
}

void compile_set_ghost_all(const Hier& H, const std::vector<std::pair<int, int>>& jobs,
                           std::vector<std::vector<GhostOp>*> out, std::vector<std::vector<int>*> stage_off) {
  // every item of every job in one parallel pass, then the jobs' staging
  std::vector<std::unique_ptr<LevelEmit>> le;
  std::vector<int> first(jobs.size() + 1, 0);
  for (size_t j = 0; j < jobs.size(); j++) {
    le.emplace_back(new LevelEmit(H, jobs[j].first, jobs[j].second));
    first[j + 1] = first[j] + le.back()->items();
  }
  std::vector<std::vector<Em>> parts(first.back());
  parallel_for(first.back(), [&](int x) {
    size_t j = std::upper_bound(first.begin(), first.end(), x) - first.begin() - 1;
    le[j]->item(x - first[j], parts[x]);
  });
  parallel_for((int)jobs.size(), [&](int j) {
    std::vector<std::vector<Em>> mine(std::make_move_iterator(parts.begin() + first[j]),
                                      std::make_move_iterator(parts.begin() + first[j + 1]));
    std::vector<Em> em = concat(mine);
    *out[j] = stage_ops(H, em, *stage_off[j]);
  });
}

namespace {

std::vector<GhostOp> stage_ops(const Hier& H, std::vector<Em>& ops, std::vector<int>& stage_off) {
  // Cells are keyed by patch and cell offset; the passes below use flat
  // arrays over the ghosted cells of the patches the operations touch.
  int m = (int)ops.size();
  std::vector<long long> base(H.patches.size(), -1);
  long long slots = 0;
  auto slot_base = [&](int p) {
    long long& b = base[p];
    if (b < 0) {
      const HostPatch& P = H.patches[p];
      b = slots;
      slots += (long long)P.qn[0] * P.qn[1] * P.qn[2];
    }
    return b;
  };
  std::vector<long long> dkey(m), skey(2 * (size_t)m);
  for (int x = 0; x < m; x++) {
    dkey[x] = slot_base((int)(ops[x].dst >> 32)) + (uint32_t)ops[x].dst;
    for (int s = 0; s < ops[x].nsrc; s++)
      skey[2 * (size_t)x + s] = slot_base((int)(ops[x].src[s] >> 32)) + (uint32_t)ops[x].src[s];
  }
  // pass 1: drop writes overwritten before any read
  std::vector<char> dead(m, 0), readf(m, 0);
  std::vector<int> last(slots, -1);
  for (int x = 0; x < m; x++) {
    for (int s = 0; s < ops[x].nsrc; s++) {
      int w = last[skey[2 * (size_t)x + s]];
      if (w >= 0) readf[w] = 1;
    }
    int w = last[dkey[x]];
    if (w >= 0 && !readf[w]) dead[w] = 1;
    last[dkey[x]] = x;
  }
  // pass 2: stage = 1 + latest conflicting live predecessor (wst: stage of
  // the last write of a cell, rst: latest stage reading it since)
  std::vector<int> wst(slots, -1), rst(slots, -1), stage(m, -1);
  int nst = 0;
  for (int x = 0; x < m; x++) {
    if (dead[x]) continue;
    int st = 0;
    for (int s = 0; s < ops[x].nsrc; s++) {
      int w = wst[skey[2 * (size_t)x + s]];
      if (w >= 0) st = std::max(st, w + 1);
    }
    long long d = dkey[x];
    if (rst[d] >= 0) st = std::max(st, rst[d] + 1);
    if (wst[d] >= 0) st = std::max(st, wst[d] + 1);
    stage[x] = st;
    for (int s = 0; s < ops[x].nsrc; s++) {
      int& r = rst[skey[2 * (size_t)x + s]];
      r = std::max(r, st);
    }
    wst[d] = st;
    rst[d] = -1;
    nst = std::max(nst, st + 1);
  }
  std::vector<GhostOp> res;
  stage_off.assign(nst + 1, 0);
  for (int x = 0; x < m; x++)
    if (!dead[x]) stage_off[stage[x] + 1]++;
  for (int s = 0; s < nst; s++) stage_off[s + 1] += stage_off[s];
  res.resize(stage_off[nst]);
  std::vector<int> fill(stage_off.begin(), stage_off.end() - 1);
  for (int x = 0; x < m; x++)
    if (!dead[x]) res[fill[stage[x]]++] = ops[x].op;
  return res;
}

}  // namespace

}  // namespace bsamg
