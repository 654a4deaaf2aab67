// Plain FP64 kernels: the drop-in path.
//
// This translation unit is compiled with --fmad=false: every product and sum
// is rounded separately, in the evaluation order of the reference Fortran, so
// results agree bit for bit with a reference build that does not contract
// multiply-adds (the CPU oracle is built that way).  Division is the IEEE
// round-to-nearest `/`.
//
// On GB300 these kernels are bounded by the FP64 pipe, not by HBM: the CH
// smoother needs ~22 FP64 operations and 2 divisions per cell update against
// 32 bytes of algorithmic traffic, and the part issues FP64 at ~1.2 TFLOP/s.
#include <cuda_runtime.h>

#include <algorithm>

#include "internal.h"
#include "launch.h"

namespace bsamg {

// C/F interpolation weights, LIBRARY/boundary.f90:54-63
__constant__ double kA1 = -01.0 / 05.0;
__constant__ double kA2 = 02.0 / 03.0;
__constant__ double kA3 = 08.0 / 15.0;
__constant__ double kB1 = 05.0 / 32.0;
__constant__ double kB2 = 15.0 / 16.0;
__constant__ double kB3 = -03.0 / 32.0;
__constant__ double kC1 = 09.0 / 16.0;
__constant__ double kC2 = 03.0 / 16.0;
__constant__ double kC3 = 03.0 / 16.0;
__constant__ double kC4 = 01.0 / 16.0;

__device__ __forceinline__ double cube(double c) { return c * c * c; }  // CH/problem.f90:918
__device__ __forceinline__ double sqr(double c) { return c * c; }       // CH/problem.f90:931

// offset of Fortran cell (i,j,k) (lower bound 0) in a ghosted plane
template <int DIM>
__device__ __forceinline__ long long gofs(const int* n, int i, int j, int k) {
  if (DIM == 2) return (long long)j * n[0] + i;
  return ((long long)k * n[1] + j) * n[0] + i;
}
// offset of Fortran cell (i,j,k) (lower bound 1) in an interior plane
template <int DIM>
__device__ __forceinline__ long long iofs(const int* mx, int i, int j, int k) {
  if (DIM == 2) return (long long)(j - 1) * mx[0] + (i - 1);
  return ((long long)(k - 1) * mx[1] + (j - 1)) * mx[0] + (i - 1);
}

// ULap2D / ULap3D, LIBRARY/gridutilities.f90:50-72, :372-399
template <int DIM>
__device__ __forceinline__ double ulap(const double* a, long long c, long long sy, long long sz) {
  if (DIM == 2) return a[c + 1] + a[c - 1] + a[c + sy] + a[c - sy] - 4.0 * a[c];
  return a[c + 1] + a[c - 1] + a[c + sy] + a[c - sy] + a[c + sz] + a[c - sz] - 6.0 * a[c];
}

// Operator2D/3D of the plugin at ghosted offset c of array a (planes of ps
// elements), with qold value o0 (variable 1 at the same cell) and patch
// coefficients cf; r receives one value per variable.  CH:
// CH/problem.f90:393-422, :638-669; BioGrowth: BioGrowth/problem.f90:320-353
// (3D: zero stub, :497-522); growth (three variables, no reference
// counterpart): phi as BioGrowth's with 2*ndims neighbours, n the BioGrowth
// uptake equation, p: -Lap(p)/h^2 - cpress*phi*n.
template <int PROB, int DIM>
__device__ __forceinline__ void op_eval(const double* a, long long c, long long sy, long long sz,
                                        long long ps, double o0, const double* cf,
                                        const ProbParams& pp, double* r) {
  const double* a0 = a;
  const double* a1 = a + ps;
  if (PROB == kCH) {
    r[0] = a0[c] - cf[0] * ulap<DIM>(a1, c, sy, sz);
    r[1] = a1[c] - cube(a0[c]) + cf[1] * ulap<DIM>(a0, c, sy, sz);
  } else if (PROB == kBio) {
    if (DIM == 2) {
      double dt = pp.dt;
      r[0] = a0[c] - cf[0] * ulap<DIM>(a0, c, sy, sz) + dt * cube(a0[c]) -
             dt * (pp.gamma * 0.5 * (o0 + 1.0)) * (a1[c] - pp.czero);
      r[1] = -cf[1] * ulap<DIM>(a1, c, sy, sz) + (pp.lambda * 0.5 * (o0 + 1.0)) * a1[c];
    } else {
      r[0] = 0.0;
      r[1] = 0.0;
    }
  } else {
    const double* a2 = a + 2 * ps;
    double dt = pp.dt;
    r[0] = a0[c] - cf[0] * ulap<DIM>(a0, c, sy, sz) + dt * cube(a0[c]) -
           dt * (pp.gamma * 0.5 * (o0 + 1.0)) * (a1[c] - pp.czero);
    r[1] = -cf[1] * ulap<DIM>(a1, c, sy, sz) + (pp.lambda * 0.5 * (o0 + 1.0)) * a1[c];
    r[2] = -cf[1] * ulap<DIM>(a2, c, sy, sz) - pp.cpress * a0[c] * a1[c];
  }
}

// Source2D/3D + SourceUpdate2D/3D values (CH/problem.f90:425-476, :672-721;
// BioGrowth/problem.f90:356-405, :525-575; growth as BioGrowth, p zero)
template <int PROB, int DIM>
__device__ __forceinline__ void source_eval(double o0, const ProbParams& pp, double* s) {
  if (PROB == kCH) {
    s[0] = o0;
    s[1] = -o0;
  } else if (PROB == kBio) {
    s[0] = DIM == 2 ? (1.0 + pp.dt) * o0 : 0.0;
    s[1] = 0.0;
  } else {
    s[0] = (1.0 + pp.dt) * o0;
    s[1] = 0.0;
    s[2] = 0.0;
  }
}

// map a unit of a colour work list to an interior cell; false if the slot is
// past the end of its row (odd mx) or past the patch.  The colour test is the
// reference loop start i = 1 + MODULO(j(+k)+ipass, 2) (CH/problem.f90:350,
// :591).
template <int DIM>
__device__ __forceinline__ bool color_cell(const PatchDev& p, int t, int ipass, int& i, int& j, int& k) {
  int hx = (p.mx[0] + 1) >> 1;
  int row = t / hx;
  int s = t - row * hx;
  if (DIM == 2) {
    j = row + 1;
    k = 1;
    if (j > p.mx[1]) return false;
    i = 1 + ((j + ipass) & 1) + 2 * s;
  } else {
    j = row % p.mx[1] + 1;
    k = row / p.mx[1] + 1;
    if (k > p.mx[2]) return false;
    i = 1 + ((k + j + ipass) & 1) + 2 * s;
  }
  return i <= p.mx[0];
}

template <int DIM>
__device__ __forceinline__ bool interior_cell(const int* mx, int t, int& i, int& j, int& k) {
  i = t % mx[0] + 1;
  int r = t / mx[0];
  if (DIM == 2) {
    j = r + 1;
    k = 1;
    return j <= mx[1];
  }
  j = r % mx[1] + 1;
  k = r / mx[1] + 1;
  return k <= mx[2];
}

template <int DIM>
__device__ __forceinline__ bool ghosted_cell(const int* n, int gs, int t, int& i, int& j, int& k) {
  // cell t of a ghosted array of extents n whose indices start at -gs
  i = t % n[0] - gs;
  int r = t / n[0];
  if (DIM == 2) {
    j = r - gs;
    k = 0;
    return r < n[1];
  }
  j = r % n[1] - gs;
  k = r / n[1];
  bool ok = k < n[2];
  k -= gs;
  return ok;
}

// ---------------------------------------------------------------------------
// Red-black pointwise relaxation of one colour over all patches of a level.

template <int PROB, int DIM>
__device__ __forceinline__ void u_relax(const PatchDev* __restrict__ P, double* __restrict__ pool, const Blk b,
                                        int tid, int ipass, const ProbParams& pp) {
  const PatchDev& p = P[b.patch];
  int i, j, k;
  if (!color_cell<DIM>(p, b.start + tid, ipass, i, j, k)) return;
  double* q0 = pool + p.oq;
  double* q1 = q0 + p.sq;
  const double* f0 = pool + p.of;
  const double* f1 = f0 + p.sf;
  long long sy = p.qn[0], sz = (long long)p.qn[0] * p.qn[1];
  long long c = gofs<DIM>(p.qn, i, j, k);
  long long fc = iofs<DIM>(p.mx, i, j, k);
  if (PROB == kCH) {
    // RelaxGrid2D CH/problem.f90:349-367, RelaxGrid3D :589-612
    double phi = q0[c];
    double a21 = -3.0 * sqr(phi) - p.c[2];
    double b1, b2;
    if (DIM == 2) {
      b1 = f0[fc] + p.c[0] * (q1[c - 1] + q1[c + 1] + q1[c - sy] + q1[c + sy]);
      b2 = f1[fc] - p.c[1] * (q0[c + 1] + q0[c - 1] + q0[c + sy] + q0[c - sy]) - 2.0 * cube(phi);
    } else {
      b1 = f0[fc] + p.c[0] * (q1[c - 1] + q1[c + 1] + q1[c - sy] + q1[c + sy] + q1[c - sz] + q1[c + sz]);
      b2 = f1[fc] - p.c[1] * (q0[c + 1] + q0[c - 1] + q0[c + sy] + q0[c - sy] + q0[c + sz] + q0[c - sz]) -
           2.0 * cube(phi);
    }
    double det = 1.0 - p.c[3] * a21;
    q0[c] = (b1 - p.c[3] * b2) / det;
    q1[c] = (b2 - a21 * b1) / det;
  } else if (PROB == kBio) {
    if (DIM == 2) {
      // RelaxGrid2D BioGrowth/problem.f90:280-294
      const double* o0 = pool + p.oqold;
      double dt = pp.dt;
      double phi = q0[c];
      double ol = o0[c];
      double tmp2 = p.c[2] + dt * sqr(phi);
      q0[c] = (f0[fc] + dt * (pp.gamma * 0.5 * (ol + 1.0)) * (q1[c] - pp.czero) +
               p.c[0] * (q0[c - 1] + q0[c + 1] + q0[c - sy] + q0[c + sy])) / tmp2;
      double tmp4 = p.c[3] + (pp.lambda * 0.5 * (ol + 1.0));
      q1[c] = (f1[fc] + p.c[1] * (q1[c + 1] + q1[c - 1] + q1[c + sy] + q1[c - sy])) / tmp4;
    } else {
      // RelaxGrid3D BioGrowth/problem.f90:467-476 (zero stub)
      q0[c] = 0.0;
      q1[c] = 0.0;
    }
  } else {
    // growth: phi and n as BioGrowth's RelaxGrid2D with 2*ndims neighbours,
    // then p from the updated phi and n
    double* q2 = q1 + p.sq;
    const double* f2 = f1 + p.sf;
    const double* o0 = pool + p.oqold;
    double dt = pp.dt;
    double phi = q0[c];
    double ol = o0[c];
    double tmp2 = p.c[2] + dt * sqr(phi);
    double s0 = q0[c - 1] + q0[c + 1] + q0[c - sy] + q0[c + sy];
    double s1 = q1[c + 1] + q1[c - 1] + q1[c + sy] + q1[c - sy];
    double s2 = q2[c + 1] + q2[c - 1] + q2[c + sy] + q2[c - sy];
    if (DIM == 3) {
      s0 = s0 + q0[c - sz] + q0[c + sz];
      s1 = s1 + q1[c + sz] + q1[c - sz];
      s2 = s2 + q2[c + sz] + q2[c - sz];
    }
    double np = (f0[fc] + dt * (pp.gamma * 0.5 * (ol + 1.0)) * (q1[c] - pp.czero) + p.c[0] * s0) / tmp2;
    double tmp4 = p.c[3] + (pp.lambda * 0.5 * (ol + 1.0));
    double nn = (f1[fc] + p.c[1] * s1) / tmp4;
    q0[c] = np;
    q1[c] = nn;
    q2[c] = (f2[fc] + p.c[1] * s2 + pp.cpress * np * nn) / p.c[3];
  }
}
template <int PROB, int DIM>
__global__ void __launch_bounds__(kBlock) k_relax(const PatchDev* __restrict__ P, double* __restrict__ pool,
                                                  const Blk* __restrict__ blk, int ipass, ProbParams pp) {
  u_relax<PROB, DIM>(P, pool, blk[blockIdx.x], threadIdx.x, ipass, pp);
}

// ---------------------------------------------------------------------------
// Restriction2D/3D (gridutilities.f90:103-126, :437-466) of plane `a`
// (accessed through `at`) at coarse cell (ci,cj,ck).

template <int DIM, typename F>
__device__ __forceinline__ double restrict_at(F at, int ci, int cj, int ck) {
  int i = 2 * ci, j = 2 * cj;
  if (DIM == 2) return 0.25 * (at(i, j, 1) + at(i - 1, j, 1) + at(i, j - 1, 1) + at(i - 1, j - 1, 1));
  int k = 2 * ck;
  return 0.125 * (at(i, j, k) + at(i - 1, j, k) + at(i, j - 1, k) + at(i - 1, j - 1, k) + at(i, j, k - 1) +
                  at(i - 1, j, k - 1) + at(i, j - 1, k - 1) + at(i - 1, j - 1, k - 1));
}

// RestrictSolution, afasroutines.f90:610-652: qc(1:cmx) = R(q);
// parent q(mb) = qc.
template <int DIM>
__device__ __forceinline__ void u_restrict_q(const PatchDev* __restrict__ P, double* __restrict__ pool, const Blk b,
                                             int tid, int nrvars) {
  const PatchDev& p = P[b.patch];
  int ci, cj, ck;
  if (!interior_cell<DIM>(p.cmx, b.start + tid, ci, cj, ck)) return;
  const PatchDev& par = P[p.parent];
  for (int v = 0; v < nrvars; v++) {
    const double* q = pool + p.oq + v * p.sq;
    auto at = [&](int i, int j, int k) { return q[gofs<DIM>(p.qn, i, j, k)]; };
    double val = restrict_at<DIM>(at, ci, cj, ck);
    pool[p.oqc + v * p.sc + gofs<DIM>(p.cn, ci, cj, ck)] = val;
    pool[par.oq + v * par.sq + gofs<DIM>(par.qn, p.mb[0] + ci - 1, p.mb[1] + cj - 1, DIM == 3 ? p.mb[2] + ck - 1 : 0)] = val;
  }
}
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_restrict_q(const PatchDev* __restrict__ P, double* __restrict__ pool,
                                                       const Blk* __restrict__ blk, int nrvars) {
  u_restrict_q<DIM>(P, pool, blk[blockIdx.x], threadIdx.x, nrvars);
}

// GetCoarseGhostPoints, boundary.f90:957-1015.  Every ring cell of qc is
// covered by exactly one of its face statements, each of which copies
// parent%q(mb-1+i, mb-1+j, mb-1+k).
template <int DIM>
__device__ __forceinline__ void u_coarse_ghost(const PatchDev* __restrict__ P, double* __restrict__ pool, const Blk b,
                                               int tid, int nrvars) {
  const PatchDev& p = P[b.patch];
  int i, j, k;
  if (!ghosted_cell<DIM>(p.cn, p.gs, b.start + tid, i, j, k)) return;
  // the first ring only (0 and cmx+1; a second layer, mbc = 2, is not set)
  bool inside = i >= 0 && i <= p.cmx[0] + 1 && j >= 0 && j <= p.cmx[1] + 1 &&
                (DIM == 2 || (k >= 0 && k <= p.cmx[2] + 1));
  bool ring = i == 0 || i == p.cmx[0] + 1 || j == 0 || j == p.cmx[1] + 1 ||
              (DIM == 3 && (k == 0 || k == p.cmx[2] + 1));
  if (!inside || !ring) return;
  const PatchDev& par = P[p.parent];
  long long src = gofs<DIM>(par.qn, p.mb[0] - 1 + i, p.mb[1] - 1 + j, DIM == 3 ? p.mb[2] - 1 + k : 0);
  long long dst = gofs<DIM>(p.cn, i, j, k);
  for (int v = 0; v < nrvars; v++) pool[p.oqc + v * p.sc + dst] = pool[par.oq + v * par.sq + src];
}
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_coarse_ghost(const PatchDev* __restrict__ P, double* __restrict__ pool,
                                                         const Blk* __restrict__ blk, int nrvars) {
  u_coarse_ghost<DIM>(P, pool, blk[blockIdx.x], threadIdx.x, nrvars);
}

// CoarseLoadingFunction, afasroutines.f90:673-736, with Residual (:817-857):
// rf = f - Op_h(q) on the children of a coarse cell;
// parent f(mb) = R(rf) + Op_2h(qc, parent qold, h_parent).
template <int PROB, int DIM>
__device__ __forceinline__ void u_coarse_load(const PatchDev* __restrict__ P, double* __restrict__ pool, const Blk b,
                                              int tid, const ProbParams& pp) {
  const PatchDev& p = P[b.patch];
  int ci, cj, ck;
  if (!interior_cell<DIM>(p.cmx, b.start + tid, ci, cj, ck)) return;
  const PatchDev& par = P[p.parent];
  const double* q = pool + p.oq;
  const double* qo = pool + p.oqold;
  long long sy = p.qn[0], sz = (long long)p.qn[0] * p.qn[1];
  constexpr int NV = PROB == kGrowth ? 3 : 2;
  double* rf = pool + p.orf;
  const double* f = pool + p.of;
  const int nk = DIM == 3 ? 2 : 1;
  for (int dk = 0; dk < nk; dk++)
    for (int dj = 0; dj < 2; dj++)
      for (int di = 0; di < 2; di++) {
        int i = 2 * ci - di, j = 2 * cj - dj, k = DIM == 3 ? 2 * ck - dk : 1;
        long long c = gofs<DIM>(p.qn, i, j, k);
        long long fc = iofs<DIM>(p.mx, i, j, k);
        double r[NV];
        op_eval<PROB, DIM>(q, c, sy, sz, p.sq, qo[c], p.c, pp, r);
        for (int v = 0; v < NV; v++) rf[v * p.sf + fc] = f[v * p.sf + fc] - r[v];
      }
  // the restriction reads rf written above by this same thread
  double R[NV];
  for (int v = 0; v < NV; v++) {
    const double* rv = rf + v * p.sf;
    auto at = [&](int i, int j, int k) { return rv[iofs<DIM>(p.mx, i, j, k)]; };
    R[v] = restrict_at<DIM>(at, ci, cj, ck);
  }
  // coarse operator on qc with the parent's spacing; parent qold at the
  // section parent%qold(mb-1:mb+1)
  const double* qc = pool + p.oqc;
  long long csy = p.cn[0], csz = (long long)p.cn[0] * p.cn[1];
  long long cc = gofs<DIM>(p.cn, ci, cj, ck);
  long long pc = gofs<DIM>(par.qn, p.mb[0] + ci - 1, p.mb[1] + cj - 1, DIM == 3 ? p.mb[2] + ck - 1 : 0);
  double o0 = pool[par.oqold + pc];
  double cr[NV];
  op_eval<PROB, DIM>(qc, cc, csy, csz, p.sc, o0, par.c, pp, cr);
  long long pf = iofs<DIM>(par.mx, p.mb[0] + ci - 1, p.mb[1] + cj - 1, DIM == 3 ? p.mb[2] + ck - 1 : 1);
  for (int v = 0; v < NV; v++) pool[par.of + v * par.sf + pf] = R[v] + cr[v];
}
template <int PROB, int DIM>
__global__ void __launch_bounds__(kBlock) k_coarse_load(const PatchDev* __restrict__ P, double* __restrict__ pool,
                                                        const Blk* __restrict__ blk, ProbParams pp) {
  u_coarse_load<PROB, DIM>(P, pool, blk[blockIdx.x], threadIdx.x, pp);
}

// CorrectFine step 1, afasroutines.f90:892-895 / :934-938:
// qc(1-mbc:cmx+mbc) = parent%q(mb-mbc:mb+mbc) - qc
template <int DIM>
__device__ __forceinline__ void u_correct_a(const PatchDev* __restrict__ P, double* __restrict__ pool, const Blk b,
                                            int tid, int nrvars) {
  const PatchDev& p = P[b.patch];
  int i, j, k;
  if (!ghosted_cell<DIM>(p.cn, p.gs, b.start + tid, i, j, k)) return;
  const PatchDev& par = P[p.parent];
  long long src = gofs<DIM>(par.qn, p.mb[0] - 1 + i, p.mb[1] - 1 + j, DIM == 3 ? p.mb[2] - 1 + k : 0);
  long long dst = gofs<DIM>(p.cn, i, j, k);
  for (int v = 0; v < nrvars; v++) {
    double* qc = pool + p.oqc + v * p.sc;
    qc[dst] = pool[par.oq + v * par.sq + src] - qc[dst];
  }
}
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_correct_a(const PatchDev* __restrict__ P, double* __restrict__ pool,
                                                      const Blk* __restrict__ blk, int nrvars) {
  u_correct_a<DIM>(P, pool, blk[blockIdx.x], threadIdx.x, nrvars);
}

// InitFields' first statement (bsamroutines.f90:1815-1818, :1834-1837):
// child qc(1-mbc:cmx+mbc) = parent%q(mb-mbc:mb+mbc), on a new patch
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_qc_from_parent(const PatchDev* __restrict__ P, double* __restrict__ pool,
                                                           const Blk* __restrict__ blk, int nrvars) {
  const Blk b = blk[blockIdx.x];
  const PatchDev& p = P[b.patch];
  int i, j, k;
  if (!ghosted_cell<DIM>(p.cn, p.gs, b.start + threadIdx.x, i, j, k)) return;
  const PatchDev& par = P[p.parent];
  long long src = gofs<DIM>(par.qn, p.mb[0] - 1 + i, p.mb[1] - 1 + j, DIM == 3 ? p.mb[2] - 1 + k : 0);
  long long dst = gofs<DIM>(p.cn, i, j, k);
  for (int v = 0; v < nrvars; v++) pool[p.oqc + v * p.sc + dst] = pool[par.oq + v * par.sq + src];
}

// CorrectFine step 2: q(1-mbc:mx+mbc) += BiLinProlongationP1/P2(qc)
// (gridutilities.f90:156-239) / TriLinProlongationP1/P2 (:510-625).  One
// thread per coarse index (ci,cj,ck) in -gs..cmx+gs produces fine cells
// 2ci..2ci+1 (and likewise in y, z) that lie in 1-mbc..mx+mbc: it forms
// the reference's intermediate b (and c) entries for its 2x2(x2) coarse
// values with the reference's expressions, so every fine value is
// bit-identical to the array form.  P2 is P1 over one more layer; it
// writes the odd cells' sum as 3 a(c+1) + a(c), the same IEEE sum.
template <int DIM>
__device__ __forceinline__ void u_correct_b(const PatchDev* __restrict__ P, double* __restrict__ pool, const Blk b,
                                            int tid, int nrvars) {
  const PatchDev& p = P[b.patch];
  const int gs = p.gs;
  int cpn[3] = {p.cmx[0] + 1 + 2 * gs, p.cmx[1] + 1 + 2 * gs, DIM == 3 ? p.cmx[2] + 1 + 2 * gs : 1};
  int t = b.start + tid;
  int ci = t % cpn[0], r = t / cpn[0];
  int cj = r % cpn[1], ck = r / cpn[1];
  if (ck >= cpn[2]) return;
  ci -= gs;
  cj -= gs;
  if (DIM == 3) ck -= gs;
  const int nz = DIM == 3 ? 2 : 1;
  for (int v = 0; v < nrvars; v++) {
    const double* a = pool + p.oqc + v * p.sc;
    double* q = pool + p.oq + v * p.sq;
    double bxv[2][2][2];
    for (int dz = 0; dz < nz; dz++)
      for (int dy = 0; dy < 2; dy++) {
        double lo = a[gofs<DIM>(p.cn, ci, cj + dy, ck + dz)], hi = a[gofs<DIM>(p.cn, ci + 1, cj + dy, ck + dz)];
        bxv[dz][dy][0] = 3.0 * lo + hi;
        bxv[dz][dy][1] = lo + 3.0 * hi;
      }
    for (int fz = 0; fz < nz; fz++)
      for (int fy = 0; fy < 2; fy++)
        for (int fx = 0; fx < 2; fx++) {
          int i = 2 * ci + fx, j = 2 * cj + fy, k = DIM == 3 ? 2 * ck + fz : 0;
          if (gs && (i < -gs || i > p.mx[0] + 1 + gs || j < -gs || j > p.mx[1] + 1 + gs ||
                     (DIM == 3 && (k < -gs || k > p.mx[2] + 1 + gs))))
            continue;
          double add;
          if (DIM == 2) {
            double blo = bxv[0][0][fx], bhi = bxv[0][1][fx];
            add = fy == 0 ? (3.0 * blo + bhi) / 16.0 : (blo + 3.0 * bhi) / 16.0;
          } else {
            double c0 = fy == 0 ? 3.0 * bxv[0][0][fx] + bxv[0][1][fx] : bxv[0][0][fx] + 3.0 * bxv[0][1][fx];
            double c1 = fy == 0 ? 3.0 * bxv[1][0][fx] + bxv[1][1][fx] : bxv[1][0][fx] + 3.0 * bxv[1][1][fx];
            add = fz == 0 ? (3.0 * c0 + c1) / 64.0 : (c0 + 3.0 * c1) / 64.0;
          }
          long long dst = gofs<DIM>(p.qn, i, j, k);
          q[dst] = q[dst] + add;
        }
  }
}
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_correct_b(const PatchDev* __restrict__ P, double* __restrict__ pool,
                                                      const Blk* __restrict__ blk, int nrvars) {
  u_correct_b<DIM>(P, pool, blk[blockIdx.x], threadIdx.x, nrvars);
}

// FillDownLevel, afasroutines.f90:257-327: parent f or q (mb) = R(child).
template <int DIM>
__device__ __forceinline__ void u_fill_down(const PatchDev* __restrict__ P, double* __restrict__ pool, const Blk b,
                                            int tid, int nrvars, int field) {
  const PatchDev& p = P[b.patch];
  int ci, cj, ck;
  if (!interior_cell<DIM>(p.cmx, b.start + tid, ci, cj, ck)) return;
  const PatchDev& par = P[p.parent];
  for (int v = 0; v < nrvars; v++) {
    if (field == 1) {
      const double* f = pool + p.of + v * p.sf;
      auto at = [&](int i, int j, int k) { return f[iofs<DIM>(p.mx, i, j, k)]; };
      pool[par.of + v * par.sf + iofs<DIM>(par.mx, p.mb[0] + ci - 1, p.mb[1] + cj - 1, DIM == 3 ? p.mb[2] + ck - 1 : 1)] =
          restrict_at<DIM>(at, ci, cj, ck);
    } else {
      const double* q = pool + p.oq + v * p.sq;
      auto at = [&](int i, int j, int k) { return q[gofs<DIM>(p.qn, i, j, k)]; };
      pool[par.oq + v * par.sq + gofs<DIM>(par.qn, p.mb[0] + ci - 1, p.mb[1] + cj - 1, DIM == 3 ? p.mb[2] + ck - 1 : 0)] =
          restrict_at<DIM>(at, ci, cj, ck);
    }
  }
}
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_fill_down(const PatchDev* __restrict__ P, double* __restrict__ pool,
                                                      const Blk* __restrict__ blk, int nrvars, int field) {
  u_fill_down<DIM>(P, pool, blk[blockIdx.x], threadIdx.x, nrvars, field);
}

// GetSourceFunction, afasroutines.f90:330-381: ftmp = Source(q, qold)
template <int PROB, int DIM>
__global__ void __launch_bounds__(kBlock) k_get_source(const PatchDev* __restrict__ P, double* __restrict__ pool,
                                                       const Blk* __restrict__ blk, ProbParams pp) {
  const Blk b = blk[blockIdx.x];
  const PatchDev& p = P[b.patch];
  int i, j, k;
  if (!interior_cell<DIM>(p.mx, b.start + threadIdx.x, i, j, k)) return;
  double o0 = pool[p.oqold + gofs<DIM>(p.qn, i, j, k)];
  constexpr int NV = PROB == kGrowth ? 3 : 2;
  double s[NV];
  source_eval<PROB, DIM>(o0, pp, s);
  long long fc = iofs<DIM>(p.mx, i, j, k);
  for (int v = 0; v < NV; v++) pool[p.oftmp + v * p.sf + fc] = s[v];
}

// UpdateSourceFunction, afasroutines.f90:438-492: f = ftmp + SourceUpdate
// (SourceUpdate is zero in both plugins).
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_update_source(const PatchDev* __restrict__ P, double* __restrict__ pool,
                                                          const Blk* __restrict__ blk, int nrvars) {
  const Blk b = blk[blockIdx.x];
  const PatchDev& p = P[b.patch];
  int i, j, k;
  if (!interior_cell<DIM>(p.mx, b.start + threadIdx.x, i, j, k)) return;
  long long fc = iofs<DIM>(p.mx, i, j, k);
  for (int v = 0; v < nrvars; v++) pool[p.of + v * p.sf + fc] = pool[p.oftmp + v * p.sf + fc] + 0.0;
}

// ErrorAFAS partial sums (afasroutines.f90:113-233): rf = f - Op(q) on the
// level's patches, per-block sums of rf^2 per variable.
template <int PROB, int DIM>
__global__ void __launch_bounds__(kBlock) k_norm_partial(const PatchDev* __restrict__ P, double* __restrict__ pool,
                                                         const Blk* __restrict__ blk, ProbParams pp,
                                                         double* __restrict__ partial, int store_rf) {
  constexpr int NV = PROB == kGrowth ? 3 : 2;
  __shared__ double red[NV][kBlock / 32];
  const Blk b = blk[blockIdx.x];
  const PatchDev& p = P[b.patch];
  int i, j, k;
  double s[NV];
  for (int v = 0; v < NV; v++) s[v] = 0.0;
  if (interior_cell<DIM>(p.mx, b.start + threadIdx.x, i, j, k)) {
    const double* q = pool + p.oq;
    long long sy = p.qn[0], sz = (long long)p.qn[0] * p.qn[1];
    long long c = gofs<DIM>(p.qn, i, j, k);
    long long fc = iofs<DIM>(p.mx, i, j, k);
    double r[NV];
    op_eval<PROB, DIM>(q, c, sy, sz, p.sq, pool[p.oqold + c], p.c, pp, r);
    for (int v = 0; v < NV; v++) {
      double e = pool[p.of + v * p.sf + fc] - r[v];
      if (store_rf) pool[p.orf + v * p.sf + fc] = e;
      s[v] = e * e;
    }
  }
  for (int o = 16; o > 0; o >>= 1)
    for (int v = 0; v < NV; v++) s[v] = s[v] + __shfl_down_sync(0xffffffffu, s[v], o);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0)
    for (int v = 0; v < NV; v++) red[v][w] = s[v];
  __syncthreads();
  if (threadIdx.x == 0)
    for (int v = 0; v < NV; v++) {
      double t = 0.0;
      for (int n = 0; n < kBlock / 32; n++) t = t + red[v][n];
      partial[NV * blockIdx.x + v] = t;
    }
}

// Final deterministic reduction of the block partials in block order.
// First stage of a long final sum: CTA g adds the partial pairs
// [g*chunk, min((g+1)*chunk, nblk)) in a fixed order and writes one pair to
// stage[2g], stage[2g+1].  Spreading the FP64 additions over many SMs
// matters on GB300, whose FP64 rate is two additions per clock per SM.
constexpr int kStageBlocks = (kNormOutLen - 8) / 3;
template <int NV>
__global__ void __launch_bounds__(kBlock) k_norm_stage(const double* __restrict__ partial, int nblk, int chunk,
                                                       double* __restrict__ stage) {
  __shared__ double red[NV][kBlock];
  int lo = blockIdx.x * chunk, hi = min(lo + chunk, nblk);
  double a[NV];
  for (int v = 0; v < NV; v++) a[v] = 0.0;
  for (int n = lo + threadIdx.x; n < hi; n += kBlock)
    for (int v = 0; v < NV; v++) a[v] = a[v] + partial[NV * n + v];
  for (int v = 0; v < NV; v++) red[v][threadIdx.x] = a[v];
  __syncthreads();
  for (int w = kBlock / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int v = 0; v < NV; v++) red[v][threadIdx.x] = red[v][threadIdx.x] + red[v][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int v = 0; v < NV; v++) stage[NV * blockIdx.x + v] = red[v][0];
}

// One CTA of 1024 threads; each thread keeps eight independent partial sums
// per variable so that eight loads are in flight, then a fixed-shape tree.
// The order of the additions depends only on nblk, so the result is
// deterministic.  Partials hold NV values per block.
constexpr int kFinishThreads = 1024;
template <int NV>
__global__ void __launch_bounds__(kFinishThreads) k_norm_finish(const double* __restrict__ partial, int nblk,
                                                                double count, int errortype, double* out,
                                                                int* nonfinite) {
  __shared__ double red[NV][kFinishThreads / 32];
  double a[NV][8];
  for (int v = 0; v < NV; v++)
    for (int u = 0; u < 8; u++) a[v][u] = 0.0;
  int n = threadIdx.x;
  for (; n + 7 * kFinishThreads < nblk; n += 8 * kFinishThreads)
    for (int u = 0; u < 8; u++)
      for (int v = 0; v < NV; v++) a[v][u] = a[v][u] + partial[NV * (n + u * kFinishThreads) + v];
  // the remaining (at most seven) partials of this thread; a constant index
  // keeps a[][] in registers
  for (; n < nblk; n += kFinishThreads)
    for (int v = 0; v < NV; v++) a[v][0] = a[v][0] + partial[NV * n + v];
  double t[NV];
  for (int v = 0; v < NV; v++)
    t[v] = ((a[v][0] + a[v][1]) + (a[v][2] + a[v][3])) + ((a[v][4] + a[v][5]) + (a[v][6] + a[v][7]));
  for (int o = 16; o > 0; o >>= 1)
    for (int v = 0; v < NV; v++) t[v] = t[v] + __shfl_down_sync(0xffffffffu, t[v], o);
  int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0)
    for (int v = 0; v < NV; v++) red[v][w] = t[v];
  __syncthreads();
  if (w == 0) {
    for (int v = 0; v < NV; v++) t[v] = red[v][threadIdx.x];
    for (int o = 16; o > 0; o >>= 1)
      for (int v = 0; v < NV; v++) t[v] = t[v] + __shfl_down_sync(0xffffffffu, t[v], o);
    if (threadIdx.x == 0)
      for (int v = 0; v < NV; v++) red[v][0] = t[v];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double sum = red[0][0];
    for (int v = 1; v < NV; v++) sum = sum + red[v][0];
    double r;
    if (errortype == 1) {
      r = sqrt(sum / count);  // integralresult(1)/integralresult(2), :135
    } else {
      double cells = count / NV;
      r = sqrt(red[0][0] / cells);
      for (int v = 1; v < NV; v++) {  // MAXVAL of component errors, :146-153
        double e = sqrt(red[v][0] / cells);
        r = e > r ? e : r;
      }
    }
    out[0] = r;
    out[1] = sum;
    if (nonfinite) nonfinite[0] = isfinite(r) ? 0 : 1;
  }
}

// ---------------------------------------------------------------------------
// Ghost programs (SetGhost, boundary.f90:67-97): one thread per operation,
// all variables of the cell.

__device__ __forceinline__ void ghost_apply(const PatchDev* __restrict__ P, double* __restrict__ pool,
                                            const GhostOp& g, const ProbParams& pp) {
  const PatchDev& d = P[g.dp];
  const PatchDev& s = P[g.sp];
  for (int v = 0; v < pp.nrvars; v++) {
    double* dq = pool + d.oq + v * d.sq;
    const double* sq = pool + s.oq + v * s.sq;
    double val;
    switch (g.type) {
      case kGCopy: val = sq[g.s0]; break;
      case kGCopyAdd: val = sq[g.s0] + pp.qpo[v]; break;
      case kGCopySub: val = sq[g.s0] - pp.qpo[v]; break;
      case kGBC: val = ((g.mask >> v) & 1) ? 2.0 - sq[g.s0] : (((g.mask >> (8 + v)) & 1) ? -sq[g.s0] : sq[g.s0]); break;
      case kGCfA: val = kA1 * dq[g.s0] + kA2 * dq[g.s1] + kA3 * sq[g.c0]; break;
      case kGCfAB:
        val = kA1 * dq[g.s0] + kA2 * dq[g.s1] + kA3 * (kB1 * sq[g.c0] + kB2 * sq[g.c1] + kB3 * sq[g.c2]);
        break;
      default:
        val = kA1 * dq[g.s0] + kA2 * dq[g.s1] +
              kA3 * (kC1 * sq[g.c0] + kC2 * sq[g.c1] + kC3 * sq[g.c2] + kC4 * sq[g.c3]);
        break;
    }
    dq[g.dcell] = val;
  }
}

__global__ void __launch_bounds__(kBlock) k_ghost_stage(const PatchDev* __restrict__ P, double* __restrict__ pool,
                                                        const GhostOp* __restrict__ ops, int n, ProbParams pp) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  GhostOp g = ops[t];
  ghost_apply(P, pool, g, pp);
}

// whole program in one block: stages separated by __syncthreads
__global__ void __launch_bounds__(kBlock) k_ghost_program(const PatchDev* __restrict__ P, double* __restrict__ pool,
                                                          const GhostOp* __restrict__ ops,
                                                          const int* __restrict__ stage_off, int nstages,
                                                          ProbParams pp) {
  for (int s = 0; s < nstages; s++) {
    int lo = stage_off[s], hi = stage_off[s + 1];
    for (int t = lo + threadIdx.x; t < hi; t += blockDim.x) {
      GhostOp g = ops[t];
      ghost_apply(P, pool, g, pp);
    }
    __syncthreads();
  }
}

// The coarse tail of the V-cycle in one block (see TailPhase): the
// operations the separate launches would run, phase by phase, each phase's
// work-list blocks executed in turn by the block's 256 threads with a
// barrier between phases.  Per-cell arithmetic and the order of dependent
// updates are those of the separate kernels, so results are bit-identical.
template <int PROB, int DIM>
__device__ __forceinline__ void run_tail(const PatchDev* __restrict__ P, double* pool, const TailPhase* __restrict__ ph,
                                         int nph, const ProbParams& pp) {
  for (int x = 0; x < nph; x++) {
    const TailPhase f = ph[x];
    if (f.op == kTGhost) {
      for (int s = 0; s < f.nstages; s++) {
        for (int t = f.stage_off[s] + threadIdx.x; t < f.stage_off[s + 1]; t += blockDim.x) {
          GhostOp g = f.ops[t];
          ghost_apply(P, pool, g, pp);
        }
        __syncthreads();
      }
      continue;
    }
    for (int b = 0; b < f.nblk; b++) {
      const Blk bb = f.blk[b];
      switch (f.op) {
        case kTRelax: u_relax<PROB, DIM>(P, pool, bb, threadIdx.x, f.arg, pp); break;
        case kTRestrict: u_restrict_q<DIM>(P, pool, bb, threadIdx.x, pp.nrvars); break;
        case kTRing:
          if (f.arg) u_correct_a<DIM>(P, pool, bb, threadIdx.x, pp.nrvars);
          else u_coarse_ghost<DIM>(P, pool, bb, threadIdx.x, pp.nrvars);
          break;
        case kTLoad: u_coarse_load<PROB, DIM>(P, pool, bb, threadIdx.x, pp); break;
        case kTFill: u_fill_down<DIM>(P, pool, bb, threadIdx.x, pp.nrvars, f.arg); break;
        default: u_correct_b<DIM>(P, pool, bb, threadIdx.x, pp.nrvars); break;
      }
    }
    __syncthreads();
  }
}

template <int PROB, int DIM>
__global__ void __launch_bounds__(kBlock) k_tail(const PatchDev* __restrict__ P, double* __restrict__ pool,
                                                 const TailPhase* __restrict__ ph, int nph, ProbParams pp) {
  run_tail<PROB, DIM>(P, pool, ph, nph, pp);
}

// The same with the tail levels' arrays staged in shared memory (P
// addresses them there); modified arrays are written back at the end.
template <int PROB, int DIM>
__global__ void __launch_bounds__(kBlock) k_tail_smem(const PatchDev* __restrict__ P, double* __restrict__ pool,
                                                      const TailPhase* __restrict__ ph, int nph, ProbParams pp,
                                                      const StageSeg* __restrict__ segs, int nsegs) {
  extern __shared__ double smd[];
  for (int x = 0; x < nsegs; x++) {
    const StageSeg sg = segs[x];
    for (int t = threadIdx.x; t < sg.n; t += blockDim.x) smd[sg.s + t] = pool[sg.g + t];
  }
  __syncthreads();
  run_tail<PROB, DIM>(P, smd, ph, nph, pp);
  for (int x = 0; x < nsegs; x++) {
    const StageSeg sg = segs[x];
    if (!sg.out) continue;
    for (int t = threadIdx.x; t < sg.n; t += blockDim.x) pool[sg.g + t] = smd[sg.s + t];
  }
}

// ---------------------------------------------------------------------------
// launchers

#define DISPATCH_DIM(c, KER, ...)                            \
  do {                                                       \
    if ((c).ndims == 2) KER<2><<<nblk, kBlock, 0, (c).s>>>(__VA_ARGS__); \
    else KER<3><<<nblk, kBlock, 0, (c).s>>>(__VA_ARGS__);    \
  } while (0)

#define DISPATCH_PD(c, KER, ...)                                                      \
  do {                                                                                \
    if ((c).pp.problem == kCH) {                                                      \
      if ((c).ndims == 2) KER<kCH, 2><<<nblk, kBlock, 0, (c).s>>>(__VA_ARGS__);       \
      else KER<kCH, 3><<<nblk, kBlock, 0, (c).s>>>(__VA_ARGS__);                      \
    } else if ((c).pp.problem == kBio) {                                              \
      if ((c).ndims == 2) KER<kBio, 2><<<nblk, kBlock, 0, (c).s>>>(__VA_ARGS__);      \
      else KER<kBio, 3><<<nblk, kBlock, 0, (c).s>>>(__VA_ARGS__);                     \
    } else {                                                                          \
      if ((c).ndims == 2) KER<kGrowth, 2><<<nblk, kBlock, 0, (c).s>>>(__VA_ARGS__);   \
      else KER<kGrowth, 3><<<nblk, kBlock, 0, (c).s>>>(__VA_ARGS__);                  \
    }                                                                                 \
  } while (0)

int launch_relax(const LaunchCtx& c, const Blk* blk, int nblk, int ipass) {
  if (nblk <= 0) return 0;
  DISPATCH_PD(c, k_relax, c.P, c.pool, blk, ipass, c.pp);
  return 1;
}
int launch_restrict_q(const LaunchCtx& c, const Blk* blk, int nblk) {
  if (nblk <= 0) return 0;
  DISPATCH_DIM(c, k_restrict_q, c.P, c.pool, blk, c.pp.nrvars);
  return 1;
}
int launch_coarse_ghost(const LaunchCtx& c, const Blk* blk, int nblk) {
  if (nblk <= 0) return 0;
  DISPATCH_DIM(c, k_coarse_ghost, c.P, c.pool, blk, c.pp.nrvars);
  return 1;
}
int launch_coarse_load(const LaunchCtx& c, const Blk* blk, int nblk) {
  if (nblk <= 0) return 0;
  DISPATCH_PD(c, k_coarse_load, c.P, c.pool, blk, c.pp);
  return 1;
}
int launch_correct_a(const LaunchCtx& c, const Blk* blk, int nblk) {
  if (nblk <= 0) return 0;
  DISPATCH_DIM(c, k_correct_a, c.P, c.pool, blk, c.pp.nrvars);
  return 1;
}
int launch_qc_from_parent(const LaunchCtx& c, const Blk* blk, int nblk) {
  if (nblk <= 0) return 0;
  DISPATCH_DIM(c, k_qc_from_parent, c.P, c.pool, blk, c.pp.nrvars);
  return 1;
}
int launch_correct_b(const LaunchCtx& c, const Blk* blk, int nblk) {
  if (nblk <= 0) return 0;
  DISPATCH_DIM(c, k_correct_b, c.P, c.pool, blk, c.pp.nrvars);
  return 1;
}
int launch_fill_down(const LaunchCtx& c, const Blk* blk, int nblk, int field) {
  if (nblk <= 0) return 0;
  DISPATCH_DIM(c, k_fill_down, c.P, c.pool, blk, c.pp.nrvars, field);
  return 1;
}
int launch_get_source(const LaunchCtx& c, const Blk* blk, int nblk) {
  if (nblk <= 0) return 0;
  DISPATCH_PD(c, k_get_source, c.P, c.pool, blk, c.pp);
  return 1;
}
int launch_update_source(const LaunchCtx& c, const Blk* blk, int nblk) {
  if (nblk <= 0) return 0;
  DISPATCH_DIM(c, k_update_source, c.P, c.pool, blk, c.pp.nrvars);
  return 1;
}
int launch_norm_partial(const LaunchCtx& c, const Blk* blk, int nblk, double* partial, int store_rf) {
  if (nblk <= 0) return 0;
  DISPATCH_PD(c, k_norm_partial, c.P, c.pool, blk, c.pp, partial, store_rf);
  return 1;
}
int launch_norm_finish(cudaStream_t s, const double* partial, int nblk, int nrvars, double count, int errortype,
                       double* out, int* nonfinite) {
  int n = 1;
  if (nblk > 2048) {
    // two stages; out[8 ..] holds the stage sums
    int g = std::min(kStageBlocks, (nblk + 511) / 512);
    int chunk = (nblk + g - 1) / g;
    g = (nblk + chunk - 1) / chunk;
    if (nrvars == 3) k_norm_stage<3><<<g, kBlock, 0, s>>>(partial, nblk, chunk, out + 8);
    else k_norm_stage<2><<<g, kBlock, 0, s>>>(partial, nblk, chunk, out + 8);
    partial = out + 8;
    nblk = g;
    n = 2;
  }
  if (nrvars == 3) k_norm_finish<3><<<1, kFinishThreads, 0, s>>>(partial, nblk, count, errortype, out, nonfinite);
  else k_norm_finish<2><<<1, kFinishThreads, 0, s>>>(partial, nblk, count, errortype, out, nonfinite);
  return n;
}
int launch_ghost_stage(const LaunchCtx& c, const GhostOp* ops, int n) {
  if (n <= 0) return 0;
  int nb = (n + kBlock - 1) / kBlock;
  k_ghost_stage<<<nb, kBlock, 0, c.s>>>(c.P, c.pool, ops, n, c.pp);
  return 1;
}
int launch_ghost_program_1cta(const LaunchCtx& c, const GhostOp* ops, const int* stage_off, int nstages) {
  if (nstages <= 0) return 0;
  k_ghost_program<<<1, kBlock, 0, c.s>>>(c.P, c.pool, ops, stage_off, nstages, c.pp);
  return 1;
}
int launch_tail(const LaunchCtx& c, const TailPhase* ph, int nph) {
  if (nph <= 0) return 0;
  const int nblk = 1;
  DISPATCH_PD(c, k_tail, c.P, c.pool, ph, nph, c.pp);
  return 1;
}

#define DISPATCH_PD_SMEM(c, SMEM, KER, ...)                                            \
  do {                                                                                 \
    if ((c).pp.problem == kCH) {                                                       \
      if ((c).ndims == 2) KER<kCH, 2><<<1, kBlock, SMEM, (c).s>>>(__VA_ARGS__);        \
      else KER<kCH, 3><<<1, kBlock, SMEM, (c).s>>>(__VA_ARGS__);                       \
    } else if ((c).pp.problem == kBio) {                                               \
      if ((c).ndims == 2) KER<kBio, 2><<<1, kBlock, SMEM, (c).s>>>(__VA_ARGS__);       \
      else KER<kBio, 3><<<1, kBlock, SMEM, (c).s>>>(__VA_ARGS__);                      \
    } else {                                                                           \
      if ((c).ndims == 2) KER<kGrowth, 2><<<1, kBlock, SMEM, (c).s>>>(__VA_ARGS__);    \
      else KER<kGrowth, 3><<<1, kBlock, SMEM, (c).s>>>(__VA_ARGS__);                   \
    }                                                                                  \
  } while (0)

int launch_tail_smem(const LaunchCtx& c, const PatchDev* shadow, const TailPhase* ph, int nph, const StageSeg* segs,
                     int nsegs, int smem_bytes) {
  if (nph <= 0) return 0;
  DISPATCH_PD_SMEM(c, smem_bytes, k_tail_smem, shadow, c.pool, ph, nph, c.pp, segs, nsegs);
  return 1;
}

int tail_smem_attributes() {
  const int m = kTailSmemMax;
  const cudaFuncAttribute a = cudaFuncAttributeMaxDynamicSharedMemorySize;
  cudaError_t e = cudaFuncSetAttribute(k_tail_smem<kCH, 2>, a, m);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_tail_smem<kCH, 3>, a, m);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_tail_smem<kBio, 2>, a, m);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_tail_smem<kBio, 3>, a, m);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_tail_smem<kGrowth, 2>, a, m);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_tail_smem<kGrowth, 3>, a, m);
  return e == cudaSuccess ? 0 : -1;
}

}  // namespace bsamg
