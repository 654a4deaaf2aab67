// Device code of the plain FP64 path shared by the library (fp64.cu) and the
// FP64 part of every problem plugin (plugins/<name>.cu): the per-unit
// operations of the V-cycle and the kernels that depend on the plugin,
// templates over the plugin struct (plugin.h).
//
// Every translation unit that includes this file is compiled with
// --fmad=false: each product and sum is rounded separately, in the
// evaluation order of the reference Fortran, so results agree bit for bit
// with a reference build that does not contract multiply-adds (the CPU
// oracle is built that way).  Division is the IEEE round-to-nearest `/`.
#pragma once
#include <cuda_runtime.h>

#include "cellops.cuh"
#include "launch.h"
#include "plugin.h"

namespace bsamg {

// C/F interpolation weights, LIBRARY/boundary.f90:54-63
constexpr double kA1 = -01.0 / 05.0;
constexpr double kA2 = 02.0 / 03.0;
constexpr double kA3 = 08.0 / 15.0;
constexpr double kB1 = 05.0 / 32.0;
constexpr double kB2 = 15.0 / 16.0;
constexpr double kB3 = -03.0 / 32.0;
constexpr double kC1 = 09.0 / 16.0;
constexpr double kC2 = 03.0 / 16.0;
constexpr double kC3 = 03.0 / 16.0;
constexpr double kC4 = 01.0 / 16.0;

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

// ---------------------------------------------------------------------------
// The plugin-dependent operations: templates over the plugin struct PL.

// Red-black pointwise relaxation of one colour (RelaxPatch,
// afasroutines.f90:560-607, calling the plugin's RelaxGrid2D/3D on the
// cells of colour ipass).
template <class PL, int DIM>
__device__ __forceinline__ void u_relax(const PatchDev* __restrict__ P, double* __restrict__ pool, const Blk b,
                                        int tid, int ipass, const ProbParams& pp) {
  const PatchDev& p = P[b.patch];
  int i, j, k;
  if (!color_cell<DIM>(p, b.start + tid, ipass, i, j, k)) return;
  Cell64 x;
  x.q = pool + p.oq;
  x.f = pool + p.of;
  x.qold = pool + p.oqold;
  x.c = gofs<DIM>(p.qn, i, j, k);
  x.fc = iofs<DIM>(p.mx, i, j, k);
  x.sy = p.qn[0];
  x.sz = (long long)p.qn[0] * p.qn[1];
  x.sq = p.sq;
  x.sf = p.sf;
  PL::template relax<DIM>(x, p.c, pp);
}
template <class PL, int DIM>
__global__ void __launch_bounds__(kBlock) k_relax(const PatchDev* __restrict__ P, double* __restrict__ pool,
                                                  const Blk* __restrict__ blk, int ipass, ProbParams pp) {
  u_relax<PL, DIM>(P, pool, blk[blockIdx.x], threadIdx.x, ipass, pp);
}

// CoarseLoadingFunction, afasroutines.f90:673-736, with Residual (:817-857):
// rf = f - Op_h(q) on the children of a coarse cell;
// parent f(mb) = R(rf) + Op_2h(qc, parent qold, h_parent).
template <class PL, int DIM>
__device__ __forceinline__ void u_coarse_load(const PatchDev* __restrict__ P, double* __restrict__ pool, const Blk b,
                                              int tid, const ProbParams& pp) {
  const PatchDev& p = P[b.patch];
  int ci, cj, ck;
  if (!interior_cell<DIM>(p.cmx, b.start + tid, ci, cj, ck)) return;
  const PatchDev& par = P[p.parent];
  const double* q = pool + p.oq;
  const double* qo = pool + p.oqold;
  long long sy = p.qn[0], sz = (long long)p.qn[0] * p.qn[1];
  constexpr int NV = PL::kNV;
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
        PL::template op<DIM>(q, c, sy, sz, p.sq, QoldView{qo + c, sy, sz, p.sq}, p.c, pp, r);
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
  QoldView po{pool + par.oqold + pc, par.qn[0], (long long)par.qn[0] * par.qn[1], par.sq};
  double cr[NV];
  PL::template op<DIM>(qc, cc, csy, csz, p.sc, po, par.c, pp, cr);
  long long pf = iofs<DIM>(par.mx, p.mb[0] + ci - 1, p.mb[1] + cj - 1, DIM == 3 ? p.mb[2] + ck - 1 : 1);
  for (int v = 0; v < NV; v++) pool[par.of + v * par.sf + pf] = R[v] + cr[v];
}
template <class PL, int DIM>
__global__ void __launch_bounds__(kBlock) k_coarse_load(const PatchDev* __restrict__ P, double* __restrict__ pool,
                                                        const Blk* __restrict__ blk, ProbParams pp) {
  u_coarse_load<PL, DIM>(P, pool, blk[blockIdx.x], threadIdx.x, pp);
}

// GetSourceFunction, afasroutines.f90:330-381: ftmp = Source(q, qold)
template <class PL, int DIM>
__global__ void __launch_bounds__(kBlock) k_get_source(const PatchDev* __restrict__ P, double* __restrict__ pool,
                                                       const Blk* __restrict__ blk, ProbParams pp) {
  const Blk b = blk[blockIdx.x];
  const PatchDev& p = P[b.patch];
  int i, j, k;
  if (!interior_cell<DIM>(p.mx, b.start + threadIdx.x, i, j, k)) return;
  long long c = gofs<DIM>(p.qn, i, j, k), sy = p.qn[0], sz = (long long)p.qn[0] * p.qn[1];
  constexpr int NV = PL::kNV;
  double s[NV];
  PL::template source<DIM>(pool + p.oq, c, sy, sz, p.sq, QoldView{pool + p.oqold + c, sy, sz, p.sq}, p.c, pp, s);
  long long fc = iofs<DIM>(p.mx, i, j, k);
  for (int v = 0; v < NV; v++) pool[p.oftmp + v * p.sf + fc] = s[v];
}

// UpdateSourceFunction, afasroutines.f90:438-492: f = ftmp + SourceUpdate
template <class PL, int DIM>
__global__ void __launch_bounds__(kBlock) k_update_source(const PatchDev* __restrict__ P, double* __restrict__ pool,
                                                          const Blk* __restrict__ blk, ProbParams pp) {
  const Blk b = blk[blockIdx.x];
  const PatchDev& p = P[b.patch];
  int i, j, k;
  if (!interior_cell<DIM>(p.mx, b.start + threadIdx.x, i, j, k)) return;
  constexpr int NV = PL::kNV;
  long long c = gofs<DIM>(p.qn, i, j, k), sy = p.qn[0], sz = (long long)p.qn[0] * p.qn[1];
  double su[NV];
  PL::template source_update<DIM>(pool + p.oq, c, sy, sz, p.sq, QoldView{pool + p.oqold + c, sy, sz, p.sq}, p.c,
                                  pp, su);
  long long fc = iofs<DIM>(p.mx, i, j, k);
  for (int v = 0; v < NV; v++) pool[p.of + v * p.sf + fc] = pool[p.oftmp + v * p.sf + fc] + su[v];
}

// ErrorAFAS partial sums (afasroutines.f90:113-233): rf = f - Op(q) on the
// level's patches, sums of rf^2 per variable over kNormGroup consecutive
// blocks of the work list per CTA (each thread adds its cells in block
// order, then one fixed reduction tree).
template <class PL, int DIM>
__global__ void __launch_bounds__(kBlock) k_norm_partial(const PatchDev* __restrict__ P, double* __restrict__ pool,
                                                         const Blk* __restrict__ blk, int nblk, ProbParams pp,
                                                         double* __restrict__ partial, int store_rf) {
  constexpr int NV = PL::kNV;
  __shared__ double red[NV][kBlock / 32];
  double s[NV];
  for (int v = 0; v < NV; v++) s[v] = 0.0;
  for (int sub = 0; sub < kNormGroup; sub++) {
    int bi = blockIdx.x * kNormGroup + sub;
    if (bi >= nblk) break;
    const Blk b = blk[bi];
    const PatchDev& p = P[b.patch];
    int i, j, k;
    if (!interior_cell<DIM>(p.mx, b.start + threadIdx.x, i, j, k)) continue;
    const double* q = pool + p.oq;
    long long sy = p.qn[0], sz = (long long)p.qn[0] * p.qn[1];
    long long c = gofs<DIM>(p.qn, i, j, k);
    long long fc = iofs<DIM>(p.mx, i, j, k);
    double r[NV];
    PL::template op<DIM>(q, c, sy, sz, p.sq, QoldView{pool + p.oqold + c, sy, sz, p.sq}, p.c, pp, r);
    for (int v = 0; v < NV; v++) {
      double e = pool[p.of + v * p.sf + fc] - r[v];
      if (store_rf) pool[p.orf + v * p.sf + fc] = e;
      s[v] = s[v] + e * e;
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

// The coarse tail of the V-cycle in one block (see TailPhase): the
// operations the separate launches would run, phase by phase, each phase's
// work-list blocks executed in turn by the block's 256 threads with a
// barrier between phases.  Per-cell arithmetic and the order of dependent
// updates are those of the separate kernels, so results are bit-identical.
template <class PL, int DIM>
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
        case kTRelax: u_relax<PL, DIM>(P, pool, bb, threadIdx.x, f.arg, pp); break;
        case kTRestrict: u_restrict_q<DIM>(P, pool, bb, threadIdx.x, pp.nrvars); break;
        case kTRing:
          if (f.arg) u_correct_a<DIM>(P, pool, bb, threadIdx.x, pp.nrvars);
          else u_coarse_ghost<DIM>(P, pool, bb, threadIdx.x, pp.nrvars);
          break;
        case kTLoad: u_coarse_load<PL, DIM>(P, pool, bb, threadIdx.x, pp); break;
        case kTFill: u_fill_down<DIM>(P, pool, bb, threadIdx.x, pp.nrvars, f.arg); break;
        default: u_correct_b<DIM>(P, pool, bb, threadIdx.x, pp.nrvars); break;
      }
    }
    __syncthreads();
  }
}

template <class PL, int DIM>
__global__ void __launch_bounds__(kBlock) k_tail(const PatchDev* __restrict__ P, double* __restrict__ pool,
                                                 const TailPhase* __restrict__ ph, int nph, ProbParams pp) {
  run_tail<PL, DIM>(P, pool, ph, nph, pp);
}

// The same with the tail levels' arrays staged in shared memory (P
// addresses them there); modified arrays are written back at the end.
template <class PL, int DIM>
__global__ void __launch_bounds__(kBlock) k_tail_smem(const PatchDev* __restrict__ P, double* __restrict__ pool,
                                                      const TailPhase* __restrict__ ph, int nph, ProbParams pp,
                                                      const StageSeg* __restrict__ segs, int nsegs) {
  extern __shared__ double smd[];
  for (int x = 0; x < nsegs; x++) {
    const StageSeg sg = segs[x];
    for (int t = threadIdx.x; t < sg.n; t += blockDim.x) smd[sg.s + t] = pool[sg.g + t];
  }
  __syncthreads();
  run_tail<PL, DIM>(P, smd, ph, nph, pp);
  for (int x = 0; x < nsegs; x++) {
    const StageSeg sg = segs[x];
    if (!sg.out) continue;
    for (int t = threadIdx.x; t < sg.n; t += blockDim.x) pool[sg.g + t] = smd[sg.s + t];
  }
}

// The launchers of one plugin's FP64 kernels (the table the plugin registers)
template <class PL>
struct Fp64Launchers {
  static int relax(const LaunchCtx& c, const Blk* blk, int nblk, int ipass) {
    if (nblk <= 0) return 0;
    if (c.ndims == 2) k_relax<PL, 2><<<nblk, kBlock, 0, c.s>>>(c.P, c.pool, blk, ipass, c.pp);
    else k_relax<PL, 3><<<nblk, kBlock, 0, c.s>>>(c.P, c.pool, blk, ipass, c.pp);
    return 1;
  }
  static int coarse_load(const LaunchCtx& c, const Blk* blk, int nblk) {
    if (nblk <= 0) return 0;
    if (c.ndims == 2) k_coarse_load<PL, 2><<<nblk, kBlock, 0, c.s>>>(c.P, c.pool, blk, c.pp);
    else k_coarse_load<PL, 3><<<nblk, kBlock, 0, c.s>>>(c.P, c.pool, blk, c.pp);
    return 1;
  }
  static int update_source(const LaunchCtx& c, const Blk* blk, int nblk) {
    if (nblk <= 0) return 0;
    if (c.ndims == 2) k_update_source<PL, 2><<<nblk, kBlock, 0, c.s>>>(c.P, c.pool, blk, c.pp);
    else k_update_source<PL, 3><<<nblk, kBlock, 0, c.s>>>(c.P, c.pool, blk, c.pp);
    return 1;
  }
  static int norm_partial(const LaunchCtx& c, const Blk* blk, int nblk, double* partial, int store_rf) {
    if (nblk <= 0) return 0;
    int g = norm_partials(nblk);
    if (c.ndims == 2) k_norm_partial<PL, 2><<<g, kBlock, 0, c.s>>>(c.P, c.pool, blk, nblk, c.pp, partial, store_rf);
    else k_norm_partial<PL, 3><<<g, kBlock, 0, c.s>>>(c.P, c.pool, blk, nblk, c.pp, partial, store_rf);
    return 1;
  }
  static int get_source(const LaunchCtx& c, const Blk* blk, int nblk) {
    if (nblk <= 0) return 0;
    if (c.ndims == 2) k_get_source<PL, 2><<<nblk, kBlock, 0, c.s>>>(c.P, c.pool, blk, c.pp);
    else k_get_source<PL, 3><<<nblk, kBlock, 0, c.s>>>(c.P, c.pool, blk, c.pp);
    return 1;
  }
  static int tail(const LaunchCtx& c, const TailPhase* ph, int nph) {
    if (nph <= 0) return 0;
    if (c.ndims == 2) k_tail<PL, 2><<<1, kBlock, 0, c.s>>>(c.P, c.pool, ph, nph, c.pp);
    else k_tail<PL, 3><<<1, kBlock, 0, c.s>>>(c.P, c.pool, ph, nph, c.pp);
    return 1;
  }
  static int tail_smem(const LaunchCtx& c, const PatchDev* shadow, const TailPhase* ph, int nph,
                       const StageSeg* segs, int nsegs, int smem_bytes) {
    if (nph <= 0) return 0;
    if (c.ndims == 2)
      k_tail_smem<PL, 2><<<1, kBlock, smem_bytes, c.s>>>(shadow, c.pool, ph, nph, c.pp, segs, nsegs);
    else
      k_tail_smem<PL, 3><<<1, kBlock, smem_bytes, c.s>>>(shadow, c.pool, ph, nph, c.pp, segs, nsegs);
    return 1;
  }
  static int tail_smem_attributes() {
    const cudaFuncAttribute a = cudaFuncAttributeMaxDynamicSharedMemorySize;
    cudaError_t e = cudaFuncSetAttribute(k_tail_smem<PL, 2>, a, kTailSmemMax);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_tail_smem<PL, 3>, a, kTailSmemMax);
    return e == cudaSuccess ? 0 : -1;
  }
};

template <class PL>
const PluginFp64* fp64_ops() {
  static const PluginFp64 ops = {&Fp64Launchers<PL>::relax,        &Fp64Launchers<PL>::coarse_load,
                                 &Fp64Launchers<PL>::norm_partial, &Fp64Launchers<PL>::get_source,
                                 &Fp64Launchers<PL>::update_source, &Fp64Launchers<PL>::tail,
                                 &Fp64Launchers<PL>::tail_smem,    &Fp64Launchers<PL>::tail_smem_attributes};
  return &ops;
}

}  // namespace bsamg
