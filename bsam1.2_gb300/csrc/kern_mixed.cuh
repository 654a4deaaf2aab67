// Device code of the mixed-precision path shared by the library (mixed.cu)
// and the mixed part of every problem plugin that has a correction form
// (plugins/<name>.cu): the per-unit operations of the FP32 correction
// V-cycle and the kernels that depend on the plugin, templates over the
// plugin struct (plugin.h).  Compiled with the default --fmad=true: the
// correction cycle needs FP32 accuracy, not the reference's rounding.
#pragma once
#include <cuda_runtime.h>

#include "cellops.cuh"
#include "launch.h"
#include "plugin.h"

namespace bsamg {
namespace mx {

// The dynamic shared memory of a one-launch solve (kern_solve.cuh): its
// FP32 data area first, then the staged program image.
extern __shared__ __align__(16) unsigned char solve_smem[];

// The base of patch p's FP32 arrays: the FP32 pool, or -- inside a
// one-launch solve (CL), for a patch whose arrays live in distributed
// shared memory -- the data area of the CTA of the cluster that owns it.
template <bool CL>
__device__ __forceinline__ float* fbase(float* fpool, const PatchDev& p) {
  if constexpr (CL) {
    if (p.dsm) {
      unsigned me;
      asm("mov.u32 %0, %%cluster_ctarank;" : "=r"(me));
      // this CTA's own data through the local window, another's through the cluster's
      if ((unsigned)p.owner == me) return reinterpret_cast<float*>(solve_smem);
      return static_cast<float*>(__cluster_map_shared_rank(static_cast<void*>(solve_smem), p.owner));
    }
  }
  return fpool;
}

constexpr float fA1 = -01.0f / 05.0f, fA2 = 02.0f / 03.0f, fA3 = 08.0f / 15.0f;
constexpr float fB1 = 05.0f / 32.0f, fB2 = 15.0f / 16.0f, fB3 = -03.0f / 32.0f;
constexpr float fC1 = 09.0f / 16.0f, fC2 = 03.0f / 16.0f, fC3 = 03.0f / 16.0f, fC4 = 01.0f / 16.0f;

template <int DIM, typename F>
__device__ __forceinline__ float restrict_at32(F at, int ci, int cj, int ck) {
  int i = 2 * ci, j = 2 * cj;
  if (DIM == 2) return 0.25f * (at(i, j, 1) + at(i - 1, j, 1) + at(i, j - 1, 1) + at(i - 1, j - 1, 1));
  int k = 2 * ck;
  return 0.125f * (at(i, j, k) + at(i - 1, j, k) + at(i, j - 1, k) + at(i - 1, j - 1, k) + at(i, j, k - 1) +
                   at(i - 1, j, k - 1) + at(i, j - 1, k - 1) + at(i - 1, j - 1, k - 1));
}

// RestrictSolution on e: ec(1:cmx) = R(e); parent e(mb) = ec
template <int DIM, bool CL = false>
__device__ __forceinline__ void u_restrict(const PatchDev* __restrict__ P, float* __restrict__ fpool, const Blk b,
                                           int tid, int nrvars) {
  const PatchDev& p = P[b.patch];
  int ci, cj, ck;
  if (!interior_cell<DIM>(p.cmx, b.start + tid, ci, cj, ck)) return;
  const PatchDev& par = P[p.parent];
  float* fp = fbase<CL>(fpool, p);
  float* fq = fbase<CL>(fpool, par);
  for (int v = 0; v < nrvars; v++) {
    const float* e = fp + p.eq + v * p.sq;
    auto at = [&](int i, int j, int k) { return e[gofs<DIM>(p.qn, i, j, k)]; };
    float val = restrict_at32<DIM>(at, ci, cj, ck);
    fp[p.ecq + v * p.sc + gofs<DIM>(p.cn, ci, cj, ck)] = val;
    fq[par.eq + v * par.sq + gofs<DIM>(par.qn, p.mb[0] + ci - 1, p.mb[1] + cj - 1, DIM == 3 ? p.mb[2] + ck - 1 : 0)] =
        val;
  }
}


// GetCoarseGhostPoints on e (ring of ec <- parent e) when corr == 0;
// CorrectFine step 1 (ec = parent e - ec over the whole ghosted ec) when
// corr == 1.
template <int DIM, bool CL = false>
__device__ __forceinline__ void u_coarse_ring(const PatchDev* __restrict__ P, float* __restrict__ fpool, const Blk b,
                                              int tid, int nrvars, int corr) {
  const PatchDev& p = P[b.patch];
  int i, j, k;
  if (!ghosted_cell<DIM>(p.cn, p.gs, b.start + tid, i, j, k)) return;
  // the correction cycle keeps one ghost layer whatever mbc is: its
  // operators read one layer, and its second layer of e stays zero
  if (i < 0 || i > p.cmx[0] + 1 || j < 0 || j > p.cmx[1] + 1 || (DIM == 3 && (k < 0 || k > p.cmx[2] + 1))) return;
  if (!corr) {
    bool ring = i == 0 || i == p.cmx[0] + 1 || j == 0 || j == p.cmx[1] + 1 ||
                (DIM == 3 && (k == 0 || k == p.cmx[2] + 1));
    if (!ring) return;
  }
  const PatchDev& par = P[p.parent];
  int pi = p.mb[0] - 1 + i, pj = p.mb[1] - 1 + j, pk = DIM == 3 ? p.mb[2] - 1 + k : 0;
  long long src = gofs<DIM>(par.qn, pi, pj, pk);
  long long dst = gofs<DIM>(p.cn, i, j, k);
  float* fp = fbase<CL>(fpool, p);
  const float* fq = fbase<CL>(fpool, par);
  for (int v = 0; v < nrvars; v++) {
    float* ec = fp + p.ecq + v * p.sc;
    float pv = fq[par.eq + v * par.sq + src];
    ec[dst] = corr ? pv - ec[dst] : pv;
  }
}


// CorrectFine step 2 on e: e(0:mx+1) += P(ec).
// One thread per coarse index (ci,cj,ck) in 0..cmx: it produces the fine
// cells 2ci..2ci+1 (x) etc. from the 2x2(x2) coarse values they share, with
// the same per-direction (3,1)/4 weights as BiLin/TriLinProlongationP1
// (gridutilities.f90:156-195, :510-566).
template <int DIM, bool CL = false>
__device__ __forceinline__ void u_prolong(const PatchDev* __restrict__ P, float* __restrict__ fpool, const Blk b,
                                          int tid, int nrvars) {
  const PatchDev& p = P[b.patch];
  // the units cover coarse indices -gs..cmx+gs (as CorrectFine's); the
  // correction cycle prolongs over one ghost layer (0..cmx)
  const int gs = p.gs;
  int cpn[3] = {p.cmx[0] + 1 + 2 * gs, p.cmx[1] + 1 + 2 * gs, DIM == 3 ? p.cmx[2] + 1 + 2 * gs : 1};
  int t = b.start + tid;
  int ci = t % cpn[0], r = t / cpn[0];
  int cj = r % cpn[1], ck = r / cpn[1];
  if (ck >= cpn[2]) return;
  ci -= gs;
  cj -= gs;
  if (DIM == 3) ck -= gs;
  if (ci < 0 || ci > p.cmx[0] || cj < 0 || cj > p.cmx[1] || (DIM == 3 && (ck < 0 || ck > p.cmx[2]))) return;
  const int nz = DIM == 3 ? 2 : 1;
  float* fp = fbase<CL>(fpool, p);
  for (int v = 0; v < nrvars; v++) {
    const float* a = fp + p.ecq + v * p.sc;
    float* e = fp + p.eq + v * p.sq;
    // x-direction values b[dz][dy][fx] for coarse rows (cj+dy, ck+dz)
    float bxv[2][2][2];
    for (int dz = 0; dz < nz; dz++)
      for (int dy = 0; dy < 2; dy++) {
        float lo = a[gofs<DIM>(p.cn, ci, cj + dy, ck + dz)], hi = a[gofs<DIM>(p.cn, ci + 1, cj + dy, ck + dz)];
        bxv[dz][dy][0] = 3.0f * lo + hi;
        bxv[dz][dy][1] = lo + 3.0f * hi;
      }
    for (int fz = 0; fz < nz; fz++)
      for (int fy = 0; fy < 2; fy++)
        for (int fx = 0; fx < 2; fx++) {
          int i = 2 * ci + fx, j = 2 * cj + fy, k = DIM == 3 ? 2 * ck + fz : 0;
          float add;
          if (DIM == 2) {
            float blo = bxv[0][0][fx], bhi = bxv[0][1][fx];
            add = (fy == 0 ? 3.0f * blo + bhi : blo + 3.0f * bhi) * (1.0f / 16.0f);
          } else {
            float c0 = fy == 0 ? 3.0f * bxv[0][0][fx] + bxv[0][1][fx] : bxv[0][0][fx] + 3.0f * bxv[0][1][fx];
            float c1 = fy == 0 ? 3.0f * bxv[1][0][fx] + bxv[1][1][fx] : bxv[1][0][fx] + 3.0f * bxv[1][1][fx];
            add = (fz == 0 ? 3.0f * c0 + c1 : c0 + 3.0f * c1) * (1.0f / 64.0f);
          }
          e[gofs<DIM>(p.qn, i, j, k)] += add;
        }
  }
}

// ghost programs on e: homogeneous boundary conditions
template <bool CL = false>
__device__ __forceinline__ void ghost32_apply(const PatchDev* __restrict__ P, float* __restrict__ fpool,
                                              const GhostOp& g, int nrvars) {
  const PatchDev& d = P[g.dp];
  const PatchDev& s = P[g.sp];
  float* fd = fbase<CL>(fpool, d);
  const float* fs = fbase<CL>(fpool, s);
  for (int v = 0; v < nrvars; v++) {
    float* dq = fd + d.eq + v * d.sq;
    const float* sq = fs + s.eq + v * s.sq;
    float val;
    switch (g.type) {
      case kGCopy:
      case kGCopyAdd:
      case kGCopySub: val = sq[g.s0]; break;  // the qpo offset cancels in a correction
      case kGBC: val = ((g.mask >> v) & 0x101) ? -sq[g.s0] : sq[g.s0]; break;  // 2 - q, -q -> -e
      case kGCfA: val = fA1 * dq[g.s0] + fA2 * dq[g.s1] + fA3 * sq[g.c0]; break;
      case kGCfAB: val = fA1 * dq[g.s0] + fA2 * dq[g.s1] + fA3 * (fB1 * sq[g.c0] + fB2 * sq[g.c1] + fB3 * sq[g.c2]); break;
      default:
        val = fA1 * dq[g.s0] + fA2 * dq[g.s1] +
              fA3 * (fC1 * sq[g.c0] + fC2 * sq[g.c1] + fC3 * sq[g.c2] + fC4 * sq[g.c3]);
        break;
    }
    dq[g.dcell] = val;
  }
}


// ---------------------------------------------------------------------------
// The plugin-dependent operations of the correction cycle: templates over
// the plugin struct PL.

// step 1 of an outer iteration: the frozen base planes and g, the FP32
// image of the FP64 residual (mode 0: base planes only, 1: g from the
// stored rf, 2: g = f - N(qbar) recomputed)
template <class PL, int DIM, bool CL = false>
__device__ __forceinline__ void u_prep(const PatchDev* __restrict__ P, double* pool, float* fpool, const Blk b,
                                       int tid, int mode, const ProbParams& pp) {
  const PatchDev& p = P[b.patch];
  int i, j, k;
  if (!interior_cell<DIM>(p.mx, b.start + tid, i, j, k)) return;
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
  float* fp = fbase<CL>(fpool, p);
  PL::template mx_prep<DIM>(x, pool + p.orf, fp + p.ephi, fp + p.eg, mode, p.c, pp);
}
template <class PL, int DIM>
__global__ void __launch_bounds__(kBlock) k_mx_prep(const PatchDev* __restrict__ P, double* pool, float* fpool,
                                                    const Blk* __restrict__ blk, int mode, ProbParams pp) {
  u_prep<PL, DIM>(P, pool, fpool, blk[blockIdx.x], threadIdx.x, mode, pp);
}

// step 3 of an outer iteration: qbar += e over the whole ghosted array; the
// same pass refreshes the first nbase base planes for the next cycle and
// clears e, so the next cycle needs neither a prep pass over those planes
// nor a memset on this level
template <int DIM, bool CL = false>
__device__ __forceinline__ void u_update(const PatchDev* __restrict__ P, double* pool, float* fpool, const Blk b,
                                         int tid, int nrvars, int nbase) {
  const PatchDev& p = P[b.patch];
  int i, j, k;
  if (!ghosted_cell<DIM>(p.qn, p.gs, b.start + tid, i, j, k)) return;
  bool interior = i >= 1 && i <= p.mx[0] && j >= 1 && j <= p.mx[1] && (DIM == 2 || (k >= 1 && k <= p.mx[2]));
  long long c = gofs<DIM>(p.qn, i, j, k);
  float* fp = fbase<CL>(fpool, p);
  for (int v = 0; v < nrvars; v++) {
    double nq = pool[p.oq + v * p.sq + c] + (double)fp[p.eq + v * p.sq + c];
    pool[p.oq + v * p.sq + c] = nq;
    fp[p.eq + v * p.sq + c] = 0.0f;
    if (v < nbase && interior) fp[p.ephi + v * p.sf + iofs<DIM>(p.mx, i, j, k)] = (float)nq;
  }
}

template <class PL, int DIM, bool CL = false>
__device__ __forceinline__ Cell32 cell32(const PatchDev& p, float* fpool, int i, int j, int k) {
  Cell32 x;
  float* fp = fbase<CL>(fpool, p);
  x.e = fp + p.eq;
  x.g = fp + p.eg;
  x.base = fp + p.ephi;
  x.c = gofs<DIM>(p.qn, i, j, k);
  x.fc = iofs<DIM>(p.mx, i, j, k);
  x.sy = p.qn[0];
  x.sz = (long long)p.qn[0] * p.qn[1];
  x.sq = p.sq;
  x.sf = p.sf;
  return x;
}

// red-black pointwise relaxation of the correction, in arithmetic T (FP64
// with the patch's FP64 coefficients on the coarsest level)
template <class PL, int DIM, bool CL = false, typename T = float>
__device__ __forceinline__ void u_relax(const PatchDev* __restrict__ P, float* __restrict__ fpool, const Blk b,
                                        int tid, int ipass, const MxParams& mp) {
  const PatchDev& p = P[b.patch];
  int i, j, k;
  if (!color_cell<DIM>(p, b.start + tid, ipass, i, j, k)) return;
  if constexpr (sizeof(T) == sizeof(double))
    PL::template mx_relax<DIM, double>(cell32<PL, DIM, CL>(p, fpool, i, j, k), p.c, mp);
  else
    PL::template mx_relax<DIM, float>(cell32<PL, DIM, CL>(p, fpool, i, j, k), p.cf, mp);
}
// ipass with kRelax64: the FP64 smoother
template <class PL, int DIM, bool CL = false>
__device__ __forceinline__ void u_relax_any(const PatchDev* __restrict__ P, float* __restrict__ fpool, const Blk b,
                                            int tid, int ipass, const MxParams& mp) {
  if (ipass & kRelax64) u_relax<PL, DIM, CL, double>(P, fpool, b, tid, ipass & 3, mp);
  else u_relax<PL, DIM, CL>(P, fpool, b, tid, ipass, mp);
}
template <class PL, int DIM, typename T>
__global__ void __launch_bounds__(kBlock) k_mx_relax(const PatchDev* __restrict__ P, float* __restrict__ fpool,
                                                     const Blk* __restrict__ blk, int ipass, MxParams mp) {
  u_relax<PL, DIM, false, T>(P, fpool, blk[blockIdx.x], threadIdx.x, ipass, mp);
}

// CoarseLoadingFunction on the correction: fine r = g - M(e) under each
// coarse cell; parent g(mb) = R(r) + M_c(ec) with the parent's base planes.
template <class PL, int DIM, bool CL = false>
__device__ __forceinline__ void u_coarse_load(const PatchDev* __restrict__ P, float* __restrict__ fpool, const Blk b,
                                              int tid, const MxParams& mp) {
  constexpr int NV = PL::kNV;
  const PatchDev& p = P[b.patch];
  int ci, cj, ck;
  if (!interior_cell<DIM>(p.cmx, b.start + tid, ci, cj, ck)) return;
  const PatchDev& par = P[p.parent];
  float* fp = fbase<CL>(fpool, p);
  float* fq = fbase<CL>(fpool, par);
  const float* e = fp + p.eq;
  long long sy = p.qn[0], sz = (long long)p.qn[0] * p.qn[1];
  float R[NV];
  for (int v = 0; v < NV; v++) R[v] = 0.f;
  const int nk = DIM == 3 ? 2 : 1;
  for (int dk = 0; dk < nk; dk++)
    for (int dj = 0; dj < 2; dj++)
      for (int di = 0; di < 2; di++) {
        int i = 2 * ci - di, j = 2 * cj - dj, k = DIM == 3 ? 2 * ck - dk : 1;
        long long c = gofs<DIM>(p.qn, i, j, k);
        long long fc = iofs<DIM>(p.mx, i, j, k);
        float m[NV];
        PL::template mx_op<DIM>(e, c, sy, sz, p.sq, fp + p.ephi, fc, p.sf, p.cf, mp, m);
        for (int v = 0; v < NV; v++) R[v] += fp[p.eg + v * p.sf + fc] - m[v];
      }
  for (int v = 0; v < NV; v++) R[v] *= DIM == 2 ? 0.25f : 0.125f;
  const float* ec = fp + p.ecq;
  long long csy = p.cn[0], csz = (long long)p.cn[0] * p.cn[1];
  long long cc = gofs<DIM>(p.cn, ci, cj, ck);
  long long pf = iofs<DIM>(par.mx, p.mb[0] + ci - 1, p.mb[1] + cj - 1, DIM == 3 ? p.mb[2] + ck - 1 : 1);
  // the coarse operator reads the ec ring, which coarse_ring has filled
  float m[NV];
  PL::template mx_op<DIM>(ec, cc, csy, csz, p.sc, fq + par.ephi, pf, par.sf, par.cf, mp, m);
  for (int v = 0; v < NV; v++) fq[par.eg + v * par.sf + pf] = R[v] + m[v];
}
template <class PL, int DIM>
__global__ void __launch_bounds__(kBlock) k_mx_coarse_load(const PatchDev* __restrict__ P, float* __restrict__ fpool,
                                                           const Blk* __restrict__ blk, MxParams mp) {
  u_coarse_load<PL, DIM>(P, fpool, blk[blockIdx.x], threadIdx.x, mp);
}

// FP64 residual rf = f - N(q) of the finest level and per-block sums of rf^2
// (ErrorAFAS, afasroutines.f90:113-233).  The plugin's FP64 operator, but
// in a translation unit that lets the compiler fuse multiply-adds, which
// cuts FP64 pipe work by about a third; the mixed path needs the true
// residual to ~1e-15 relative, not bit-identical rounding.  kNormCells
// consecutive blocks of the (padded) interior list per CTA, so the shuffle
// reduction (FP64 adds on every lane) is paid once per kNormCells cells.
template <class PL, int DIM>
__global__ void __launch_bounds__(kBlock) k_mx_norm(const PatchDev* __restrict__ P, double* __restrict__ pool,
                                                    const Blk* __restrict__ blk, ProbParams pp,
                                                    double* __restrict__ partial) {
  constexpr int NV = PL::kNV;
  __shared__ double red[NV][kBlock / 32];
  double s[NV];
  for (int v = 0; v < NV; v++) s[v] = 0.0;
  for (int sub = 0; sub < kNormCells; sub++) {
    const Blk b = blk[blockIdx.x * kNormCells + sub];
    if (b.patch < 0) break;
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
      pool[p.orf + v * p.sf + fc] = e;
      s[v] = fma(e, e, s[v]);
    }
  }
  for (int o = 16; o > 0; o >>= 1)
    for (int v = 0; v < NV; v++) s[v] += __shfl_down_sync(0xffffffffu, s[v], o);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0)
    for (int v = 0; v < NV; v++) red[v][w] = s[v];
  __syncthreads();
  if (threadIdx.x == 0)
    for (int v = 0; v < NV; v++) {
      double t = 0.0;
      for (int m = 0; m < kBlock / 32; m++) t += red[v][m];
      partial[NV * blockIdx.x + v] = t;
    }
}

// Residual tracked in FP32 between FP64 evaluations: after qbar += e the
// new residual is exactly g - M(e) (M is the difference N(qbar+e) - N(qbar)),
// so g <- g - M(e) on the finest level gives the next right-hand side and,
// summed, the tracked norm.  Sums of squares in FP32 (the tracked norm only
// decides when to re-evaluate in FP64); one conversion per block.
template <class PL, int DIM>
__global__ void __launch_bounds__(kBlock) k_mx_track(const PatchDev* __restrict__ P, float* __restrict__ fpool,
                                                     const Blk* __restrict__ blk, double* __restrict__ partial,
                                                     MxParams mp) {
  constexpr int NV = PL::kNV;
  __shared__ float red[NV][kBlock / 32];
  const Blk b = blk[blockIdx.x];
  const PatchDev& p = P[b.patch];
  int i, j, k;
  float s[NV];
  for (int v = 0; v < NV; v++) s[v] = 0.f;
  if (interior_cell<DIM>(p.mx, b.start + threadIdx.x, i, j, k)) {
    long long sy = p.qn[0], sz = (long long)p.qn[0] * p.qn[1];
    long long c = gofs<DIM>(p.qn, i, j, k);
    long long fc = iofs<DIM>(p.mx, i, j, k);
    float m[NV];
    PL::template mx_op<DIM>(fpool + p.eq, c, sy, sz, p.sq, fpool + p.ephi, fc, p.sf, p.cf, mp, m);
    for (int v = 0; v < NV; v++) {
      float gv = fpool[p.eg + v * p.sf + fc] - m[v];
      fpool[p.eg + v * p.sf + fc] = gv;
      s[v] = gv * gv;
    }
  }
  for (int o = 16; o > 0; o >>= 1)
    for (int v = 0; v < NV; v++) s[v] += __shfl_down_sync(0xffffffffu, s[v], o);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0)
    for (int v = 0; v < NV; v++) red[v][w] = s[v];
  __syncthreads();
  if (threadIdx.x == 0)
    for (int v = 0; v < NV; v++) {
      float t = 0.f;
      for (int m = 0; m < kBlock / 32; m++) t += red[v][m];
      partial[NV * blockIdx.x + v] = (double)t;
    }
}

// The coarse tail of a V-cycle in one CTA.  Below some level every level of
// a hierarchy is small (a few thousand cells), and the launches of its
// V-cycle (~20 per level) cost more than their work.  The tail program is
// the sequence of operations the V-cycle would launch from that level down,
// recorded once on the host; this kernel executes it phase by phase, every
// work-list block of a phase by the whole CTA (256 threads = one block's
// units), with a barrier between phases.  Each unit computes exactly what
// the stand-alone kernel computes, so results are bit-identical.
template <class PL, int DIM>
__device__ __forceinline__ void run_tail(const PatchDev* __restrict__ P, float* fpool, const TailPhase* __restrict__ ph,
                                         int nph, int nrvars, const MxParams& mp) {
  for (int x = 0; x < nph; x++) {
    const TailPhase f = ph[x];
    if (f.op == kTGhost) {
      for (int s = 0; s < f.nstages; s++) {
        for (int t = f.stage_off[s] + threadIdx.x; t < f.stage_off[s + 1]; t += blockDim.x) {
          GhostOp g = f.ops[t];
          ghost32_apply(P, fpool, g, nrvars);
        }
        __syncthreads();
      }
      continue;
    }
    for (int b = 0; b < f.nblk; b++) {
      const Blk bb = f.blk[b];
      switch (f.op) {
        case kTRelax: u_relax_any<PL, DIM>(P, fpool, bb, threadIdx.x, f.arg, mp); break;
        case kTRestrict: u_restrict<DIM>(P, fpool, bb, threadIdx.x, nrvars); break;
        case kTRing: u_coarse_ring<DIM>(P, fpool, bb, threadIdx.x, nrvars, f.arg); break;
        case kTLoad: u_coarse_load<PL, DIM>(P, fpool, bb, threadIdx.x, mp); break;
        default: u_prolong<DIM>(P, fpool, bb, threadIdx.x, nrvars); break;
      }
    }
    __syncthreads();
  }
}

template <class PL, int DIM>
__global__ void __launch_bounds__(kBlock) k_mx_tail(const PatchDev* __restrict__ P, float* __restrict__ fpool,
                                                   const TailPhase* __restrict__ ph, int nph, int nrvars, MxParams mp) {
  run_tail<PL, DIM>(P, fpool, ph, nph, nrvars, mp);
}

// The same with the tail levels' arrays staged in shared memory: P is a
// patch table whose tail patches address the block's shared memory, so the
// phases run on on-chip copies; the modified arrays are written back at the
// end.  Same arithmetic on the same values: results are bit-identical.
template <class PL, int DIM>
__global__ void __launch_bounds__(kBlock) k_mx_tail_smem(const PatchDev* __restrict__ P, float* __restrict__ fpool,
                                                        const TailPhase* __restrict__ ph, int nph, int nrvars,
                                                        MxParams mp, const StageSeg* __restrict__ segs, int nsegs) {
  extern __shared__ float sm[];
  for (int x = 0; x < nsegs; x++) {
    const StageSeg sg = segs[x];
    for (int t = threadIdx.x; t < sg.n; t += blockDim.x) sm[sg.s + t] = fpool[sg.g + t];
  }
  __syncthreads();
  run_tail<PL, DIM>(P, sm, ph, nph, nrvars, mp);
  for (int x = 0; x < nsegs; x++) {
    const StageSeg sg = segs[x];
    if (!sg.out) continue;
    for (int t = threadIdx.x; t < sg.n; t += blockDim.x) fpool[sg.g + t] = sm[sg.s + t];
  }
}

}  // namespace mx
}  // namespace bsamg

#include "kern_solve.cuh"

namespace bsamg {
namespace mx {

// The launchers of one plugin's correction-form kernels (the table the
// plugin registers)
template <class PL>
struct Launchers {
  static int prep(const MxLaunch& L, const Blk* blk, int nblk, int mode) {
    if (nblk <= 0) return 0;
    if (L.ndims == 2) k_mx_prep<PL, 2><<<nblk, kBlock, 0, L.s>>>(L.P, L.pool, L.fpool, blk, mode, L.pp);
    else k_mx_prep<PL, 3><<<nblk, kBlock, 0, L.s>>>(L.P, L.pool, L.fpool, blk, mode, L.pp);
    return 1;
  }
  static int relax(const MxLaunch& L, const Blk* blk, int nblk, int ipass) {
    if (nblk <= 0) return 0;
    MxParams mp = PL::mx_params(L.pp);
    const int ip = ipass & 3;
    if (ipass & kRelax64) {
      if (L.ndims == 2) k_mx_relax<PL, 2, double><<<nblk, kBlock, 0, L.s>>>(L.P, L.fpool, blk, ip, mp);
      else k_mx_relax<PL, 3, double><<<nblk, kBlock, 0, L.s>>>(L.P, L.fpool, blk, ip, mp);
    } else {
      if (L.ndims == 2) k_mx_relax<PL, 2, float><<<nblk, kBlock, 0, L.s>>>(L.P, L.fpool, blk, ip, mp);
      else k_mx_relax<PL, 3, float><<<nblk, kBlock, 0, L.s>>>(L.P, L.fpool, blk, ip, mp);
    }
    return 1;
  }
  static int coarse_load(const MxLaunch& L, const Blk* blk, int nblk) {
    if (nblk <= 0) return 0;
    MxParams mp = PL::mx_params(L.pp);
    if (L.ndims == 2) k_mx_coarse_load<PL, 2><<<nblk, kBlock, 0, L.s>>>(L.P, L.fpool, blk, mp);
    else k_mx_coarse_load<PL, 3><<<nblk, kBlock, 0, L.s>>>(L.P, L.fpool, blk, mp);
    return 1;
  }
  static int track(const MxLaunch& L, const Blk* blk, int nblk, double* partial) {
    if (nblk <= 0) return 0;
    MxParams mp = PL::mx_params(L.pp);
    if (L.ndims == 2) k_mx_track<PL, 2><<<nblk, kBlock, 0, L.s>>>(L.P, L.fpool, blk, partial, mp);
    else k_mx_track<PL, 3><<<nblk, kBlock, 0, L.s>>>(L.P, L.fpool, blk, partial, mp);
    return 1;
  }
  static int norm(const MxLaunch& L, const Blk* padded, int nb, double* partial) {
    if (nb <= 0) return 0;
    if (L.ndims == 2) k_mx_norm<PL, 2><<<nb, kBlock, 0, L.s>>>(L.P, L.pool, padded, L.pp, partial);
    else k_mx_norm<PL, 3><<<nb, kBlock, 0, L.s>>>(L.P, L.pool, padded, L.pp, partial);
    return 1;
  }
  static int tail(const MxLaunch& L, const PatchDev* table, const TailPhase* ph, int nph, const StageSeg* segs,
                  int nsegs, int smem_bytes) {
    if (nph <= 0) return 0;
    MxParams mp = PL::mx_params(L.pp);
    int nr = L.pp.nrvars;
    if (smem_bytes) {
      if (L.ndims == 2)
        k_mx_tail_smem<PL, 2><<<1, kBlock, smem_bytes, L.s>>>(table, L.fpool, ph, nph, nr, mp, segs, nsegs);
      else
        k_mx_tail_smem<PL, 3><<<1, kBlock, smem_bytes, L.s>>>(table, L.fpool, ph, nph, nr, mp, segs, nsegs);
    } else {
      if (L.ndims == 2) k_mx_tail<PL, 2><<<1, kBlock, 0, L.s>>>(table, L.fpool, ph, nph, nr, mp);
      else k_mx_tail<PL, 3><<<1, kBlock, 0, L.s>>>(table, L.fpool, ph, nph, nr, mp);
    }
    return 1;
  }
  // the whole solve in one cluster launch (kern_solve.cuh); 1 on success,
  // -1 when the launch shape is not one of the compiled ones or the launch
  // failed (cudaGetLastError then says why)
  template <int DIM, int T>
  static cudaError_t solve_launch(const MxLaunch& L, const void* img, SolveImage im, SolveCtl* ctl, double* res,
                                  double* partial, int ctas) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(ctas);
    cfg.blockDim = dim3(T);
    cfg.dynamicSmemBytes = im.data + im.ops + im.bytes;  // FP32 data, ghost operations, image
    cfg.stream = L.s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = ctas;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_mx_solve<PL, DIM, T>, static_cast<const unsigned char*>(img), im, L.pool,
                              L.fpool, ctl, res, partial, L.pp, PL::mx_params(L.pp));
  }
  static int solve(const MxLaunch& L, const void* ph, SolveImage im, SolveCtl* ctl, double* res, double* partial,
                   SolveShape sh) {
    cudaError_t e = cudaErrorInvalidValue;
    if (L.ndims == 2) {
      if (sh.threads == 256) e = solve_launch<2, 256>(L, ph, im, ctl, res, partial, sh.ctas);
      else if (sh.threads == 512) e = solve_launch<2, 512>(L, ph, im, ctl, res, partial, sh.ctas);
      else if (sh.threads == 1024) e = solve_launch<2, 1024>(L, ph, im, ctl, res, partial, sh.ctas);
    } else {
      if (sh.threads == 256) e = solve_launch<3, 256>(L, ph, im, ctl, res, partial, sh.ctas);
      else if (sh.threads == 512) e = solve_launch<3, 512>(L, ph, im, ctl, res, partial, sh.ctas);
      else if (sh.threads == 1024) e = solve_launch<3, 1024>(L, ph, im, ctl, res, partial, sh.ctas);
    }
    return e == cudaSuccess ? 1 : -1;
  }
  // allow clusters above the portable 8 CTAs and report how many clusters of
  // this shape fit on the device at once (0: the shape cannot run)
  template <int DIM, int T>
  static int solve_fit(int ctas) {
    auto k = k_mx_solve<PL, DIM, T>;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) return 0;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, kSolveSmemMax) != cudaSuccess) return 0;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(ctas);
    cfg.blockDim = dim3(T);
    cfg.dynamicSmemBytes = kSolveSmemMax;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = ctas;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, k, &cfg) != cudaSuccess) return 0;
    return n;
  }
  static int solve_setup(int ndims, SolveShape sh) {
    int n = 0;
    if (ndims == 2) {
      if (sh.threads == 256) n = solve_fit<2, 256>(sh.ctas);
      else if (sh.threads == 512) n = solve_fit<2, 512>(sh.ctas);
      else if (sh.threads == 1024) n = solve_fit<2, 1024>(sh.ctas);
    } else {
      if (sh.threads == 256) n = solve_fit<3, 256>(sh.ctas);
      else if (sh.threads == 512) n = solve_fit<3, 512>(sh.ctas);
      else if (sh.threads == 1024) n = solve_fit<3, 1024>(sh.ctas);
    }
    cudaGetLastError();  // a shape that does not fit is an answer, not an error
    return n;
  }
  static int tail_smem_attributes(int ndims) {
    const cudaFuncAttribute a = cudaFuncAttributeMaxDynamicSharedMemorySize;
    cudaError_t e = ndims == 2 ? cudaFuncSetAttribute(k_mx_tail_smem<PL, 2>, a, kTailSmemMax)
                               : cudaFuncSetAttribute(k_mx_tail_smem<PL, 3>, a, kTailSmemMax);
    return e == cudaSuccess ? 0 : -1;
  }
};

template <class PL>
const PluginMixed* mixed_ops() {
  static const PluginMixed ops = {PL::kMxBase,           PL::kMxUpdate,          &Launchers<PL>::prep,
                                  &Launchers<PL>::relax, &Launchers<PL>::coarse_load, &Launchers<PL>::track,
                                  &Launchers<PL>::norm,  &Launchers<PL>::tail,   &Launchers<PL>::tail_smem_attributes,
                                  &Launchers<PL>::solve, &Launchers<PL>::solve_setup};
  return &ops;
}

}  // namespace mx
}  // namespace bsamg
