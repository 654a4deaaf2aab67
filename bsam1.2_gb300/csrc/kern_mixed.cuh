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
template <int DIM>
__device__ __forceinline__ void u_restrict(const PatchDev* __restrict__ P, float* __restrict__ fpool, const Blk b,
                                           int tid, int nrvars) {
  const PatchDev& p = P[b.patch];
  int ci, cj, ck;
  if (!interior_cell<DIM>(p.cmx, b.start + tid, ci, cj, ck)) return;
  const PatchDev& par = P[p.parent];
  for (int v = 0; v < nrvars; v++) {
    const float* e = fpool + p.eq + v * p.sq;
    auto at = [&](int i, int j, int k) { return e[gofs<DIM>(p.qn, i, j, k)]; };
    float val = restrict_at32<DIM>(at, ci, cj, ck);
    fpool[p.ecq + v * p.sc + gofs<DIM>(p.cn, ci, cj, ck)] = val;
    fpool[par.eq + v * par.sq +
          gofs<DIM>(par.qn, p.mb[0] + ci - 1, p.mb[1] + cj - 1, DIM == 3 ? p.mb[2] + ck - 1 : 0)] = val;
  }
}


// GetCoarseGhostPoints on e (ring of ec <- parent e) when corr == 0;
// CorrectFine step 1 (ec = parent e - ec over the whole ghosted ec) when
// corr == 1.
template <int DIM>
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
  for (int v = 0; v < nrvars; v++) {
    float* ec = fpool + p.ecq + v * p.sc;
    float pv = fpool[par.eq + v * par.sq + src];
    ec[dst] = corr ? pv - ec[dst] : pv;
  }
}


// CorrectFine step 2 on e: e(0:mx+1) += P(ec).
// One thread per coarse index (ci,cj,ck) in 0..cmx: it produces the fine
// cells 2ci..2ci+1 (x) etc. from the 2x2(x2) coarse values they share, with
// the same per-direction (3,1)/4 weights as BiLin/TriLinProlongationP1
// (gridutilities.f90:156-195, :510-566).
template <int DIM>
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
  for (int v = 0; v < nrvars; v++) {
    const float* a = fpool + p.ecq + v * p.sc;
    float* e = fpool + p.eq + v * p.sq;
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
__device__ __forceinline__ void ghost32_apply(const PatchDev* __restrict__ P, float* __restrict__ fpool,
                                              const GhostOp& g, int nrvars) {
  const PatchDev& d = P[g.dp];
  const PatchDev& s = P[g.sp];
  for (int v = 0; v < nrvars; v++) {
    float* dq = fpool + d.eq + v * d.sq;
    const float* sq = fpool + s.eq + v * s.sq;
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
template <class PL, int DIM>
__global__ void __launch_bounds__(kBlock) k_mx_prep(const PatchDev* __restrict__ P, const double* __restrict__ pool,
                                                    float* __restrict__ fpool, const Blk* __restrict__ blk, int mode,
                                                    ProbParams pp) {
  const Blk b = blk[blockIdx.x];
  const PatchDev& p = P[b.patch];
  int i, j, k;
  if (!interior_cell<DIM>(p.mx, b.start + threadIdx.x, i, j, k)) return;
  Cell64 x;
  x.q = const_cast<double*>(pool) + p.oq;
  x.f = pool + p.of;
  x.qold = pool + p.oqold;
  x.c = gofs<DIM>(p.qn, i, j, k);
  x.fc = iofs<DIM>(p.mx, i, j, k);
  x.sy = p.qn[0];
  x.sz = (long long)p.qn[0] * p.qn[1];
  x.sq = p.sq;
  x.sf = p.sf;
  PL::template mx_prep<DIM>(x, pool + p.orf, fpool + p.ephi, fpool + p.eg, mode, p.c, pp);
}

template <class PL, int DIM>
__device__ __forceinline__ Cell32 cell32(const PatchDev& p, float* fpool, int i, int j, int k) {
  Cell32 x;
  x.e = fpool + p.eq;
  x.g = fpool + p.eg;
  x.base = fpool + p.ephi;
  x.c = gofs<DIM>(p.qn, i, j, k);
  x.fc = iofs<DIM>(p.mx, i, j, k);
  x.sy = p.qn[0];
  x.sz = (long long)p.qn[0] * p.qn[1];
  x.sq = p.sq;
  x.sf = p.sf;
  return x;
}

// red-black pointwise relaxation of the correction
template <class PL, int DIM>
__device__ __forceinline__ void u_relax(const PatchDev* __restrict__ P, float* __restrict__ fpool, const Blk b,
                                        int tid, int ipass, const MxParams& mp) {
  const PatchDev& p = P[b.patch];
  int i, j, k;
  if (!color_cell<DIM>(p, b.start + tid, ipass, i, j, k)) return;
  PL::template mx_relax<DIM>(cell32<PL, DIM>(p, fpool, i, j, k), p.cf, mp);
}
template <class PL, int DIM>
__global__ void __launch_bounds__(kBlock) k_mx_relax(const PatchDev* __restrict__ P, float* __restrict__ fpool,
                                                     const Blk* __restrict__ blk, int ipass, MxParams mp) {
  u_relax<PL, DIM>(P, fpool, blk[blockIdx.x], threadIdx.x, ipass, mp);
}

// CoarseLoadingFunction on the correction: fine r = g - M(e) under each
// coarse cell; parent g(mb) = R(r) + M_c(ec) with the parent's base planes.
template <class PL, int DIM>
__device__ __forceinline__ void u_coarse_load(const PatchDev* __restrict__ P, float* __restrict__ fpool, const Blk b,
                                              int tid, const MxParams& mp) {
  constexpr int NV = PL::kNV;
  const PatchDev& p = P[b.patch];
  int ci, cj, ck;
  if (!interior_cell<DIM>(p.cmx, b.start + tid, ci, cj, ck)) return;
  const PatchDev& par = P[p.parent];
  const float* e = fpool + p.eq;
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
        PL::template mx_op<DIM>(e, c, sy, sz, p.sq, fpool + p.ephi, fc, p.sf, p.cf, mp, m);
        for (int v = 0; v < NV; v++) R[v] += fpool[p.eg + v * p.sf + fc] - m[v];
      }
  for (int v = 0; v < NV; v++) R[v] *= DIM == 2 ? 0.25f : 0.125f;
  const float* ec = fpool + p.ecq;
  long long csy = p.cn[0], csz = (long long)p.cn[0] * p.cn[1];
  long long cc = gofs<DIM>(p.cn, ci, cj, ck);
  long long pf = iofs<DIM>(par.mx, p.mb[0] + ci - 1, p.mb[1] + cj - 1, DIM == 3 ? p.mb[2] + ck - 1 : 1);
  // the coarse operator reads the ec ring, which coarse_ring has filled
  float m[NV];
  PL::template mx_op<DIM>(ec, cc, csy, csz, p.sc, fpool + par.ephi, pf, par.sf, par.cf, mp, m);
  for (int v = 0; v < NV; v++) fpool[par.eg + v * par.sf + pf] = R[v] + m[v];
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
        case kTRelax: u_relax<PL, DIM>(P, fpool, bb, threadIdx.x, f.arg, mp); break;
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
    if (L.ndims == 2) k_mx_relax<PL, 2><<<nblk, kBlock, 0, L.s>>>(L.P, L.fpool, blk, ipass, mp);
    else k_mx_relax<PL, 3><<<nblk, kBlock, 0, L.s>>>(L.P, L.fpool, blk, ipass, mp);
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
                                  &Launchers<PL>::norm,  &Launchers<PL>::tail,   &Launchers<PL>::tail_smem_attributes};
  return &ops;
}

}  // namespace mx
}  // namespace bsamg
