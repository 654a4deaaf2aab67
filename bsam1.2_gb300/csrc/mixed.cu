// Mixed-precision path: FP32 smoothing, restriction, tau and prolongation
// of a correction inside an FP64 defect-correction loop.
//
// One outer iteration (one "V-cycle" of the iteration count):
//   1. FP64: g = f - N(qbar) on every level >= 0 (on the finest level this is
//      the residual the previous convergence norm already computed), stored
//      as FP32; the base phase field phib = (float)qbar_phi on every level;
//      the correction e = 0 everywhere.
//   2. FP32: one AFAS V-cycle (afasroutines.f90:495-529) on the correction
//      equation M(e) := N(qbar + e) - N(qbar) = g, with the reference's
//      red-black pointwise 2x2 Newton smoother rewritten for e, the same
//      restriction, FAS tau (coarse load) and bilinear/trilinear
//      prolongation, and the same ghost programs applied to e (with the
//      homogeneous form of each boundary condition).
//   3. FP64: qbar += e on every level >= 0, FillDown(q), and the FP64
//      residual norm of the finest level, which decides convergence.
// The FP64 norm is the true residual of the reference's discrete problem,
// so the loop converges to the FP64 solution; FP32 only limits how much one
// outer iteration can gain (about 7 digits), not the final accuracy.
//
// The smoother here is HBM-bound on GB300 (FP32 runs at ~70 TFLOP/s), unlike
// the plain FP64 smoother, which the FP64 pipe bounds.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "launch.h"
#include "box.h"
#include "mixed.h"

namespace bsamg {

namespace {

constexpr float fA1 = -01.0f / 05.0f, fA2 = 02.0f / 03.0f, fA3 = 08.0f / 15.0f;
constexpr float fB1 = 05.0f / 32.0f, fB2 = 15.0f / 16.0f, fB3 = -03.0f / 32.0f;
constexpr float fC1 = 09.0f / 16.0f, fC2 = 03.0f / 16.0f, fC3 = 03.0f / 16.0f, fC4 = 01.0f / 16.0f;

template <int DIM>
__device__ __forceinline__ long long gofs(const int* n, int i, int j, int k) {
  if (DIM == 2) return (long long)j * n[0] + i;
  return ((long long)k * n[1] + j) * n[0] + i;
}
template <int DIM>
__device__ __forceinline__ long long iofs(const int* mx, int i, int j, int k) {
  if (DIM == 2) return (long long)(j - 1) * mx[0] + (i - 1);
  return ((long long)(k - 1) * mx[1] + (j - 1)) * mx[0] + (i - 1);
}
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

template <int DIM, typename T>
__device__ __forceinline__ T ulap(const T* a, long long c, long long sy, long long sz) {
  if (DIM == 2) return a[c + 1] + a[c - 1] + a[c + sy] + a[c - sy] - T(4) * a[c];
  return a[c + 1] + a[c - 1] + a[c + sy] + a[c - sy] + a[c + sz] + a[c - sz] - T(6) * a[c];
}

// ---------------------------------------------------------------------------
// Neighbour offsets of a cell in a ghosted array.

template <int DIM>
struct Nbr {
  long long xm, xp, ym, yp, zm, zp;
  __device__ __forceinline__ Nbr(long long c, long long sy, long long sz) {
    xm = c - 1; xp = c + 1; ym = c - sy; yp = c + sy; zm = c - sz; zp = c + sz;
  }
};

template <int DIM, typename T>
__device__ __forceinline__ T ulapn(const T* a, long long c, const Nbr<DIM>& n) {
  if (DIM == 2) return a[n.xp] + a[n.xm] + a[n.yp] + a[n.ym] - T(4) * a[c];
  return a[n.xp] + a[n.xm] + a[n.yp] + a[n.ym] + a[n.zp] + a[n.zm] - T(6) * a[c];
}

// correction operator at a fine cell with neighbour set n
template <int DIM>
__device__ __forceinline__ void mopn(const float* e, long long c, const Nbr<DIM>& n, long long ps, float pb,
                                     float c0, float c1, float& m0, float& m1) {
  const float* e0 = e;
  const float* e1 = e + ps;
  float x = e0[c];
  m0 = x - c0 * ulapn<DIM>(e1, c, n);
  m1 = e1[c] - x * (3.0f * pb * (pb + x) + x * x) + c1 * ulapn<DIM>(e0, c, n);
}

constexpr int kNormCells = 8;  // interior blocks per CTA in k_mx_norm

// step 1: phib = (float)qbar_phi everywhere; g = FP32 of the FP64 residual:
// mode 0: phib only, 1: g from the stored rf, 2: g = f - N(qbar) recomputed
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_mx_prep(const PatchDev* __restrict__ P, const double* __restrict__ pool,
                                                    float* __restrict__ fpool, const Blk* __restrict__ blk, int mode) {
  const Blk b = blk[blockIdx.x];
  const PatchDev& p = P[b.patch];
  int i, j, k;
  if (!interior_cell<DIM>(p.mx, b.start + threadIdx.x, i, j, k)) return;
  long long c = gofs<DIM>(p.qn, i, j, k);
  long long fc = iofs<DIM>(p.mx, i, j, k);
  const double* q0 = pool + p.oq;
  const double* q1 = q0 + p.sq;
  fpool[p.ephi + fc] = (float)q0[c];
  if (mode == 0) return;
  double r0, r1;
  if (mode == 1) {
    r0 = pool[p.orf + fc];
    r1 = pool[p.orf + p.sf + fc];
  } else {
    long long sy = p.qn[0], sz = (long long)p.qn[0] * p.qn[1];
    double o0 = q0[c] - p.c[0] * ulap<DIM>(q1, c, sy, sz);
    double o1 = q1[c] - q0[c] * q0[c] * q0[c] + p.c[1] * ulap<DIM>(q0, c, sy, sz);
    r0 = pool[p.of + fc] - o0;
    r1 = pool[p.of + p.sf + fc] - o1;
  }
  fpool[p.eg + fc] = (float)r0;
  fpool[p.eg + p.sf + fc] = (float)r1;
}

// red-black pointwise Newton on the correction (RelaxGrid2D/3D,
// CH/problem.f90:318-369, :554-614, in correction form):
//   a21 = -3 (pb + e)^2 - tmp3
//   b1  = g1 + tmp1 * sum(e_mu neighbours)
//   b2  = g2 - tmp2 * sum(e_phi neighbours) - e^2 (3 pb + 2 e)
template <int DIM>
__device__ __forceinline__ void u_relax(const PatchDev* __restrict__ P, float* __restrict__ fpool, const Blk b,
                                        int tid, int ipass) {
  const PatchDev& p = P[b.patch];
  int i, j, k;
  if (!color_cell<DIM>(p, b.start + tid, ipass, i, j, k)) return;
  float* e0 = fpool + p.eq;
  float* e1 = e0 + p.sq;
  long long sy = p.qn[0], sz = (long long)p.qn[0] * p.qn[1];
  long long c = gofs<DIM>(p.qn, i, j, k);
  long long fc = iofs<DIM>(p.mx, i, j, k);
  Nbr<DIM> n(c, sy, sz);
  float tmp1 = p.cf[0], tmp2 = p.cf[1], tmp3 = p.cf[2], a12 = p.cf[3];
  float pb = fpool[p.ephi + fc];
  float x = e0[c];
  float w = pb + x;
  float a21 = -3.0f * w * w - tmp3;
  float s1, s0;
  if (DIM == 2) {
    s1 = e1[n.xm] + e1[n.xp] + e1[n.ym] + e1[n.yp];
    s0 = e0[n.xp] + e0[n.xm] + e0[n.yp] + e0[n.ym];
  } else {
    s1 = e1[n.xm] + e1[n.xp] + e1[n.ym] + e1[n.yp] + e1[n.zm] + e1[n.zp];
    s0 = e0[n.xp] + e0[n.xm] + e0[n.yp] + e0[n.ym] + e0[n.zp] + e0[n.zm];
  }
  float b1 = fpool[p.eg + fc] + tmp1 * s1;
  float b2 = fpool[p.eg + p.sf + fc] - tmp2 * s0 - x * x * (3.0f * pb + 2.0f * x);
  float rdet = 1.0f / (1.0f - a12 * a21);
  e0[c] = (b1 - a12 * b2) * rdet;
  e1[c] = (b2 - a21 * b1) * rdet;
}
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_mx_relax(const PatchDev* __restrict__ P, float* __restrict__ fpool,
                                                     const Blk* __restrict__ blk, int ipass) {
  u_relax<DIM>(P, fpool, blk[blockIdx.x], threadIdx.x, ipass);
}

template <int DIM, typename F>
__device__ __forceinline__ float restrict_at(F at, int ci, int cj, int ck) {
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
    float val = restrict_at<DIM>(at, ci, cj, ck);
    fpool[p.ecq + v * p.sc + gofs<DIM>(p.cn, ci, cj, ck)] = val;
    fpool[par.eq + v * par.sq +
          gofs<DIM>(par.qn, p.mb[0] + ci - 1, p.mb[1] + cj - 1, DIM == 3 ? p.mb[2] + ck - 1 : 0)] = val;
  }
}
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_mx_restrict(const PatchDev* __restrict__ P, float* __restrict__ fpool,
                                                        const Blk* __restrict__ blk, int nrvars) {
  u_restrict<DIM>(P, fpool, blk[blockIdx.x], threadIdx.x, nrvars);
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
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_mx_coarse_ring(const PatchDev* __restrict__ P, float* __restrict__ fpool,
                                                           const Blk* __restrict__ blk, int nrvars, int corr) {
  u_coarse_ring<DIM>(P, fpool, blk[blockIdx.x], threadIdx.x, nrvars, corr);
}

// CoarseLoadingFunction on the correction: fine r = g - M(e) under each
// coarse cell; parent g(mb) = R(r) + M_c(ec) with the parent's base field.
template <int DIM>
__device__ __forceinline__ void u_coarse_load(const PatchDev* __restrict__ P, float* __restrict__ fpool, const Blk b,
                                              int tid) {
  const PatchDev& p = P[b.patch];
  int ci, cj, ck;
  if (!interior_cell<DIM>(p.cmx, b.start + tid, ci, cj, ck)) return;
  const PatchDev& par = P[p.parent];
  const float* e = fpool + p.eq;
  long long sy = p.qn[0], sz = (long long)p.qn[0] * p.qn[1];
  float c0 = p.cf[0], c1 = p.cf[1];
  float R0 = 0.f, R1 = 0.f;
  const int nk = DIM == 3 ? 2 : 1;
  for (int dk = 0; dk < nk; dk++)
    for (int dj = 0; dj < 2; dj++)
      for (int di = 0; di < 2; di++) {
        int i = 2 * ci - di, j = 2 * cj - dj, k = DIM == 3 ? 2 * ck - dk : 1;
        long long c = gofs<DIM>(p.qn, i, j, k);
        long long fc = iofs<DIM>(p.mx, i, j, k);
        Nbr<DIM> n(c, sy, sz);
        float m0, m1;
        mopn<DIM>(e, c, n, p.sq, fpool[p.ephi + fc], c0, c1, m0, m1);
        R0 += fpool[p.eg + fc] - m0;
        R1 += fpool[p.eg + p.sf + fc] - m1;
      }
  R0 *= DIM == 2 ? 0.25f : 0.125f;
  R1 *= DIM == 2 ? 0.25f : 0.125f;
  const float* ec = fpool + p.ecq;
  long long csy = p.cn[0], csz = (long long)p.cn[0] * p.cn[1];
  long long cc = gofs<DIM>(p.cn, ci, cj, ck);
  long long pf = iofs<DIM>(par.mx, p.mb[0] + ci - 1, p.mb[1] + cj - 1, DIM == 3 ? p.mb[2] + ck - 1 : 1);
  // the coarse operator reads the ec ring, which coarse_ring has filled
  Nbr<DIM> n(cc, csy, csz);
  float m0, m1;
  mopn<DIM>(ec, cc, n, p.sc, fpool[par.ephi + pf], par.cf[0], par.cf[1], m0, m1);
  fpool[par.eg + pf] = R0 + m0;
  fpool[par.eg + par.sf + pf] = R1 + m1;
}
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_mx_coarse_load(const PatchDev* __restrict__ P, float* __restrict__ fpool,
                                                           const Blk* __restrict__ blk) {
  u_coarse_load<DIM>(P, fpool, blk[blockIdx.x], threadIdx.x);
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
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_mx_prolong(const PatchDev* __restrict__ P, float* __restrict__ fpool,
                                                       const Blk* __restrict__ blk, int nrvars) {
  u_prolong<DIM>(P, fpool, blk[blockIdx.x], threadIdx.x, nrvars);
}

// step 3: qbar += e (whole ghosted array).  The
// same pass refreshes the base field phib of the next cycle and clears e,
// so the next cycle needs neither a separate prep pass over q nor a memset
// on this level.
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_mx_update(const PatchDev* __restrict__ P, double* __restrict__ pool,
                                                      float* __restrict__ fpool, const Blk* __restrict__ blk,
                                                      int nrvars, int nbase) {
  const Blk b = blk[blockIdx.x];
  const PatchDev& p = P[b.patch];
  int i, j, k;
  if (!ghosted_cell<DIM>(p.qn, p.gs, b.start + threadIdx.x, i, j, k)) return;
  bool interior = i >= 1 && i <= p.mx[0] && j >= 1 && j <= p.mx[1] && (DIM == 2 || (k >= 1 && k <= p.mx[2]));
  long long c = gofs<DIM>(p.qn, i, j, k);
  for (int v = 0; v < nrvars; v++) {
    double nq = pool[p.oq + v * p.sq + c] + (double)fpool[p.eq + v * p.sq + c];
    pool[p.oq + v * p.sq + c] = nq;
    fpool[p.eq + v * p.sq + c] = 0.0f;
    if (v < nbase && interior) fpool[p.ephi + v * p.sf + iofs<DIM>(p.mx, i, j, k)] = (float)nq;
  }
}

// FP64 residual rf = f - N(q) of the finest level and per-block sums of rf^2
// (ErrorAFAS, afasroutines.f90:113-233).  Same arithmetic as the plain
// path's norm kernel, but this translation unit lets the compiler fuse
// multiply-adds, which cuts FP64 pipe work by about a third; the mixed path
// needs the true residual to ~1e-15 relative, not bit-identical rounding.
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_mx_norm(const PatchDev* __restrict__ P, double* __restrict__ pool,
                                                    const Blk* __restrict__ blk, double* __restrict__ partial) {
  // kNormCells consecutive blocks of the interior list per CTA, so the
  // shuffle reduction (FP64 adds on every lane) is paid once per kNormCells
  // cells instead of once per cell
  __shared__ double red[2][kBlock / 32];
  double s0 = 0.0, s1 = 0.0;
  for (int sub = 0; sub < kNormCells; sub++) {
    const Blk b = blk[blockIdx.x * kNormCells + sub];
    if (b.patch < 0) break;
    const PatchDev& p = P[b.patch];
    int i, j, k;
    if (!interior_cell<DIM>(p.mx, b.start + threadIdx.x, i, j, k)) continue;
    const double* q0 = pool + p.oq;
    const double* q1 = q0 + p.sq;
    long long sy = p.qn[0], sz = (long long)p.qn[0] * p.qn[1];
    long long c = gofs<DIM>(p.qn, i, j, k);
    long long fc = iofs<DIM>(p.mx, i, j, k);
    Nbr<DIM> n(c, sy, sz);
    double phi = q0[c];
    double o0 = phi - p.c[0] * ulapn<DIM>(q1, c, n);
    double o1 = q1[c] - phi * phi * phi + p.c[1] * ulapn<DIM>(q0, c, n);
    double e0 = pool[p.of + fc] - o0;
    double e1 = pool[p.of + p.sf + fc] - o1;
    pool[p.orf + fc] = e0;
    pool[p.orf + p.sf + fc] = e1;
    s0 = fma(e0, e0, s0);
    s1 = fma(e1, e1, s1);
  }
  for (int o = 16; o > 0; o >>= 1) {
    s0 += __shfl_down_sync(0xffffffffu, s0, o);
    s1 += __shfl_down_sync(0xffffffffu, s1, o);
  }
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    red[0][w] = s0;
    red[1][w] = s1;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t0 = 0.0, t1 = 0.0;
    for (int m = 0; m < kBlock / 32; m++) {
      t0 += red[0][m];
      t1 += red[1][m];
    }
    partial[2 * blockIdx.x] = t0;
    partial[2 * blockIdx.x + 1] = t1;
  }
}

// Residual tracked in FP32 between FP64 evaluations: after qbar += e the
// new residual is exactly g - M(e) (M is the difference N(qbar+e) - N(qbar)),
// so g <- g - M(e) on the finest level gives the next right-hand side and,
// summed, the tracked norm.
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_mx_track(const PatchDev* __restrict__ P, float* __restrict__ fpool,
                                                     const Blk* __restrict__ blk, double* __restrict__ partial) {
  // sums of squares in FP32 (the tracked norm only decides when to
  // re-evaluate in FP64); one conversion per block, no FP64 shuffles
  __shared__ float red[2][kBlock / 32];
  const Blk b = blk[blockIdx.x];
  const PatchDev& p = P[b.patch];
  int i, j, k;
  float s0 = 0.f, s1 = 0.f;
  if (interior_cell<DIM>(p.mx, b.start + threadIdx.x, i, j, k)) {
    const float* e = fpool + p.eq;
    long long sy = p.qn[0], sz = (long long)p.qn[0] * p.qn[1];
    long long c = gofs<DIM>(p.qn, i, j, k);
    long long fc = iofs<DIM>(p.mx, i, j, k);
    Nbr<DIM> n(c, sy, sz);
    float m0, m1;
    mopn<DIM>(e, c, n, p.sq, fpool[p.ephi + fc], p.cf[0], p.cf[1], m0, m1);
    float g0 = fpool[p.eg + fc] - m0;
    float g1 = fpool[p.eg + p.sf + fc] - m1;
    fpool[p.eg + fc] = g0;
    fpool[p.eg + p.sf + fc] = g1;
    s0 = g0 * g0;
    s1 = g1 * g1;
  }
  for (int o = 16; o > 0; o >>= 1) {
    s0 += __shfl_down_sync(0xffffffffu, s0, o);
    s1 += __shfl_down_sync(0xffffffffu, s1, o);
  }
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    red[0][w] = s0;
    red[1][w] = s1;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float t0 = 0.f, t1 = 0.f;
    for (int m = 0; m < kBlock / 32; m++) {
      t0 += red[0][m];
      t1 += red[1][m];
    }
    partial[2 * blockIdx.x] = (double)t0;
    partial[2 * blockIdx.x + 1] = (double)t1;
  }
}

// ---------------------------------------------------------------------------
// The growth plugin (three variables phi, n, p; see fp64.cu) in correction
// form.  Base planes at ephi (sf each): phib, nb (the frozen phi and n),
// G = gamma (phi_old + 1)/2 and U = lambda (phi_old + 1)/2.  With
// w = phib + e_phi:
//   M0 = e_phi - c0 ULap(e_phi) + dt e_phi (3 phib w + e_phi^2) - dt G e_n
//   M1 = -c1 ULap(e_n) + U e_n
//   M2 = -c1 ULap(e_p) - cp (phib e_n + e_phi nb + e_phi e_n)
// and the smoother is the FP64 one (phi from its lagged equation with the
// current n, then n, then p from the new phi and n) rewritten for e so that
// no term cancels: e_phi = (g0 + dt G e_n + c0 sum(e_phi) - dt phib e_phi
// (2 phib + e_phi)) / (c2 + dt w^2), e_n = (g1 + c1 sum(e_n)) / (c3 + U),
// e_p = (g2 + c1 sum(e_p) + cp (phib e_n + e_phi nb + e_phi e_n)) / c3.

template <int DIM>
__device__ __forceinline__ void mop_growth(const float* e, long long c, const Nbr<DIM>& n, long long ps,
                                           const float* base, long long fc, long long sf, float c0, float c1,
                                           float dt, float cp, float* m) {
  const float* e0 = e;
  const float* e1 = e + ps;
  const float* e2 = e + 2 * ps;
  float pb = base[fc], nb = base[sf + fc], G = base[2 * sf + fc], U = base[3 * sf + fc];
  float x = e0[c], y = e1[c];
  m[0] = x - c0 * ulapn<DIM>(e0, c, n) + dt * x * (3.0f * pb * (pb + x) + x * x) - dt * G * y;
  m[1] = -c1 * ulapn<DIM>(e1, c, n) + U * y;
  m[2] = -c1 * ulapn<DIM>(e2, c, n) - cp * (pb * y + x * nb + x * y);
}

// step 1 for growth: base planes; g as in k_mx_prep (mode 0: base only,
// 1: from the stored rf, 2: f - N(qbar) with the FP64 growth operator)
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_mg_prep(const PatchDev* __restrict__ P, const double* __restrict__ pool,
                                                    float* __restrict__ fpool, const Blk* __restrict__ blk, int mode,
                                                    ProbParams pp) {
  const Blk b = blk[blockIdx.x];
  const PatchDev& p = P[b.patch];
  int i, j, k;
  if (!interior_cell<DIM>(p.mx, b.start + threadIdx.x, i, j, k)) return;
  long long c = gofs<DIM>(p.qn, i, j, k);
  long long fc = iofs<DIM>(p.mx, i, j, k);
  const double* q0 = pool + p.oq;
  const double* q1 = q0 + p.sq;
  const double* q2 = q1 + p.sq;
  double ol = pool[p.oqold + c];
  double G = pp.gamma * 0.5 * (ol + 1.0), U = pp.lambda * 0.5 * (ol + 1.0);
  float* base = fpool + p.ephi;
  base[fc] = (float)q0[c];
  base[p.sf + fc] = (float)q1[c];
  base[2 * p.sf + fc] = (float)G;
  base[3 * p.sf + fc] = (float)U;
  if (mode == 0) return;
  double r[3];
  if (mode == 1) {
    for (int v = 0; v < 3; v++) r[v] = pool[p.orf + v * p.sf + fc];
  } else {
    long long sy = p.qn[0], sz = (long long)p.qn[0] * p.qn[1];
    double phi = q0[c];
    double o0 = phi - p.c[0] * ulap<DIM>(q0, c, sy, sz) + pp.dt * phi * phi * phi - pp.dt * G * (q1[c] - pp.czero);
    double o1 = -p.c[1] * ulap<DIM>(q1, c, sy, sz) + U * q1[c];
    double o2 = -p.c[1] * ulap<DIM>(q2, c, sy, sz) - pp.cpress * phi * q1[c];
    r[0] = pool[p.of + fc] - o0;
    r[1] = pool[p.of + p.sf + fc] - o1;
    r[2] = pool[p.of + 2 * p.sf + fc] - o2;
  }
  for (int v = 0; v < 3; v++) fpool[p.eg + v * p.sf + fc] = (float)r[v];
}

template <int DIM>
__device__ __forceinline__ void u_mg_relax(const PatchDev* __restrict__ P, float* __restrict__ fpool, const Blk b,
                                           int tid, int ipass, float dt, float cp) {
  const PatchDev& p = P[b.patch];
  int i, j, k;
  if (!color_cell<DIM>(p, b.start + tid, ipass, i, j, k)) return;
  float* e0 = fpool + p.eq;
  float* e1 = e0 + p.sq;
  float* e2 = e1 + p.sq;
  long long sy = p.qn[0], sz = (long long)p.qn[0] * p.qn[1];
  long long c = gofs<DIM>(p.qn, i, j, k);
  long long fc = iofs<DIM>(p.mx, i, j, k);
  Nbr<DIM> n(c, sy, sz);
  const float* base = fpool + p.ephi;
  const float* g = fpool + p.eg;
  float pb = base[fc], nb = base[p.sf + fc], G = base[2 * p.sf + fc], U = base[3 * p.sf + fc];
  float c0 = p.cf[0], c1 = p.cf[1], c2 = p.cf[2], c3 = p.cf[3];
  float s0 = e0[n.xm] + e0[n.xp] + e0[n.ym] + e0[n.yp];
  float s1 = e1[n.xm] + e1[n.xp] + e1[n.ym] + e1[n.yp];
  float s2 = e2[n.xm] + e2[n.xp] + e2[n.ym] + e2[n.yp];
  if (DIM == 3) {
    s0 += e0[n.zm] + e0[n.zp];
    s1 += e1[n.zm] + e1[n.zp];
    s2 += e2[n.zm] + e2[n.zp];
  }
  float x = e0[c], y = e1[c];
  float w = pb + x;
  float xn = (g[fc] + dt * G * y + c0 * s0 - dt * pb * x * (2.0f * pb + x)) / (c2 + dt * w * w);
  float yn = (g[p.sf + fc] + c1 * s1) / (c3 + U);
  float zn = (g[2 * p.sf + fc] + c1 * s2 + cp * (pb * yn + xn * nb + xn * yn)) / c3;
  e0[c] = xn;
  e1[c] = yn;
  e2[c] = zn;
}
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_mg_relax(const PatchDev* __restrict__ P, float* __restrict__ fpool,
                                                     const Blk* __restrict__ blk, int ipass, float dt, float cp) {
  u_mg_relax<DIM>(P, fpool, blk[blockIdx.x], threadIdx.x, ipass, dt, cp);
}

// CoarseLoadingFunction on the growth correction (see u_coarse_load)
template <int DIM>
__device__ __forceinline__ void u_mg_coarse_load(const PatchDev* __restrict__ P, float* __restrict__ fpool,
                                                 const Blk b, int tid, float dt, float cp) {
  const PatchDev& p = P[b.patch];
  int ci, cj, ck;
  if (!interior_cell<DIM>(p.cmx, b.start + tid, ci, cj, ck)) return;
  const PatchDev& par = P[p.parent];
  const float* e = fpool + p.eq;
  long long sy = p.qn[0], sz = (long long)p.qn[0] * p.qn[1];
  float R[3] = {0.f, 0.f, 0.f};
  const int nk = DIM == 3 ? 2 : 1;
  for (int dk = 0; dk < nk; dk++)
    for (int dj = 0; dj < 2; dj++)
      for (int di = 0; di < 2; di++) {
        int i = 2 * ci - di, j = 2 * cj - dj, k = DIM == 3 ? 2 * ck - dk : 1;
        long long c = gofs<DIM>(p.qn, i, j, k);
        long long fc = iofs<DIM>(p.mx, i, j, k);
        Nbr<DIM> n(c, sy, sz);
        float m[3];
        mop_growth<DIM>(e, c, n, p.sq, fpool + p.ephi, fc, p.sf, p.cf[0], p.cf[1], dt, cp, m);
        for (int v = 0; v < 3; v++) R[v] += fpool[p.eg + v * p.sf + fc] - m[v];
      }
  const float rs = DIM == 2 ? 0.25f : 0.125f;
  const float* ec = fpool + p.ecq;
  long long csy = p.cn[0], csz = (long long)p.cn[0] * p.cn[1];
  long long cc = gofs<DIM>(p.cn, ci, cj, ck);
  long long pf = iofs<DIM>(par.mx, p.mb[0] + ci - 1, p.mb[1] + cj - 1, DIM == 3 ? p.mb[2] + ck - 1 : 1);
  Nbr<DIM> n(cc, csy, csz);
  float m[3];
  mop_growth<DIM>(ec, cc, n, p.sc, fpool + par.ephi, pf, par.sf, par.cf[0], par.cf[1], dt, cp, m);
  for (int v = 0; v < 3; v++) fpool[par.eg + v * par.sf + pf] = R[v] * rs + m[v];
}
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_mg_coarse_load(const PatchDev* __restrict__ P, float* __restrict__ fpool,
                                                           const Blk* __restrict__ blk, float dt, float cp) {
  u_mg_coarse_load<DIM>(P, fpool, blk[blockIdx.x], threadIdx.x, dt, cp);
}

// tracked residual g <- g - M(e) of the growth correction; per-block sums of
// squares of the three variables
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_mg_track(const PatchDev* __restrict__ P, float* __restrict__ fpool,
                                                     const Blk* __restrict__ blk, double* __restrict__ partial,
                                                     float dt, float cp) {
  __shared__ float red[3][kBlock / 32];
  const Blk b = blk[blockIdx.x];
  const PatchDev& p = P[b.patch];
  int i, j, k;
  float s[3] = {0.f, 0.f, 0.f};
  if (interior_cell<DIM>(p.mx, b.start + threadIdx.x, i, j, k)) {
    long long sy = p.qn[0], sz = (long long)p.qn[0] * p.qn[1];
    long long c = gofs<DIM>(p.qn, i, j, k);
    long long fc = iofs<DIM>(p.mx, i, j, k);
    Nbr<DIM> n(c, sy, sz);
    float m[3];
    mop_growth<DIM>(fpool + p.eq, c, n, p.sq, fpool + p.ephi, fc, p.sf, p.cf[0], p.cf[1], dt, cp, m);
    for (int v = 0; v < 3; v++) {
      float gv = fpool[p.eg + v * p.sf + fc] - m[v];
      fpool[p.eg + v * p.sf + fc] = gv;
      s[v] = gv * gv;
    }
  }
  for (int o = 16; o > 0; o >>= 1)
    for (int v = 0; v < 3; v++) s[v] += __shfl_down_sync(0xffffffffu, s[v], o);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0)
    for (int v = 0; v < 3; v++) red[v][w] = s[v];
  __syncthreads();
  if (threadIdx.x == 0)
    for (int v = 0; v < 3; v++) {
      float t = 0.f;
      for (int m = 0; m < kBlock / 32; m++) t += red[v][m];
      partial[3 * blockIdx.x + v] = (double)t;
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

__global__ void __launch_bounds__(kBlock) k_ghost32_stage(const PatchDev* __restrict__ P, float* __restrict__ fpool,
                                                          const GhostOp* __restrict__ ops, int n, int nrvars) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  GhostOp g = ops[t];
  ghost32_apply(P, fpool, g, nrvars);
}

__global__ void __launch_bounds__(kBlock) k_ghost32_program(const PatchDev* __restrict__ P, float* __restrict__ fpool,
                                                            const GhostOp* __restrict__ ops,
                                                            const int* __restrict__ stage_off, int nstages,
                                                            int nrvars) {
  for (int s = 0; s < nstages; s++) {
    for (int t = stage_off[s] + threadIdx.x; t < stage_off[s + 1]; t += blockDim.x) {
      GhostOp g = ops[t];
      ghost32_apply(P, fpool, g, nrvars);
    }
    __syncthreads();
  }
}

// The coarse tail of a V-cycle in one CTA.  Below some level every level of
// a hierarchy is small (a few thousand cells), and the launches of its
// V-cycle (~20 per level) cost more than their work.  The tail program is
// the sequence of operations mx_vcycle would launch from that level down,
// recorded once on the host; this kernel executes it phase by phase, every
// work-list block of a phase by the whole CTA (256 threads = one block's
// units), with a barrier between phases.  Each unit computes exactly what
// the stand-alone kernel computes, so results are bit-identical.

template <int DIM, int PR>
__device__ __forceinline__ void run_tail(const PatchDev* __restrict__ P, float* fpool, const TailPhase* __restrict__ ph,
                                         int nph, int nrvars, float dt, float cp) {
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
        case kTRelax:
          if (PR == kGrowth) u_mg_relax<DIM>(P, fpool, bb, threadIdx.x, f.arg, dt, cp);
          else u_relax<DIM>(P, fpool, bb, threadIdx.x, f.arg);
          break;
        case kTRestrict: u_restrict<DIM>(P, fpool, bb, threadIdx.x, nrvars); break;
        case kTRing: u_coarse_ring<DIM>(P, fpool, bb, threadIdx.x, nrvars, f.arg); break;
        case kTLoad:
          if (PR == kGrowth) u_mg_coarse_load<DIM>(P, fpool, bb, threadIdx.x, dt, cp);
          else u_coarse_load<DIM>(P, fpool, bb, threadIdx.x);
          break;
        default: u_prolong<DIM>(P, fpool, bb, threadIdx.x, nrvars); break;
      }
    }
    __syncthreads();
  }
}

template <int DIM, int PR>
__global__ void __launch_bounds__(kBlock) k_mx_tail(const PatchDev* __restrict__ P, float* __restrict__ fpool,
                                                   const TailPhase* __restrict__ ph, int nph, int nrvars, float dt,
                                                   float cp) {
  run_tail<DIM, PR>(P, fpool, ph, nph, nrvars, dt, cp);
}

// The same with the tail levels' arrays staged in shared memory: P is a
// patch table whose tail patches address the block's shared memory, so the
// phases run on on-chip copies; the modified arrays are written back at the
// end.  Same arithmetic on the same values: results are bit-identical.
template <int DIM, int PR>
__global__ void __launch_bounds__(kBlock) k_mx_tail_smem(const PatchDev* __restrict__ P, float* __restrict__ fpool,
                                                        const TailPhase* __restrict__ ph, int nph, int nrvars,
                                                        float dt, float cp, const StageSeg* __restrict__ segs,
                                                        int nsegs) {
  extern __shared__ float sm[];
  for (int x = 0; x < nsegs; x++) {
    const StageSeg sg = segs[x];
    for (int t = threadIdx.x; t < sg.n; t += blockDim.x) sm[sg.s + t] = fpool[sg.g + t];
  }
  __syncthreads();
  run_tail<DIM, PR>(P, sm, ph, nph, nrvars, dt, cp);
  for (int x = 0; x < nsegs; x++) {
    const StageSeg sg = segs[x];
    if (!sg.out) continue;
    for (int t = threadIdx.x; t < sg.n; t += blockDim.x) fpool[sg.g + t] = sm[sg.s + t];
  }
}

// ---------------------------------------------------------------------------
// schedule

#define MX_LAUNCH(H, kind, KER, ...)                                                        \
  do {                                                                                      \
    int nb__ = L.nblk[kind];                                                                \
    if (nb__ > 0) {                                                                         \
      if ((H).ndims == 2) KER<2><<<nb__, kBlock, 0, (H).s>>>(__VA_ARGS__);                  \
      else KER<3><<<nb__, kBlock, 0, (H).s>>>(__VA_ARGS__);                                 \
      int r__ = after_launch(H, 1);                                                         \
      if (r__) return r__;                                                                  \
    }                                                                                       \
  } while (0)

#define MX_LAUNCH_W MX_LAUNCH

// the tail program being recorded (mx_vcycle records instead of launching)
std::vector<TailPhase>* rec_of(Hier& H) { return static_cast<std::vector<TailPhase>*>(H.rec); }

int mx_set_ghost(Hier& H, int level, int ipass) {
  GhostProg& g = H.L(level).gp[ipass];
  int nst = (int)g.stage_off.size() - 1;
  if (nst <= 0) return BSAMG_OK;
  if (auto* rec = rec_of(H)) {
    rec->push_back(TailPhase{kTGhost, 0, 0, nst, nullptr, g.d_ops, g.d_stage_off});
    return BSAMG_OK;
  }
  int nops = g.stage_off[nst];
  if (nops <= 2048) {
    k_ghost32_program<<<1, kBlock, 0, H.s>>>(H.dP, H.fpool, g.d_ops, g.d_stage_off, nst, H.nrvars);
    return after_launch(H, 1);
  }
  for (int s = 0; s < nst; s++) {
    int n = g.stage_off[s + 1] - g.stage_off[s];
    if (n <= 0) continue;
    k_ghost32_stage<<<(n + kBlock - 1) / kBlock, kBlock, 0, H.s>>>(H.dP, H.fpool, g.d_ops + g.stage_off[s], n,
                                                                    H.nrvars);
    int r = after_launch(H, 1);
    if (r) return r;
  }
  return BSAMG_OK;
}

// one work-list operation of the V-cycle: launched, or recorded into the
// tail program
int mx_op(Hier& H, int level, int kind, int op, int arg) {
  LevelT& L = H.L(level);
  if (auto* rec = rec_of(H)) {
    if (L.nblk[kind] > 0) rec->push_back(TailPhase{op, arg, L.nblk[kind], 0, L.d_blk[kind], nullptr, nullptr});
    return BSAMG_OK;
  }
  switch (op) {
    case kTRelax:
      if (H.problem == kGrowth)
        MX_LAUNCH_W(H, kind, k_mg_relax, H.dP, H.fpool, L.d_blk[kind], arg, (float)H.pp.dt, (float)H.pp.cpress);
      else
        MX_LAUNCH_W(H, kind, k_mx_relax, H.dP, H.fpool, L.d_blk[kind], arg);
      break;
    case kTRestrict: MX_LAUNCH(H, kind, k_mx_restrict, H.dP, H.fpool, L.d_blk[kind], H.nrvars); break;
    case kTRing: MX_LAUNCH_W(H, kind, k_mx_coarse_ring, H.dP, H.fpool, L.d_blk[kind], H.nrvars, arg); break;
    case kTLoad:
      if (H.problem == kGrowth)
        MX_LAUNCH_W(H, kind, k_mg_coarse_load, H.dP, H.fpool, L.d_blk[kind], (float)H.pp.dt, (float)H.pp.cpress);
      else
        MX_LAUNCH_W(H, kind, k_mx_coarse_load, H.dP, H.fpool, L.d_blk[kind]);
      break;
    default: MX_LAUNCH_W(H, kind, k_mx_prolong, H.dP, H.fpool, L.d_blk[kind], H.nrvars); break;
  }
  return BSAMG_OK;
}

int mx_level_relax(Hier& H, int level, int nsmooth) {
  for (int pass = 1; pass <= nsmooth; pass++)
    for (int rb = 1; rb <= 2; rb++) {
      int r = mx_op(H, level, kKindColor, kTRelax, rb);
      if (!r) r = mx_set_ghost(H, level, rb);
      if (r) return r;
    }
  return BSAMG_OK;
}

int mx_vcycle(Hier& H, int level, int minlevel, int nsmooth) {
  if (!H.rec && level <= H.tail_level && level >= minlevel) {
    auto it = H.mx_tail_progs.find(std::make_tuple(level, minlevel, nsmooth));
    if (it != H.mx_tail_progs.end()) {  // the whole V-cycle from here down in one CTA
      const Hier::TailProg& T = it->second;
      const TailPhase* ph = static_cast<const TailPhase*>(T.phases);
      float dt = (float)H.pp.dt, cp = (float)H.pp.cpress;
      int n = T.nph, nr = H.nrvars;
      if (T.smem_bytes) {
        const PatchDev* sp = static_cast<const PatchDev*>(T.shadow);
        const StageSeg* sg = static_cast<const StageSeg*>(T.segs);
        int sb = T.smem_bytes, ns = T.nsegs;
        if (H.problem == kGrowth) {
          if (H.ndims == 2) k_mx_tail_smem<2, kGrowth><<<1, kBlock, sb, H.s>>>(sp, H.fpool, ph, n, nr, dt, cp, sg, ns);
          else k_mx_tail_smem<3, kGrowth><<<1, kBlock, sb, H.s>>>(sp, H.fpool, ph, n, nr, dt, cp, sg, ns);
        } else {
          if (H.ndims == 2) k_mx_tail_smem<2, kCH><<<1, kBlock, sb, H.s>>>(sp, H.fpool, ph, n, nr, dt, cp, sg, ns);
          else k_mx_tail_smem<3, kCH><<<1, kBlock, sb, H.s>>>(sp, H.fpool, ph, n, nr, dt, cp, sg, ns);
        }
      } else if (H.problem == kGrowth) {
        if (H.ndims == 2) k_mx_tail<2, kGrowth><<<1, kBlock, 0, H.s>>>(H.dP, H.fpool, ph, n, nr, dt, cp);
        else k_mx_tail<3, kGrowth><<<1, kBlock, 0, H.s>>>(H.dP, H.fpool, ph, n, nr, dt, cp);
      } else {
        if (H.ndims == 2) k_mx_tail<2, kCH><<<1, kBlock, 0, H.s>>>(H.dP, H.fpool, ph, n, nr, dt, cp);
        else k_mx_tail<3, kCH><<<1, kBlock, 0, H.s>>>(H.dP, H.fpool, ph, n, nr, dt, cp);
      }
      return after_launch(H, 1);
    }
  }
  int r = mx_level_relax(H, level, nsmooth);
  if (r) return r;
  if (level > minlevel) {
    if ((r = mx_op(H, level, kKindCoarse, kTRestrict, 0))) return r;
    if ((r = mx_set_ghost(H, level - 1, 0))) return r;
    if ((r = mx_op(H, level, kKindCGhost, kTRing, 0))) return r;
    if ((r = mx_op(H, level, kKindCoarse, kTLoad, 0))) return r;
    if ((r = mx_vcycle(H, level - 1, minlevel, nsmooth))) return r;
    if ((r = mx_op(H, level, kKindCGhost, kTRing, 1))) return r;
    if ((r = mx_op(H, level, kKindProl, kTProlong, 0))) return r;
    if ((r = mx_set_ghost(H, level, 0))) return r;
    if ((r = mx_level_relax(H, level, nsmooth))) return r;
  }
  return BSAMG_OK;
}

// Record and upload the tail program of (minlevel, nsmooth) once, outside
// any stream capture.
int mx_prepare_tail(Hier& H, int finest, int minlevel, int nsmooth) {
  int start = std::min(finest, H.tail_level);
  if (start < minlevel) return BSAMG_OK;
  auto key = std::make_tuple(start, minlevel, nsmooth);
  if (H.mx_tail_progs.count(key)) return BSAMG_OK;
  std::vector<TailPhase> prog;
  H.rec = &prog;
  int r = mx_vcycle(H, start, minlevel, nsmooth);
  H.rec = nullptr;
  if (r) return r;
  Hier::TailProg T;
  T.nph = (int)prog.size();
  if (!prog.empty()) {
    cudaError_t e = dev_alloc(H, &T.phases, sizeof(TailPhase) * prog.size());
    if (e == cudaSuccess)  // staged from pageable memory before it returns
      e = cudaMemcpyAsync(T.phases, prog.data(), sizeof(TailPhase) * prog.size(), cudaMemcpyHostToDevice, H.s);
    if (e != cudaSuccess) return cuda_fail(e, "tail program upload");
  }
  // shared-memory staging of the tail levels' FP32 arrays (e, ec, g: read
  // and written back; base fields: read) when they fit
  std::vector<PatchDev> shadow = H.hP;
  std::vector<StageSeg> segs;
  long long so = 0;
  long long nbase = H.problem == kGrowth ? 4 : 1;
  auto add = [&](long long g, long long n, int out) {
    segs.push_back(StageSeg{g, (int)so, (int)n, out, 0});
    long long at = so;
    so += (n + 3) & ~3LL;
    return at;
  };
  for (size_t p = 0; p < H.patches.size(); p++) {
    const HostPatch& P = H.patches[p];
    if (P.level < minlevel || P.level > start) continue;
    PatchDev& D = shadow[p];
    long long zq = origin_of(H, P.qn), zc = origin_of(H, P.cn);  // staged from the arrays' starts
    D.eq = add(P.e_oq, (long long)H.nrvars * P.sq, 1) + zq;
    D.ecq = add(P.e_oqc, (long long)H.nrvars * P.sc, 1) + zc;
    D.eg = add(D.eg, (long long)H.nrvars * P.sf, 1);
    D.ephi = add(D.ephi, nbase * P.sf, 0);
  }
  if (so * (long long)sizeof(float) <= kTailSmemMax && !segs.empty()) {
    T.smem_bytes = (int)(so * sizeof(float));
    T.nsegs = (int)segs.size();
    static std::atomic<unsigned long long> attr[2][2];  // the kernels' shared-memory limit, per device
    int a = H.ndims - 2, b = H.problem == kGrowth;
    if (needs_setup(attr[a][b], H.ctx->device)) {
      cudaError_t e;
      if (H.problem == kGrowth)
        e = H.ndims == 2 ? cudaFuncSetAttribute(k_mx_tail_smem<2, kGrowth>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTailSmemMax)
                         : cudaFuncSetAttribute(k_mx_tail_smem<3, kGrowth>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTailSmemMax);
      else
        e = H.ndims == 2 ? cudaFuncSetAttribute(k_mx_tail_smem<2, kCH>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTailSmemMax)
                         : cudaFuncSetAttribute(k_mx_tail_smem<3, kCH>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTailSmemMax);
      if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(tail)");
      mark_setup(attr[a][b], H.ctx->device);
    }
    cudaError_t e = dev_alloc(H, &T.shadow, sizeof(PatchDev) * shadow.size());
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(T.shadow, shadow.data(), sizeof(PatchDev) * shadow.size(), cudaMemcpyHostToDevice, H.s);
    T.hshadow = shadow;
    if (e == cudaSuccess) e = dev_alloc(H, &T.segs, sizeof(StageSeg) * segs.size());
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(T.segs, segs.data(), sizeof(StageSeg) * segs.size(), cudaMemcpyHostToDevice, H.s);
    if (e != cudaSuccess) return cuda_fail(e, "tail staging upload");
  }
  H.mx_tail_progs[key] = T;
  return BSAMG_OK;
}

// FP32 pool layout.  Region order: e of levels >= 0, e of levels < 0 (so
// the coarse corrections can be cleared with one memset), all ec, all g, all
// phib.  Returns per patch {e, ec, g, phib} offsets.
std::vector<long long> layout(const Hier& H, size_t* total, size_t* e_len, size_t* e_coarse_off) {
  size_t np = H.patches.size();
  std::vector<long long> off(4 * np);
  long long o = 0;
  auto al = [](long long x) { return (x + 63) & ~63LL; };
  for (int pass = 0; pass < 2; pass++) {
    if (pass == 1) *e_coarse_off = (size_t)o;
    for (size_t p = 0; p < np; p++)
      if ((H.patches[p].level < 0) == (pass == 1)) {
        off[4 * p] = o;
        o = al(o + H.patches[p].sq * H.nrvars);
      }
  }
  *e_len = (size_t)o;
  for (size_t p = 0; p < np; p++) { off[4 * p + 1] = o; o = al(o + H.patches[p].sc * H.nrvars); }
  for (size_t p = 0; p < np; p++) { off[4 * p + 2] = o; o = al(o + H.patches[p].sf * H.nrvars); }
  // base fields: phib (CH); phib, nb, G, U (growth)
  long long nbase = H.problem == kGrowth ? 4 : 1;
  for (size_t p = 0; p < np; p++) { off[4 * p + 3] = o; o = al(o + nbase * H.patches[p].sf); }
  *total = (size_t)o;
  return off;
}

int mx_norm(Hier& H, int level, int errortype) {
  LevelT& L = H.L(level);
  if (H.problem == kGrowth) {  // the plain path's FP64 residual (three variables)
    int r = after_launch(H, launch_norm_partial(H.lc(), L.d_blk[kKindInterior], L.nblk[kKindInterior], H.d_partial, 1));
    if (r) return r;
    return after_launch(H, launch_norm_finish(H.s, H.d_partial, L.nblk[kKindInterior], H.nrvars, L.count, errortype,
                                              H.d_norm, H.d_nonfinite));
  }
  int nb = (L.nblk[kKindInterior] + kNormCells - 1) / kNormCells;
  if (nb <= 0) return BSAMG_OK;
  // the interior list is padded with patch = -1 entries to a multiple of
  // kNormCells (see mixed_alloc)
  if (H.ndims == 2) {
    k_mx_norm<2><<<nb, kBlock, 0, H.s>>>(H.dP, H.pool, H.mx_norm_blk[level + kMaxDepth], H.d_partial);
  } else {
    k_mx_norm<3><<<nb, kBlock, 0, H.s>>>(H.dP, H.pool, H.mx_norm_blk[level + kMaxDepth], H.d_partial);
  }
  int r = after_launch(H, 1);
  if (r) return r;
  return after_launch(H, launch_norm_finish(H.s, H.d_partial, nb, H.nrvars, L.count, errortype, H.d_norm,
                                            H.d_nonfinite));
}

int to_host(Hier& H) {
  cudaError_t ce = cudaMemcpyAsync(H.h_norm, H.d_norm, 2 * sizeof(double), cudaMemcpyDeviceToHost, H.s);
  if (ce != cudaSuccess) return cuda_fail(ce, "cudaMemcpyAsync(norm)");
  ce = cudaMemcpyAsync(H.h_nonfinite, H.d_nonfinite, sizeof(int), cudaMemcpyDeviceToHost, H.s);
  if (ce != cudaSuccess) return cuda_fail(ce, "cudaMemcpyAsync(nonfinite)");
  return BSAMG_OK;
}

// FillDown of q in FP64 (restriction to the parents, with their ghosts)
int mx_fill_down_q(Hier& H, int finest, int minlevel) { return enq_fill_down(H, 2, finest, minlevel); }

// one outer iteration; resync: take g on the finest level from the FP64 rf
int mx_iteration(Hier& H, int finest, int minlevel, int nsmooth, int errortype, bool resync) {
  int r__ = 0;
  // e of levels >= 0 was cleared by the previous update pass (or by
  // mixed_iterations before the first cycle); clear the coarse ones
  if (H.e_coarse_len) {
    cudaError_t ce = cudaMemsetAsync(H.fpool + H.e_coarse_off, 0, H.e_coarse_len * sizeof(float), H.s);
    if (ce != cudaSuccess) return cuda_fail(ce, "cudaMemsetAsync(e)");
  }
  for (int level = finest; level >= minlevel; level--) {
    LevelT& L = H.L(level);
    // phib of levels >= 0 comes from the update pass; g of the finest level
    // from the FP64 rf after a resync, else from the tracked update
    if (level == finest && !resync) continue;
    int mode = level < 0 ? 0 : (level == finest ? 1 : 2);
    bool all_coarse = level < 0 && minlevel == H.minlevel && H.mx_prep_coarse_n > 0;
    const Blk* blk = all_coarse ? H.mx_prep_coarse : L.d_blk[kKindInterior];
    int nb = all_coarse ? H.mx_prep_coarse_n : L.nblk[kKindInterior];
    if (nb > 0) {  // all levels below the root at once (base fields only)
      if (H.problem == kGrowth) {
        if (H.ndims == 2) k_mg_prep<2><<<nb, kBlock, 0, H.s>>>(H.dP, H.pool, H.fpool, blk, mode, H.pp);
        else k_mg_prep<3><<<nb, kBlock, 0, H.s>>>(H.dP, H.pool, H.fpool, blk, mode, H.pp);
      } else {
        if (H.ndims == 2) k_mx_prep<2><<<nb, kBlock, 0, H.s>>>(H.dP, H.pool, H.fpool, blk, mode);
        else k_mx_prep<3><<<nb, kBlock, 0, H.s>>>(H.dP, H.pool, H.fpool, blk, mode);
      }
      if ((r__ = after_launch(H, 1))) return r__;
    }
    if (all_coarse) break;
  }
  int r = mx_vcycle(H, finest, minlevel, nsmooth);
  if (r) return r;
  // tracked residual g - M(e): M needs this cycle's base field, so it runs
  // before the update pass replaces phib with the new base
  {
    LevelT& L = H.L(finest);
    if (H.problem == kGrowth)
      MX_LAUNCH_W(H, kKindInterior, k_mg_track, H.dP, H.fpool, L.d_blk[kKindInterior], H.d_partial,
                  (float)H.pp.dt, (float)H.pp.cpress);
    else
      MX_LAUNCH_W(H, kKindInterior, k_mx_track, H.dP, H.fpool, L.d_blk[kKindInterior], H.d_partial);
    if ((r = after_launch(H, launch_norm_finish(H.s, H.d_partial, L.nblk[kKindInterior], H.nrvars, L.count,
                                                 errortype, H.d_norm, H.d_nonfinite))))
      return r;
  }
  for (int level = finest; level >= 0; level--) {
    LevelT& L = H.L(level);
    MX_LAUNCH_W(H, kKindFGhost, k_mx_update, H.dP, H.pool, H.fpool, L.d_blk[kKindFGhost], H.nrvars,
                H.problem == kGrowth ? 2 : 1);
  }
  if ((r = mx_fill_down_q(H, finest, minlevel))) return r;
  // refinement levels: ghosts from the updated FP64 state (coarse-fine
  // interpolation reads the parent values FillDown just restricted)
  for (int level = 1; level <= finest; level++)
    if ((r = enq_set_ghost(H, level, 0))) return r;
  return to_host(H);
}

int mx_verify(Hier& H, int finest, int errortype) {
  int r = mx_norm(H, finest, errortype);
  if (r) return r;
  return to_host(H);
}

}  // namespace

size_t mixed_pool_bytes(const Hier& H) {
  if (H.problem != kCH && H.problem != kGrowth) return 0;
  size_t n, ne, ec;
  layout(H, &n, &ne, &ec);
  return n * sizeof(float);
}

int mixed_alloc(Hier& H) {
  if (H.problem != kCH && H.problem != kGrowth) return BSAMG_OK;
  if (H.box) {
    H.fpool_elems = box_layout(H);
    cudaError_t e = dev_alloc(H, (void**)&H.fpool, H.fpool_elems * sizeof(float));
    if (e != cudaSuccess) return cuda_fail(e, "device allocation (fpool)");
    e = cudaMemsetAsync(H.fpool, 0, H.fpool_elems * sizeof(float), H.s);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(fpool)");
    return BSAMG_OK;
  }
  size_t n, ne, ec;
  std::vector<long long> off = layout(H, &n, &ne, &ec);
  H.e_len = ne;
  H.e_coarse_off = ec;
  H.e_coarse_len = ne - ec;
  for (size_t p = 0; p < H.patches.size(); p++) {
    HostPatch& P = H.patches[p];
    P.e_oq = off[4 * p];
    P.e_oqc = off[4 * p + 1];
    P.e_of = off[4 * p + 2];
    P.e_ophi = off[4 * p + 3];
  }
  H.fpool_elems = n;
  cudaError_t e = dev_alloc(H, (void**)&H.fpool, n * sizeof(float));
  if (e != cudaSuccess) return cuda_fail(e, "device allocation (fpool)");
  e = cudaMemsetAsync(H.fpool, 0, n * sizeof(float), H.s);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(fpool)");
  return BSAMG_OK;
}

void mixed_free(Hier& H) {
  if (H.fpool) cudaFreeAsync(H.fpool, H.s);
  H.fpool = nullptr;
  if (H.mx_prep_coarse) cudaFreeAsync(H.mx_prep_coarse, H.s);
  H.mx_prep_coarse = nullptr;
  for (auto& kv : H.mx_tail_progs) free_tail(H, kv.second);
  H.mx_tail_progs.clear();
  for (int l = 0; l < kNLev; l++) {
    if (H.mx_norm_blk[l]) cudaFreeAsync(H.mx_norm_blk[l], H.s);
    H.mx_norm_blk[l] = nullptr;
  }
}

int mixed_tables(Hier& H) {
  if ((H.problem != kCH && H.problem != kGrowth) || !H.fpool || H.box) return BSAMG_OK;
  for (int l = H.minlevel; l <= H.maxlevel; l++) {
    // interior work list padded with patch = -1 to a multiple of kNormCells
    std::vector<Blk> v;
    for (int p : H.L(l).patches) {
      const HostPatch& P = H.patches[p];
      long long units = (long long)P.mx[0] * P.mx[1] * P.mx[2];
      for (long long s = 0; s < units; s += kBlock) v.push_back(Blk{p, (int)s});
    }
    while (v.size() % kNormCells) v.push_back(Blk{-1, 0});
    Blk* d = nullptr;
    cudaError_t e = dev_alloc(H, (void**)&d, sizeof(Blk) * v.size());
    if (e != cudaSuccess) return cuda_fail(e, "device allocation (norm list)");
    // staged from pageable memory before the call returns: v may go
    e = cudaMemcpyAsync(d, v.data(), sizeof(Blk) * v.size(), cudaMemcpyHostToDevice, H.s);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(norm list)");
    H.mx_norm_blk[l + kMaxDepth] = d;
    H.bytes += sizeof(Blk) * v.size();
  }
  // the interior lists of all levels below the root, concatenated
  std::vector<Blk> v;
  for (int l = H.minlevel; l < 0; l++)
    for (int p : H.L(l).patches) {
      const HostPatch& P = H.patches[p];
      long long units = (long long)P.mx[0] * P.mx[1] * P.mx[2];
      for (long long s = 0; s < units; s += kBlock) v.push_back(Blk{p, (int)s});
    }
  if (!v.empty()) {
    cudaError_t e = dev_alloc(H, (void**)&H.mx_prep_coarse, sizeof(Blk) * v.size());
    if (e == cudaSuccess)  // staged from pageable memory before it returns
      e = cudaMemcpyAsync(H.mx_prep_coarse, v.data(), sizeof(Blk) * v.size(), cudaMemcpyHostToDevice, H.s);
    if (e != cudaSuccess) return cuda_fail(e, "coarse prep list");
    H.mx_prep_coarse_n = (int)v.size();
    H.bytes += sizeof(Blk) * v.size();
  }
  return BSAMG_OK;
}

void set_tail(Hier& H, long long cells) {
  // the highest level whose level and every level below it together hold at
  // most `cells` interior cells runs the rest of the V-cycle in one CTA
  for (auto* progs : {&H.mx_tail_progs, &H.fp_tail_progs}) {
    for (auto& kv : *progs) free_tail(H, kv.second);
    progs->clear();
  }
  H.tail_cells = cells;
  H.tail_level = -kMaxDepth - 2;
  long long sum = 0;
  for (int l = H.minlevel; l <= H.maxlevel; l++) {
    for (int p : H.L(l).patches) {
      const HostPatch& P = H.patches[p];
      sum += (long long)P.mx[0] * P.mx[1] * P.mx[2];
    }
    if (sum > cells) break;
    H.tail_level = l;
  }
}

int mixed_enq_relax(Hier& H, int level, int ipass) {
  if ((H.problem != kCH && H.problem != kGrowth) || !H.fpool) return BSAMG_ERR_UNSUPPORTED;
  if (H.box) return box_enq_relax(H, level, ipass);
  return mx_op(H, level, kKindColor, kTRelax, ipass);
}

int mixed_iterations(Hier& H, int finest, int minlevel, int nsmooth, int maxvcycles, double tol, int errortype,
                     int strict, int* ncycles, double* residuals) {
  if ((H.problem != kCH && H.problem != kGrowth) || !H.fpool) return BSAMG_ERR_UNSUPPORTED;
  // the first outer iteration takes its right-hand side from the FP64
  // residual of the finest level
  int r = mx_norm(H, finest, errortype);
  if (r) return r;
  if ((r = to_host(H))) return r;
  if (int rw = stream_wait(H)) return rw;
  double r_sync = H.h_norm[0];  // FP64 residual the current g was taken from
  if ((r = mx_prepare_tail(H, finest, minlevel, nsmooth))) return r;
  Hier::GraphRec *ga = nullptr, *gt = nullptr, *gv = nullptr;
  auto key = [&](int m) { return std::make_tuple(m, finest, minlevel, nsmooth, errortype); };
  if ((r = capture_graph(H, key(11), [&] { return mx_iteration(H, finest, minlevel, nsmooth, errortype, true); },
                         &ga)))
    return r;
  if ((r = capture_graph(H, key(13), [&] { return mx_verify(H, finest, errortype); }, &gv))) return r;
  // With refinement levels the coarse-fine ghosts of the finest level are
  // re-interpolated from the updated parents after every cycle, which
  // g - M(e) does not see; there the FP64 residual is evaluated every cycle.
  bool track = finest == 0;
  // every update pass leaves e = 0; clear it anyway in case an earlier call
  // stopped between cycles
  cudaError_t ce0 = cudaMemsetAsync(H.fpool, 0, H.e_len * sizeof(float), H.s);
  if (ce0 != cudaSuccess) return cuda_fail(ce0, "cudaMemsetAsync(e)");
  bool resync = true, conv = false;
  int it;
  double res = 0.0;
  for (it = 1; it <= maxvcycles; it++) {
    // the tracked-residual cycle is captured when first needed (with
    // refinement levels every cycle starts from the FP64 residual)
    if (!resync && !gt &&
        (r = capture_graph(H, key(12), [&] { return mx_iteration(H, finest, minlevel, nsmooth, errortype, false); },
                           &gt)))
      return r;
    if ((r = replay(H, resync ? ga : gt))) return r;
    if (*H.h_nonfinite) return BSAMG_ERR_NONFINITE;
    double tracked = H.h_norm[0];
    res = tracked;
    resync = false;
    // Re-evaluate the residual in FP64 when the FP32-tracked one says the
    // iterate has converged, on the last cycle, and
    // once the tracked value has fallen 1e5 below the FP64 residual it
    // started from -- about where FP32 rounding of g stops being negligible.
    if (!track || tracked < tol || tracked < 1e-5 * r_sync || it == maxvcycles) {
      if ((r = replay(H, gv))) return r;
      if (*H.h_nonfinite) return BSAMG_ERR_NONFINITE;
      res = H.h_norm[0];
      r_sync = res;
      resync = true;  // the next cycle starts from this FP64 residual
    }
    if (residuals) residuals[it - 1] = res;
    if (resync && res < tol) {
      conv = true;
      break;
    }
  }
  if (ncycles) *ncycles = conv ? it : maxvcycles;
  // leave the state as the FP64 path leaves it: fresh ghosts, coarse levels
  // restricted from the finest (FillDown, afasroutines.f90:83)
  if (finest == 0)
    if ((r = enq_set_ghost(H, finest, 0))) return r;
  if (!conv && strict) return BSAMG_ERR_NOT_CONVERGED;
  return BSAMG_OK;
}

}  // namespace bsamg
