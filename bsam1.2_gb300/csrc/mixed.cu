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

#include <vector>

#include "launch.h"
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
__device__ __forceinline__ bool ghosted_cell(const int* n, int t, int& i, int& j, int& k) {
  i = t % n[0];
  int r = t / n[0];
  if (DIM == 2) {
    j = r;
    k = 0;
    return j < n[1];
  }
  j = r % n[1];
  k = r / n[1];
  return k < n[2];
}

template <int DIM, typename T>
__device__ __forceinline__ T ulap(const T* a, long long c, long long sy, long long sz) {
  if (DIM == 2) return a[c + 1] + a[c - 1] + a[c + sy] + a[c - sy] - T(4) * a[c];
  return a[c + 1] + a[c - 1] + a[c + sy] + a[c - sy] + a[c + sz] + a[c - sz] - T(6) * a[c];
}

// correction operator M(e) = N(qbar+e) - N(qbar) of the CH plugin
// (Operator2D/3D, CH/problem.f90:393-422, :638-669), cube difference
// written as e*(3 pb (pb + e) + e^2) to keep the small terms exact.
template <int DIM>
__device__ __forceinline__ void mop(const float* e, long long c, long long sy, long long sz, long long ps, float pb,
                                    float c0, float c1, float& m0, float& m1) {
  const float* e0 = e;
  const float* e1 = e + ps;
  float x = e0[c];
  m0 = x - c0 * ulap<DIM>(e1, c, sy, sz);
  m1 = e1[c] - x * (3.0f * pb * (pb + x) + x * x) + c1 * ulap<DIM>(e0, c, sy, sz);
}

// ---------------------------------------------------------------------------

// step 1: phib = (float)qbar_phi everywhere; on levels >= 0 the FP64
// residual g = f - N(qbar) (or the stored rf) as FP32.
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_mx_prep(const PatchDev* __restrict__ P, const double* __restrict__ pool,
                                                    float* __restrict__ fpool, const Blk* __restrict__ blk,
                                                    int mode /*0 phib only, 1 from rf, 2 recompute*/) {
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
__global__ void __launch_bounds__(kBlock) k_mx_relax(const PatchDev* __restrict__ P, float* __restrict__ fpool,
                                                     const Blk* __restrict__ blk, int ipass) {
  const Blk b = blk[blockIdx.x];
  const PatchDev& p = P[b.patch];
  int i, j, k;
  if (!color_cell<DIM>(p, b.start + threadIdx.x, ipass, i, j, k)) return;
  float* e0 = fpool + p.eq;
  float* e1 = e0 + p.sq;
  long long sy = p.qn[0], sz = (long long)p.qn[0] * p.qn[1];
  long long c = gofs<DIM>(p.qn, i, j, k);
  long long fc = iofs<DIM>(p.mx, i, j, k);
  float tmp1 = (float)p.c[0], tmp2 = (float)p.c[1], tmp3 = (float)p.c[2], a12 = (float)p.c[3];
  float pb = fpool[p.ephi + fc];
  float x = e0[c];
  float w = pb + x;
  float a21 = -3.0f * w * w - tmp3;
  float s1, s0;
  if (DIM == 2) {
    s1 = e1[c - 1] + e1[c + 1] + e1[c - sy] + e1[c + sy];
    s0 = e0[c + 1] + e0[c - 1] + e0[c + sy] + e0[c - sy];
  } else {
    s1 = e1[c - 1] + e1[c + 1] + e1[c - sy] + e1[c + sy] + e1[c - sz] + e1[c + sz];
    s0 = e0[c + 1] + e0[c - 1] + e0[c + sy] + e0[c - sy] + e0[c + sz] + e0[c - sz];
  }
  float b1 = fpool[p.eg + fc] + tmp1 * s1;
  float b2 = fpool[p.eg + p.sf + fc] - tmp2 * s0 - x * x * (3.0f * pb + 2.0f * x);
  float rdet = 1.0f / (1.0f - a12 * a21);
  e0[c] = (b1 - a12 * b2) * rdet;
  e1[c] = (b2 - a21 * b1) * rdet;
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
__global__ void __launch_bounds__(kBlock) k_mx_restrict(const PatchDev* __restrict__ P, float* __restrict__ fpool,
                                                        const Blk* __restrict__ blk, int nrvars) {
  const Blk b = blk[blockIdx.x];
  const PatchDev& p = P[b.patch];
  int ci, cj, ck;
  if (!interior_cell<DIM>(p.cmx, b.start + threadIdx.x, ci, cj, ck)) return;
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

// GetCoarseGhostPoints on e (ring of ec <- parent e) when corr == 0;
// CorrectFine step 1 (ec = parent e - ec over the whole ghosted ec) when
// corr == 1.
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_mx_coarse_ring(const PatchDev* __restrict__ P, float* __restrict__ fpool,
                                                           const Blk* __restrict__ blk, int nrvars, int corr) {
  const Blk b = blk[blockIdx.x];
  const PatchDev& p = P[b.patch];
  int i, j, k;
  if (!ghosted_cell<DIM>(p.cn, b.start + threadIdx.x, i, j, k)) return;
  if (!corr) {
    bool ring = i == 0 || i == p.cmx[0] + 1 || j == 0 || j == p.cmx[1] + 1 ||
                (DIM == 3 && (k == 0 || k == p.cmx[2] + 1));
    if (!ring) return;
  }
  const PatchDev& par = P[p.parent];
  long long src = gofs<DIM>(par.qn, p.mb[0] - 1 + i, p.mb[1] - 1 + j, DIM == 3 ? p.mb[2] - 1 + k : 0);
  long long dst = gofs<DIM>(p.cn, i, j, k);
  for (int v = 0; v < nrvars; v++) {
    float* ec = fpool + p.ecq + v * p.sc;
    float pv = fpool[par.eq + v * par.sq + src];
    ec[dst] = corr ? pv - ec[dst] : pv;
  }
}

// CoarseLoadingFunction on the correction: fine r = g - M(e) under each
// coarse cell; parent g(mb) = R(r) + M_c(ec) with the parent's base field.
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_mx_coarse_load(const PatchDev* __restrict__ P, float* __restrict__ fpool,
                                                           const Blk* __restrict__ blk) {
  const Blk b = blk[blockIdx.x];
  const PatchDev& p = P[b.patch];
  int ci, cj, ck;
  if (!interior_cell<DIM>(p.cmx, b.start + threadIdx.x, ci, cj, ck)) return;
  const PatchDev& par = P[p.parent];
  const float* e = fpool + p.eq;
  long long sy = p.qn[0], sz = (long long)p.qn[0] * p.qn[1];
  float c0 = (float)p.c[0], c1 = (float)p.c[1];
  float r0[8], r1[8];
  const int nk = DIM == 3 ? 2 : 1;
  // children in the reference's restriction order: (2i,2j,2k), (2i-1,2j,2k),
  // (2i,2j-1,2k), (2i-1,2j-1,2k), then the k-1 layer
  int n = 0;
  for (int dk = 0; dk < nk; dk++)
    for (int dj = 0; dj < 2; dj++)
      for (int di = 0; di < 2; di++, n++) {
        int i = 2 * ci - di, j = 2 * cj - dj, k = DIM == 3 ? 2 * ck - dk : 1;
        long long c = gofs<DIM>(p.qn, i, j, k);
        long long fc = iofs<DIM>(p.mx, i, j, k);
        float m0, m1;
        mop<DIM>(e, c, sy, sz, p.sq, fpool[p.ephi + fc], c0, c1, m0, m1);
        r0[n] = fpool[p.eg + fc] - m0;
        r1[n] = fpool[p.eg + p.sf + fc] - m1;
      }
  float R0 = 0.f, R1 = 0.f;
  for (int x = 0; x < 2 * 2 * nk; x++) {
    R0 += r0[x];
    R1 += r1[x];
  }
  R0 *= DIM == 2 ? 0.25f : 0.125f;
  R1 *= DIM == 2 ? 0.25f : 0.125f;
  const float* ec = fpool + p.ecq;
  long long csy = p.cn[0], csz = (long long)p.cn[0] * p.cn[1];
  long long cc = gofs<DIM>(p.cn, ci, cj, ck);
  long long pf = iofs<DIM>(par.mx, p.mb[0] + ci - 1, p.mb[1] + cj - 1, DIM == 3 ? p.mb[2] + ck - 1 : 1);
  float m0, m1;
  mop<DIM>(ec, cc, csy, csz, p.sc, fpool[par.ephi + pf], (float)par.c[0], (float)par.c[1], m0, m1);
  fpool[par.eg + pf] = R0 + m0;
  fpool[par.eg + par.sf + pf] = R1 + m1;
}

// CorrectFine step 2 on e: e(0:mx+1) += P(ec)
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_mx_prolong(const PatchDev* __restrict__ P, float* __restrict__ fpool,
                                                       const Blk* __restrict__ blk, int nrvars) {
  const Blk b = blk[blockIdx.x];
  const PatchDev& p = P[b.patch];
  int i, j, k;
  if (!ghosted_cell<DIM>(p.qn, b.start + threadIdx.x, i, j, k)) return;
  int ci = i >> 1, cj = j >> 1, ck = k >> 1;
  bool ei = (i & 1) == 0, ej = (j & 1) == 0, ek = (k & 1) == 0;
  long long dst = gofs<DIM>(p.qn, i, j, k);
  for (int v = 0; v < nrvars; v++) {
    const float* a = fpool + p.ecq + v * p.sc;
    auto bx = [&](int cy, int cz) {
      float lo = a[gofs<DIM>(p.cn, ci, cy, cz)], hi = a[gofs<DIM>(p.cn, ci + 1, cy, cz)];
      return ei ? 3.0f * lo + hi : lo + 3.0f * hi;
    };
    float add;
    if (DIM == 2) {
      float blo = bx(cj, 0), bhi = bx(cj + 1, 0);
      add = (ej ? 3.0f * blo + bhi : blo + 3.0f * bhi) * (1.0f / 16.0f);
    } else {
      auto cy = [&](int cz) {
        float blo = bx(cj, cz), bhi = bx(cj + 1, cz);
        return ej ? 3.0f * blo + bhi : blo + 3.0f * bhi;
      };
      float clo = cy(ck), chi = cy(ck + 1);
      add = (ek ? 3.0f * clo + chi : clo + 3.0f * chi) * (1.0f / 64.0f);
    }
    fpool[p.eq + v * p.sq + dst] += add;
  }
}

// step 3: qbar += e over the whole ghosted q of a level
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_mx_update(const PatchDev* __restrict__ P, double* __restrict__ pool,
                                                      const float* __restrict__ fpool, const Blk* __restrict__ blk,
                                                      int nrvars) {
  const Blk b = blk[blockIdx.x];
  const PatchDev& p = P[b.patch];
  int i, j, k;
  if (!ghosted_cell<DIM>(p.qn, b.start + threadIdx.x, i, j, k)) return;
  long long c = gofs<DIM>(p.qn, i, j, k);
  for (int v = 0; v < nrvars; v++) pool[p.oq + v * p.sq + c] += (double)fpool[p.eq + v * p.sq + c];
}

// FP64 residual rf = f - N(q) of the finest level and per-block sums of rf^2
// (ErrorAFAS, afasroutines.f90:113-233).  Same arithmetic as the plain
// path's norm kernel, but this translation unit lets the compiler fuse
// multiply-adds, which cuts FP64 pipe work by about a third; the mixed path
// needs the true residual to ~1e-15 relative, not bit-identical rounding.
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_mx_norm(const PatchDev* __restrict__ P, double* __restrict__ pool,
                                                    const Blk* __restrict__ blk, double* __restrict__ partial) {
  __shared__ double red[2][kBlock / 32];
  const Blk b = blk[blockIdx.x];
  const PatchDev& p = P[b.patch];
  int i, j, k;
  double s0 = 0.0, s1 = 0.0;
  if (interior_cell<DIM>(p.mx, b.start + threadIdx.x, i, j, k)) {
    const double* q0 = pool + p.oq;
    const double* q1 = q0 + p.sq;
    long long sy = p.qn[0], sz = (long long)p.qn[0] * p.qn[1];
    long long c = gofs<DIM>(p.qn, i, j, k);
    long long fc = iofs<DIM>(p.mx, i, j, k);
    double phi = q0[c];
    double o0 = phi - p.c[0] * ulap<DIM>(q1, c, sy, sz);
    double o1 = q1[c] - phi * phi * phi + p.c[1] * ulap<DIM>(q0, c, sy, sz);
    double e0 = pool[p.of + fc] - o0;
    double e1 = pool[p.of + p.sf + fc] - o1;
    pool[p.orf + fc] = e0;
    pool[p.orf + p.sf + fc] = e1;
    s0 = e0 * e0;
    s1 = e1 * e1;
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
    for (int n = 0; n < kBlock / 32; n++) {
      t0 += red[0][n];
      t1 += red[1][n];
    }
    partial[2 * blockIdx.x] = t0;
    partial[2 * blockIdx.x + 1] = t1;
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
      case kGBC: val = ((g.mask >> v) & 1) ? -sq[g.s0] : sq[g.s0]; break;  // 2 - q -> -e
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

int mx_set_ghost(Hier& H, int level, int ipass) {
  GhostProg& g = H.L(level).gp[ipass];
  int nst = (int)g.stage_off.size() - 1;
  if (nst <= 0) return BSAMG_OK;
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

int mx_level_relax(Hier& H, int level, int nsmooth) {
  LevelT& L = H.L(level);
  for (int pass = 1; pass <= nsmooth; pass++)
    for (int rb = 1; rb <= 2; rb++) {
      MX_LAUNCH(H, kKindColor, k_mx_relax, H.dP, H.fpool, L.d_blk[kKindColor], rb);
      int r = mx_set_ghost(H, level, rb);
      if (r) return r;
    }
  return BSAMG_OK;
}

int mx_vcycle(Hier& H, int level, int minlevel, int nsmooth) {
  int r = mx_level_relax(H, level, nsmooth);
  if (r) return r;
  if (level > minlevel) {
    LevelT& L = H.L(level);
    MX_LAUNCH(H, kKindCoarse, k_mx_restrict, H.dP, H.fpool, L.d_blk[kKindCoarse], H.nrvars);
    if ((r = mx_set_ghost(H, level - 1, 0))) return r;
    MX_LAUNCH(H, kKindCGhost, k_mx_coarse_ring, H.dP, H.fpool, L.d_blk[kKindCGhost], H.nrvars, 0);
    MX_LAUNCH(H, kKindCoarse, k_mx_coarse_load, H.dP, H.fpool, L.d_blk[kKindCoarse]);
    if ((r = mx_vcycle(H, level - 1, minlevel, nsmooth))) return r;
    MX_LAUNCH(H, kKindCGhost, k_mx_coarse_ring, H.dP, H.fpool, L.d_blk[kKindCGhost], H.nrvars, 1);
    MX_LAUNCH(H, kKindFGhost, k_mx_prolong, H.dP, H.fpool, L.d_blk[kKindFGhost], H.nrvars);
    if ((r = mx_set_ghost(H, level, 0))) return r;
    if ((r = mx_level_relax(H, level, nsmooth))) return r;
  }
  return BSAMG_OK;
}

std::vector<long long> layout(const Hier& H, size_t* total, size_t* e_len) {
  // region order: all e (sq*V), all ec (sc*V), all g (sf*V), all phib (sf);
  // e is one contiguous region so one memset clears every correction
  size_t np = H.patches.size();
  std::vector<long long> off(4 * np);
  long long o = 0;
  auto al = [](long long x) { return (x + 63) & ~63LL; };
  for (size_t p = 0; p < np; p++) { off[4 * p] = o; o = al(o + H.patches[p].sq * H.nrvars); }
  *e_len = (size_t)o;
  for (size_t p = 0; p < np; p++) { off[4 * p + 1] = o; o = al(o + H.patches[p].sc * H.nrvars); }
  for (size_t p = 0; p < np; p++) { off[4 * p + 2] = o; o = al(o + H.patches[p].sf * H.nrvars); }
  for (size_t p = 0; p < np; p++) { off[4 * p + 3] = o; o = al(o + H.patches[p].sf); }
  *total = (size_t)o;
  return off;
}

}  // namespace

size_t mixed_pool_bytes(const Hier& H) {
  if (H.problem != kCH) return 0;
  size_t n, ne;
  layout(H, &n, &ne);
  return n * sizeof(float);
}

int mixed_alloc(Hier& H) {
  if (H.problem != kCH) return BSAMG_OK;
  size_t n, ne;
  std::vector<long long> off = layout(H, &n, &ne);
  H.e_len = ne;
  for (size_t p = 0; p < H.patches.size(); p++) {
    HostPatch& P = H.patches[p];
    P.e_oq = off[4 * p];
    P.e_oqc = off[4 * p + 1];
    P.e_of = off[4 * p + 2];
    P.e_ophi = off[4 * p + 3];
  }
  H.fpool_elems = n;
  cudaError_t e = cudaMalloc(&H.fpool, n * sizeof(float));
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(fpool)");
  e = cudaMemsetAsync(H.fpool, 0, n * sizeof(float), H.s);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(fpool)");
  return BSAMG_OK;
}

void mixed_free(Hier& H) {
  if (H.fpool) cudaFree(H.fpool);
  H.fpool = nullptr;
}

int mx_norm(Hier& H, int level, int errortype) {
  LevelT& L = H.L(level);
  MX_LAUNCH(H, kKindInterior, k_mx_norm, H.dP, H.pool, L.d_blk[kKindInterior], H.d_partial);
  return after_launch(H, launch_norm_finish(H.s, H.d_partial, L.nblk[kKindInterior], H.nrvars, L.count, errortype,
                                            H.d_norm, H.d_nonfinite));
}

int mixed_enq_relax(Hier& H, int level, int ipass) {
  if (H.problem != kCH || !H.fpool) return BSAMG_ERR_UNSUPPORTED;
  LevelT& L = H.L(level);
  MX_LAUNCH(H, kKindColor, k_mx_relax, H.dP, H.fpool, L.d_blk[kKindColor], ipass);
  return BSAMG_OK;
}

int mixed_prepare(Hier& H, int finest, int minlevel) {
  if (H.problem != kCH || !H.fpool) return BSAMG_ERR_UNSUPPORTED;
  (void)minlevel;
  // the first outer iteration needs the FP64 residual of the finest level
  return mx_norm(H, finest, 1);
}

int mixed_enq_iteration(Hier& H, int finest, int minlevel, int nsmooth, int errortype) {
  if (H.problem != kCH || !H.fpool) return BSAMG_ERR_UNSUPPORTED;
  // 1. FP64 residuals -> g, phib, e = 0
  cudaError_t ce = cudaMemsetAsync(H.fpool, 0, H.e_len * sizeof(float), H.s);
  if (ce != cudaSuccess) return cuda_fail(ce, "cudaMemsetAsync(e)");
  for (int level = finest; level >= minlevel; level--) {
    LevelT& L = H.L(level);
    int mode = level < 0 ? 0 : (level == finest ? 1 : 2);
    MX_LAUNCH(H, kKindInterior, k_mx_prep, H.dP, H.pool, H.fpool, L.d_blk[kKindInterior], mode);
  }
  // 2. FP32 correction V-cycle
  int r = mx_vcycle(H, finest, minlevel, nsmooth);
  if (r) return r;
  // 3. FP64 update, FillDown(q), norm (stores rf for the next iteration)
  for (int level = finest; level >= 0; level--) {
    LevelT& L = H.L(level);
    MX_LAUNCH(H, kKindFGhost, k_mx_update, H.dP, H.pool, H.fpool, L.d_blk[kKindFGhost], H.nrvars);
  }
  if ((r = enq_fill_down(H, 2, finest, minlevel))) return r;
  // refinement levels: ghosts from the updated FP64 state (coarse-fine
  // interpolation reads the parent values FillDown just restricted)
  for (int level = 1; level <= finest; level++)
    if ((r = enq_set_ghost(H, level, 0))) return r;
  if ((r = mx_norm(H, finest, errortype))) return r;
  ce = cudaMemcpyAsync(H.h_norm, H.d_norm, 2 * sizeof(double), cudaMemcpyDeviceToHost, H.s);
  if (ce != cudaSuccess) return cuda_fail(ce, "cudaMemcpyAsync(norm)");
  ce = cudaMemcpyAsync(H.h_nonfinite, H.d_nonfinite, sizeof(int), cudaMemcpyDeviceToHost, H.s);
  if (ce != cudaSuccess) return cuda_fail(ce, "cudaMemcpyAsync(nonfinite)");
  return BSAMG_OK;
}

}  // namespace bsamg
