// Device side of the after-step statistics and of the uniform-mesh output.
//
// Built with --fmad=false like the other FP64 kernels: the uniform-mesh
// prolongation repeats the reference's operation order exactly, so the
// composite it writes is bit-identical to the host restatement.
//
// Statistics (AfterStepStatistics, LIBRARY/bsamroutines.f90:918-963, with
// the plugins' AfterStep2D/3D, PROBLEM/CH/problem.f90:149-215): one
// deterministic reduction over the fine interior cells of levels 0..finest
// and, with a minus sign, the parent cells under every level > 0 patch.  The
// per-cell terms are the reference's (h^d q1; h^2 (Ff(c) + eps^2/h^2/4 *
// squared differences) for the CH 2D energy); the sum order is a fixed tree,
// not the reference's sequential SUM, so results agree to rounding.
//
// Uniform mesh (WriteUniformMeshQ, LIBRARY/bsaminputoutput.f90:446-572):
// each level of the composite is the mass-corrected bilinear/trilinear
// prolongation (BiLinProlongationP1MC / TriLinProlongationP1MC,
// LIBRARY/gridutilities.f90) of the level below over the whole domain, ghost
// layers included, with the level's patches copied over it in visiting
// order.
#include <cuda_runtime.h>

#include "internal.h"
#include "launch.h"

namespace bsamg {
namespace {

constexpr int kStatThreads = 256;

template <int DIM>
__device__ __forceinline__ long long qofs(const int* n, int i, int j, int k) {
  if (DIM == 2) return (long long)j * n[0] + i;
  return ((long long)k * n[1] + j) * n[0] + i;
}

__device__ __forceinline__ double ff_energy(double c) {  // Ff, CH/problem.f90:901-915
  double c2 = c * c;
  return c2 * (c2 - 2.0) / 4.0;
}

// fixed-order tree sum of two values over the block; thread 0 gets the result
__device__ void block_sum2(double& a, double& b) {
  __shared__ double sa[kStatThreads], sb[kStatThreads];
  sa[threadIdx.x] = a;
  sb[threadIdx.x] = b;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      sa[threadIdx.x] = sa[threadIdx.x] + sa[threadIdx.x + s];
      sb[threadIdx.x] = sb[threadIdx.x] + sb[threadIdx.x + s];
    }
    __syncthreads();
  }
  a = sa[0];
  b = sb[0];
}

// One block of a level's interior (COARSE = false: the patch's own cells)
// or coarse list (COARSE = true: the parent cells under the patch, counted
// with a minus sign).  partial[2*(pofs + block)] = (mass, energy).
template <int DIM, bool COARSE>
__global__ void __launch_bounds__(kStatThreads)
    k_stats(const PatchDev* __restrict__ P, const double* __restrict__ pool, const Blk* __restrict__ blk,
            int mass, int energy, double eps2, double* __restrict__ partial, int pofs) {
  const Blk b = blk[blockIdx.x];
  const PatchDev& p = P[b.patch];
  const int* m = COARSE ? p.cmx : p.mx;
  int t = b.start + threadIdx.x;
  int i = t % m[0] + 1, r = t / m[0], j, k;
  bool ok;
  if (DIM == 2) {
    j = r + 1;
    k = 0;
    ok = j <= m[1];
  } else {
    j = r % m[1] + 1;
    k = r / m[1] + 1;
    ok = k <= m[2];
  }
  double ms = 0.0, en = 0.0;
  if (ok) {
    const PatchDev& s = COARSE ? P[p.parent] : p;
    if (COARSE) {
      i += p.mb[0] - 1;
      j += p.mb[1] - 1;
      if (DIM == 3) k += p.mb[2] - 1;
    }
    const double* q = pool + s.oq;  // variable 1
    long long c = qofs<DIM>(s.qn, i, j, k);
    double hh = COARSE ? p.h * 2.0 : p.h;
    double hd = DIM == 2 ? hh * hh : hh * hh * hh;
    double v = q[c];
    if (mass) ms = hd * v;
    if (DIM == 2 && energy) {
      long long sy = s.qn[0];
      double a1 = q[c + 1] - v, b1 = v - q[c - 1], c1 = q[c + sy] - v, d1 = v - q[c - sy];
      double h2 = hh * hh;
      double tmp = eps2 / h2 / 4.0;
      en = h2 * (ff_energy(v) + tmp * (((a1 * a1 + b1 * b1) + c1 * c1) + d1 * d1));
    }
    if (COARSE) {
      ms = -ms;
      en = -en;
    }
  }
  block_sum2(ms, en);
  if (threadIdx.x == 0) {
    partial[2 * (long long)(pofs + blockIdx.x)] = ms;
    partial[2 * (long long)(pofs + blockIdx.x) + 1] = en;
  }
}

// out[0..1] = the fixed-order sum of n partial pairs (one block)
__global__ void __launch_bounds__(kStatThreads) k_stats_finish(const double* __restrict__ partial, int n,
                                                               double* __restrict__ out) {
  double a = 0.0, b = 0.0;
  for (int x = threadIdx.x; x < n; x += blockDim.x) {
    a = a + partial[2 * (long long)x];
    b = b + partial[2 * (long long)x + 1];
  }
  block_sum2(a, b);
  if (threadIdx.x == 0) {
    out[0] = a;
    out[1] = b;
  }
}

// One variable of the mass-corrected prolongation of a whole uniform level:
// A is the coarse (n+2)^d block, F the fine (2n+2)^d block.  Every fine
// value is formed exactly as the host restatement forms it: the x stage
// 3a+b / a+3b, the y stage (and z stage in 3D), the division by 16 (64),
// then, inside the domain, the correction A(I,J[,K]) - mean of the coarse
// cell's children added to each child.
template <int DIM>
__global__ void __launch_bounds__(256) k_uni_prolong(const double* __restrict__ A, double* __restrict__ F, int n0,
                                                     int n1, int n2, long long total) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total) return;
  const int cn0 = n0 + 2, cn1 = n1 + 2;
  const int fn0 = 2 * n0 + 2, fn1 = 2 * n1 + 2;
  int i = (int)(t % fn0);
  long long r = t / fn0;
  int j = (int)(r % fn1);
  int k = DIM == 3 ? (int)(r / fn1) : 0;
  auto a = [&](int I, int J, int K) { return A[((long long)K * cn1 + J) * cn0 + I]; };
  // x stage at fine column x of coarse row (J, K)
  auto bx = [&](int x, int J, int K) {
    int I = x >> 1;
    return (x & 1) ? a(I, J, K) + 3.0 * a(I + 1, J, K) : 3.0 * a(I, J, K) + a(I + 1, J, K);
  };
  // uncorrected fine value at (x, y[, z])
  auto fine = [&](int x, int y, int z) {
    int J = y >> 1;
    if (DIM == 2) {
      return (y & 1) ? (bx(x, J, 0) + 3.0 * bx(x, J + 1, 0)) / 16.0 : (3.0 * bx(x, J, 0) + bx(x, J + 1, 0)) / 16.0;
    }
    auto cy = [&](int K) {
      return (y & 1) ? bx(x, J, K) + 3.0 * bx(x, J + 1, K) : 3.0 * bx(x, J, K) + bx(x, J + 1, K);
    };
    int K = z >> 1;
    return (z & 1) ? (cy(K) + 3.0 * cy(K + 1)) / 64.0 : (3.0 * cy(K) + cy(K + 1)) / 64.0;
  };
  double v = fine(i, j, k);
  bool inside = i >= 1 && i <= 2 * n0 && j >= 1 && j <= 2 * n1 && (DIM == 2 || (k >= 1 && k <= 2 * n2));
  if (inside) {
    int I = (i + 1) >> 1, J = (j + 1) >> 1, K = DIM == 3 ? (k + 1) >> 1 : 0;
    double cor;
    if (DIM == 2) {
      cor = a(I, J, 0) -
            0.25 * (((fine(2 * I, 2 * J, 0) + fine(2 * I - 1, 2 * J, 0)) + fine(2 * I, 2 * J - 1, 0)) +
                    fine(2 * I - 1, 2 * J - 1, 0));
    } else {
      cor = a(I, J, K) -
            0.125 * (((((((fine(2 * I, 2 * J, 2 * K) + fine(2 * I - 1, 2 * J, 2 * K)) + fine(2 * I, 2 * J - 1, 2 * K)) +
                        fine(2 * I - 1, 2 * J - 1, 2 * K)) +
                       fine(2 * I, 2 * J, 2 * K - 1)) +
                      fine(2 * I - 1, 2 * J, 2 * K - 1)) +
                     fine(2 * I, 2 * J - 1, 2 * K - 1)) +
                     fine(2 * I - 1, 2 * J - 1, 2 * K - 1));
    }
    v = v + cor;
  }
  F[t] = v;
}

// CopyPatchToUniformGrid (bsaminputoutput.f90:543-572): q(0:mx+1) of one
// patch (all variables) into the uniform block U ((un0 x un1 x un2) per
// variable, planes of uplane) at global cell mglobal - 1.  oq is the offset
// of the patch's cell (0,0,0), qn its ghosted extents (any mbc).
template <int DIM>
__global__ void __launch_bounds__(256) k_uni_scatter(const double* __restrict__ pool, long long oq, long long sq,
                                                     int qn0, int qn1, int e0, int e1, int e2, int g0, int g1, int g2,
                                                     double* __restrict__ U, int un0, int un1, long long uplane,
                                                     int nv) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long cells = (long long)e0 * e1 * e2;
  if (t >= cells * nv) return;
  int v = (int)(t / cells);
  long long c = t % cells;
  int i = (int)(c % e0);
  long long r = c / e0;
  int j = (int)(r % e1);
  int k = (int)(r / e1);
  long long u = ((long long)(DIM == 3 ? g2 - 1 + k : 0) * un1 + (g1 - 1 + j)) * un0 + (g0 - 1 + i);
  long long src = ((long long)(DIM == 3 ? k : 0) * qn1 + j) * qn0 + i;
  U[v * uplane + u] = pool[oq + v * sq + src];
}

// splitmix64 of the seeded inputs: U(-1,1) from splitmix64(seed ^ (g * golden))
__device__ __forceinline__ double seeded_pm1(unsigned long long seed, unsigned long long g) {
  const unsigned long long gold = 0x9E3779B97F4A7C15ull;
  unsigned long long z = seed ^ (g * gold);
  z = z + gold;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z = z ^ (z >> 31);
  return 2.0 * ((double)(z >> 11) * (1.0 / 9007199254740992.0)) - 1.0;
}

// The seeded spinodal start of one CH patch, in the order the host generator
// evaluates it: phi = mean + amp*U on the cell's index within the patch
// (i fastest), mu = ((phi*phi*phi) - phi) - eps2 * lap, lap =
// ((-2 d) phi + (phi[i-1] + phi[i+1]) + ...) / (h*h) with the neighbours
// wrapped over the patch; ghost layers (mbc = gs + 1 of them) zero.  q is
// the array's start, t runs over its ghosted cells.
template <int DIM>
__global__ void __launch_bounds__(256) k_seed_spinodal(double* __restrict__ q, long long sq, int m0, int m1, int m2,
                                                       int gs, unsigned long long seed, double mean, double amp,
                                                       double eps2, double hh) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int n0 = m0 + 2 + 2 * gs, n1 = m1 + 2 + 2 * gs, n2 = DIM == 3 ? m2 + 2 + 2 * gs : 1;
  if (t >= (long long)n0 * n1 * n2) return;
  int i = (int)(t % n0) - gs;
  long long r = t / n0;
  int j = (int)(r % n1) - gs;
  int k = DIM == 3 ? (int)(r / n1) - gs : 1;
  bool ghost = i < 1 || i > m0 || j < 1 || j > m1 || (DIM == 3 && (k < 1 || k > m2));
  if (ghost) {
    q[t] = 0.0;
    q[sq + t] = 0.0;
    return;
  }
  auto phi = [&](int a, int b, int c) {  // interior cell (a, b, c), 0-based, wrapped
    a = (a + m0) % m0;
    b = (b + m1) % m1;
    c = DIM == 3 ? (c + m2) % m2 : 0;
    unsigned long long g = ((unsigned long long)c * m1 + b) * m0 + a;
    return mean + amp * seeded_pm1(seed, g);
  };
  int a = i - 1, b = j - 1, c = DIM == 3 ? k - 1 : 0;
  double p = phi(a, b, c);
  double lap = (-2.0 * DIM) * p;
  lap = (lap + phi(a - 1, b, c)) + phi(a + 1, b, c);
  lap = (lap + phi(a, b - 1, c)) + phi(a, b + 1, c);
  if (DIM == 3) lap = (lap + phi(a, b, c - 1)) + phi(a, b, c + 1);
  lap = lap / (hh * hh);
  q[t] = p;
  q[sq + t] = ((p * p * p) - p) - eps2 * lap;
}

}  // namespace

int launch_seed_spinodal(cudaStream_t s, int ndims, int mbc, double* q, long long sq, const int mx[3],
                         unsigned long long seed, double mean, double amp, double eps2, double h) {
  long long n = (long long)(mx[0] + 2 * mbc) * (mx[1] + 2 * mbc) * (ndims == 3 ? mx[2] + 2 * mbc : 1);
  unsigned grid = (unsigned)((n + 255) / 256);
  int gs = mbc - 1;
  if (ndims == 2) k_seed_spinodal<2><<<grid, 256, 0, s>>>(q, sq, mx[0], mx[1], 1, gs, seed, mean, amp, eps2, h);
  else k_seed_spinodal<3><<<grid, 256, 0, s>>>(q, sq, mx[0], mx[1], mx[2], gs, seed, mean, amp, eps2, h);
  return 1;
}

int launch_stats(const LaunchCtx& c, const Blk* blk, int nblk, bool coarse, int mass, int energy, double* partial,
                 int pofs) {
  if (nblk <= 0) return 0;
  double eps2 = c.pp.eps2;
  if (c.ndims == 2) {
    if (coarse) k_stats<2, true><<<nblk, kStatThreads, 0, c.s>>>(c.P, c.pool, blk, mass, energy, eps2, partial, pofs);
    else k_stats<2, false><<<nblk, kStatThreads, 0, c.s>>>(c.P, c.pool, blk, mass, energy, eps2, partial, pofs);
  } else {
    if (coarse) k_stats<3, true><<<nblk, kStatThreads, 0, c.s>>>(c.P, c.pool, blk, mass, energy, eps2, partial, pofs);
    else k_stats<3, false><<<nblk, kStatThreads, 0, c.s>>>(c.P, c.pool, blk, mass, energy, eps2, partial, pofs);
  }
  return 1;
}

int launch_stats_finish(cudaStream_t s, const double* partial, int n, double* out) {
  k_stats_finish<<<1, kStatThreads, 0, s>>>(partial, n, out);
  return 1;
}

int launch_uniform_prolong(cudaStream_t s, int ndims, const double* A, double* F, const int n[3]) {
  long long total = (long long)(2 * n[0] + 2) * (2 * n[1] + 2) * (ndims == 3 ? 2 * n[2] + 2 : 1);
  unsigned grid = (unsigned)((total + 255) / 256);
  if (ndims == 2) k_uni_prolong<2><<<grid, 256, 0, s>>>(A, F, n[0], n[1], 1, total);
  else k_uni_prolong<3><<<grid, 256, 0, s>>>(A, F, n[0], n[1], n[2], total);
  return 1;
}

int launch_uniform_scatter(cudaStream_t s, int ndims, const double* pool, long long oq, long long sq, const int qn[3],
                           const int mx[3], const int g[3], double* U, const int un[3], int nv) {
  int e[3] = {mx[0] + 2, mx[1] + 2, ndims == 3 ? mx[2] + 2 : 1};
  long long cells = (long long)e[0] * e[1] * e[2] * nv;
  unsigned grid = (unsigned)((cells + 255) / 256);
  long long uplane = (long long)un[0] * un[1] * un[2];
  if (ndims == 2)
    k_uni_scatter<2><<<grid, 256, 0, s>>>(pool, oq, sq, qn[0], qn[1], e[0], e[1], e[2], g[0], g[1], g[2], U, un[0],
                                          un[1], uplane, nv);
  else
    k_uni_scatter<3><<<grid, 256, 0, s>>>(pool, oq, sq, qn[0], qn[1], e[0], e[1], e[2], g[0], g[1], g[2], U, un[0],
                                          un[1], uplane, nv);
  return 1;
}

}  // namespace bsamg
