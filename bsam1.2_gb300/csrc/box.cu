// Mixed-precision MultigridIterations on periodic boxes.
//
// Applies when every level of the hierarchy is one fully periodic patch with
// even extents that covers its parent (a uniform periodic grid and its
// below-root levels, RootInit/InitSeed, bsamroutines.f90:226-510).  The
// algorithm is the one of mixed.cu -- an FP32 FAS V-cycle on the correction
// equation M(e) = N(qbar + e) - N(qbar) = g inside an outer loop that updates
// qbar and confirms convergence on the true residual f - N(qbar) -- with a
// data layout and precision split chosen for GB300:
//
//  * No ghost cells and no work lists.  Neighbours wrap around the box, and
//    every kernel derives its cell from a 3D grid, so a thread's first loads
//    are its data (no dependent table lookups).
//  * Colour-split FP32 arrays (BoxLev).  A red half-sweep reads whole
//    sectors of black values and writes whole sectors of red ones, instead
//    of touching every sector of an interleaved array for half its bytes.
//  * The FP64 iterate is held for the whole solve as a pair of floats
//    (hi + lo, about 48 significant bits).  qbar += e is a TwoSum, and the
//    residual f - N(qbar) is evaluated in double-float arithmetic, all on the
//    FP32 pipe; GB300's FP64 rate is 1/64 of its FP32 rate.  The rounding
//    error of the double-float residual is about 2^-47 times the largest
//    term (|c0 ulap(mu)|, |phi^3| ~ 1-100 here), i.e. ~1e-12, four orders
//    below the 1e-8..1e-9 tolerances the residual is tested against.  FP64 is
//    used only to split q at the start (integer bit operations, exact) and
//    to write it back at the end (one FP64 add per value).
//  * The tracked residual update g <- g - M(e) and qbar += e are one pass,
//    and e is never cleared: the first two half-sweeps of a cycle on the
//    finest level treat the previous cycle's e as zero.
//
// Plugin: CH (CH/problem.f90), whose source is f = (phi_old, -phi_old)
// (Source2D/3D, :425-450, :672-695) and whose operator is
// N(q) = (phi - dt/h^2 ULap(mu), mu - phi^3 + eps^2/h^2 ULap(phi))
// (Operator2D/3D, :393-422, :638-669).
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstddef>
#include <functional>

#include "box.h"
#include "launch.h"

namespace bsamg {

namespace {

// colour of 0-based cell (x, y, z): parity of the 1-based i + j (+ k)
template <int DIM>
__device__ __forceinline__ int colour(int x, int y, int z) {
  return DIM == 3 ? (x + y + z + 1) & 1 : (x + y) & 1;
}

// A cell and its six neighbours as 32-bit indices into a colour-split array
// of one variable, the colour offset included: own = c*half + row*hh + x/2,
// the neighbours in the other colour's half.  A kernel forms one base
// pointer per array and variable (fp + offset + v*2*half), the same for all
// its threads, so that a load costs one address instruction.
template <int DIM>
struct Loc {
  int c;
  unsigned own, xm, xp, ym, yp, zm, zp;
  __device__ __forceinline__ Loc(const BoxLev& L, int x, int y, int z) {
    c = colour<DIM>(x, y, z);
    unsigned hh = (unsigned)L.hh, n1 = (unsigned)L.n[1], half = (unsigned)L.half;
    unsigned h = (unsigned)x >> 1, b = (unsigned)x & 1u;
    unsigned r = (unsigned)z * n1 + (unsigned)y;
    unsigned on = c ? 0u : half;  // start of the other colour
    own = (c ? half : 0u) + r * hh + h;
    unsigned row = on + r * hh;
    xm = row + (b ? h : (h ? h - 1 : hh - 1));
    xp = row + (b ? (h + 1 < hh ? h + 1 : 0u) : h);
    unsigned rz = r - (unsigned)y;  // z * n1
    ym = on + (rz + (y ? (unsigned)y - 1 : n1 - 1)) * hh + h;
    yp = on + (rz + ((unsigned)y + 1 < n1 ? (unsigned)y + 1 : 0u)) * hh + h;
    if (DIM == 3) {
      unsigned n2 = (unsigned)L.n[2];
      zm = on + ((z ? (unsigned)z - 1 : n2 - 1) * n1 + (unsigned)y) * hh + h;
      zp = on + (((unsigned)z + 1 < n2 ? (unsigned)z + 1 : 0u) * n1 + (unsigned)y) * hh + h;
    } else {
      zm = zp = 0;
    }
  }
};

template <int DIM, typename T = float>
__device__ __forceinline__ T nsum(const float* a, const Loc<DIM>& l) {
  T s = T(a[l.xm]) + T(a[l.xp]) + T(a[l.ym]) + T(a[l.yp]);
  if (DIM == 3) s += T(a[l.zm]) + T(a[l.zp]);
  return s;
}

// bases of variables 0 and 1 of a two-variable colour-split array
struct V2 {
  float* v0;
  float* v1;
};
__device__ __forceinline__ V2 var2(float* fp, long long off, long long half) {
  return {fp + off, fp + off + 2 * half};
}

// correction operator M(e) at a cell (see mixed.cu, mopn)
template <int DIM>
__device__ __forceinline__ void mop(V2 E, const BoxLev& L, const Loc<DIM>& l, float pb, float& m0, float& m1) {
  float x = E.v0[l.own], y = E.v1[l.own];
  const float k = DIM == 2 ? 4.0f : 6.0f;
  m0 = x - L.c0 * (nsum<DIM>(E.v1, l) - k * y);
  m1 = y - x * (3.0f * pb * (pb + x) + x * x) + L.c1 * (nsum<DIM>(E.v0, l) - k * x);
}

// the undivided Laplacian as a sum of neighbour differences: for a smooth
// correction each difference of two close values is exact (Sterbenz), so the
// rounding error is relative to the Laplacian, not to the values (the sum of
// neighbours minus k times the centre cancels and keeps ~1e-7 of |e|)
template <int DIM>
__device__ __forceinline__ float ndiff(const float* a, const Loc<DIM>& l, float c) {
  float s = ((a[l.xm] - c) + (a[l.xp] - c)) + ((a[l.ym] - c) + (a[l.yp] - c));
  if (DIM == 3) s += (a[l.zm] - c) + (a[l.zp] - c);
  return s;
}

// M(e) for the tracked residual g <- g - M(e): its rounding accumulates into
// the right-hand side of every later cycle (the smoother's and the coarse
// correction's only slow convergence down), so the Laplacians are evaluated
// in the difference form.  With c0 = dt/h^2 ~ 33 at 256^3 the summed form
// left a floor near 1e-5 |e| in g: from the 12th step on the last cycle of a
// step gained 5x instead of 12x, and later steps needed a sixth cycle.
template <int DIM>
__device__ __forceinline__ void mop_track(V2 E, const BoxLev& L, const Loc<DIM>& l, float pb, float& m0, float& m1) {
  float x = E.v0[l.own], y = E.v1[l.own];
  m0 = x - L.c0 * ndiff<DIM>(E.v1, l, y);
  m1 = y - x * (3.0f * pb * (pb + x) + x * x) + L.c1 * ndiff<DIM>(E.v0, l, x);
}

// ---------------------------------------------------------------------------
// double-float arithmetic (value = h + l, |l| <= ulp(h)/2 after
// normalisation): Dekker/Knuth error-free transformations

struct DF {
  float h, l;
};
__device__ __forceinline__ DF two_sum(float a, float b) {
  float s = a + b;
  float bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ DF fast_two_sum(float a, float b) {
  float s = a + b;
  return {s, b - (s - a)};
}
__device__ __forceinline__ DF df_add(DF x, DF y) {
  DF s = two_sum(x.h, y.h);
  return fast_two_sum(s.h, s.l + (x.l + y.l));
}
__device__ __forceinline__ DF df_neg(DF x) { return {-x.h, -x.l}; }
__device__ __forceinline__ DF df_mul(DF x, DF y) {
  float p = x.h * y.h;
  float e = fmaf(x.h, y.h, -p);
  e = fmaf(x.h, y.l, e);
  e = fmaf(x.l, y.h, e);
  return fast_two_sum(p, e);
}
// undivided Laplacian sum(neighbours) - k*centre of double-float values
template <int DIM>
__device__ __forceinline__ DF df_lap(const DF* nb, DF c) {
  float sh = nb[0].h, el = nb[0].l;
  for (int m = 1; m < 2 * DIM; m++) {
    DF t = two_sum(sh, nb[m].h);
    sh = t.h;
    el += t.l + nb[m].l;
  }
  const float k = DIM == 2 ? 4.0f : 6.0f;
  float p = k * c.h;
  float pe = fmaf(k, c.h, -p);  // k*c.h = p + pe exactly
  DF t = two_sum(sh, -p);
  el += t.l - pe - k * c.l;
  return fast_two_sum(t.h, el);
}

// Split a double into hi + lo floats with integer operations only (no FP64
// instructions).  hi keeps the leading 24 significant bits (truncated), lo
// the next 29 rounded to 24, so hi + lo carries 48 of the 53 bits.  Values
// whose magnitude is outside [2^-70, 2^120] (zero, denormals, infinities,
// NaN, extremes) take the conversion instructions instead.
__device__ __forceinline__ DF split64(double x) {
  unsigned long long b = (unsigned long long)__double_as_longlong(x);
  unsigned int top = (unsigned int)(b >> 32);
  int e = (int)((top >> 20) & 0x7FFu) - 1023;
  if (e >= -70 && e <= 120) {
    unsigned int s = top & 0x80000000u;
    float hi = __uint_as_float(s | ((unsigned int)(e + 127) << 23) | ((unsigned int)(b >> 29) & 0x7FFFFFu));
    float rf = __uint2float_rn((unsigned int)b & 0x1FFFFFFFu);
    float lo = rf * __uint_as_float((unsigned int)(e - 52 + 127) << 23);
    return {hi, s ? -lo : lo};
  }
  if ((b << 1) == 0) return {__uint_as_float(top & 0x80000000u), 0.0f};
  float hi = (float)x;
  return {hi, (float)(x - (double)hi)};
}
// float -> double by bit operations for normal floats and zeros
__device__ __forceinline__ double f2d(float f) {
  unsigned int u = __float_as_uint(f);
  unsigned int ex = (u >> 23) & 0xFFu;
  if (ex != 0 && ex != 0xFFu)
    return __longlong_as_double((long long)(((unsigned long long)(u & 0x80000000u) << 32) |
                                            ((unsigned long long)(ex + 896u) << 52) |
                                            ((unsigned long long)(u & 0x7FFFFFu) << 29)));
  if ((u << 1) == 0) return __longlong_as_double((long long)((unsigned long long)u << 32));
  return (double)f;
}

// deterministic per-CTA sums of two values -> partial[2*cta], [2*cta+1]:
// warp shuffles then one thread over the warp sums when the block is whole
// warps, else a shared-memory tree
__device__ __forceinline__ void cta_sum2(float s0, float s1, double* partial) {
  __shared__ float red[2][256];
  int t = threadIdx.y * blockDim.x + threadIdx.x;
  int nt = blockDim.x * blockDim.y;
  if ((nt & 31) == 0) {
    for (int o = 16; o > 0; o >>= 1) {
      s0 += __shfl_down_sync(0xffffffffu, s0, o);
      s1 += __shfl_down_sync(0xffffffffu, s1, o);
    }
    if ((t & 31) == 0) {
      red[0][t >> 5] = s0;
      red[1][t >> 5] = s1;
    }
    __syncthreads();
    if (t == 0)
      for (int w = 1; w < (nt >> 5); w++) {
        red[0][0] += red[0][w];
        red[1][0] += red[1][w];
      }
  } else {
    red[0][t] = s0;
    red[1][t] = s1;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
      if (t < w && t + w < nt) {
        red[0][t] += red[0][t + w];
        red[1][t] += red[1][t + w];
      }
      __syncthreads();
    }
  }
  if (t == 0) {
    long long cta = ((long long)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
    partial[2 * cta] = (double)red[0][0];
    partial[2 * cta + 1] = (double)red[1][0];
  }
}

// ---------------------------------------------------------------------------
// kernels.  Grid (x, y, z) = (position in a colour row or coarse x,
// y, z); blockDim.z = 1.

// The pointwise Newton update of one cell in FP32 (the 2x2 solve of
// RelaxGrid2D/3D in correction form), every rounding explicit so that each
// kernel that smooths computes the same bits whatever the compiler would
// contract:  a21 = -3 (pb + xv)^2 - tmp3,  b1 = g0 + c0 s1,
// b2 = g1 - c1 s0 - xv^2 (3 pb + 2 xv),  det = 1 - a12 a21,
// e0 = (b1 - a12 b2) / det,  e1 = (b2 - a21 b1) / det.
__device__ __forceinline__ void newton_cell(const BoxLev& L, float pb, float xv, float s0, float s1, float g0,
                                            float g1, float& r0, float& r1) {
  const float w = __fadd_rn(pb, xv);
  const float a21 = __fmaf_rn(__fmul_rn(-3.0f, w), w, -L.tmp3);
  const float b1 = __fmaf_rn(L.c0, s1, g0);
  const float t = __fmaf_rn(3.0f, pb, __fmul_rn(2.0f, xv));
  const float b2 = __fmaf_rn(-__fmul_rn(xv, xv), t, __fmaf_rn(-L.c1, s0, g1));
  const float rdet = __frcp_rn(__fmaf_rn(-L.a12, a21, 1.0f));
  r0 = __fmul_rn(__fmaf_rn(-L.a12, b2, b1), rdet);
  r1 = __fmul_rn(__fmaf_rn(-a21, b1, b2), rdet);
}

// One cell of a colour half-sweep of the correction smoother (RelaxGrid2D/3D
// in correction form, see mixed.cu k_mx_relax).  first = 1: e of both
// colours counts as zero (first half-sweep of a cycle); first = 2: the own
// colour's e counts as zero (second half-sweep).  Arithmetic T: float, or
// double with the FP64 coefficients on the coarsest level (FP32 storage).
template <int DIM, typename T = float>
__device__ __forceinline__ void relax_at(float* __restrict__ fp, const BoxLev& L, int c, int first, int h, int y,
                                         int z) {
  constexpr bool D = sizeof(T) == sizeof(double);
  const T c0 = D ? T(L.cd[0]) : T(L.c0), c1 = D ? T(L.cd[1]) : T(L.c1);
  const T tmp3 = D ? T(L.cd[2]) : T(L.tmp3), a12 = D ? T(L.cd[3]) : T(L.a12);
  V2 E = var2(fp, L.oe, L.half), G = var2(fp, L.og, L.half);
  const float* PB = fp + L.opb;
  int x = 2 * h + ((c + y + z + (DIM == 3 ? 1 : 0)) & 1);
  Loc<DIM> l(L, x, y, z);
  T pb = PB[l.own];
  T s0 = T(0), s1 = T(0), xv = T(0);
  if (first != 1) {
    s0 = nsum<DIM, T>(E.v0, l);
    s1 = nsum<DIM, T>(E.v1, l);
    if (first == 0) xv = E.v0[l.own];
  }
  if constexpr (!D) {
    float r0, r1;
    newton_cell(L, pb, xv, s0, s1, G.v0[l.own], G.v1[l.own], r0, r1);
    E.v0[l.own] = r0;
    E.v1[l.own] = r1;
  } else {
    T w = pb + xv;
    T a21 = T(-3) * w * w - tmp3;
    T b1 = T(G.v0[l.own]) + c0 * s1;
    T b2 = T(G.v1[l.own]) - c1 * s0 - xv * xv * (T(3) * pb + T(2) * xv);
    T rdet = T(1) / (T(1) - a12 * a21);
    E.v0[l.own] = (float)((b1 - a12 * b2) * rdet);
    E.v1[l.own] = (float)((b2 - a21 * b1) * rdet);
  }
}

// the FP64 smoother over a whole level (the coarsest level of a V-cycle
// that no small-level cycle covers): one cell of the colour per thread
template <int DIM>
__global__ void __launch_bounds__(256) k_bx_relax64(float* __restrict__ fp, BoxLev L, int c, int first) {
  int h = blockIdx.x * blockDim.x + threadIdx.x;
  int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (h < L.hh && y < L.n[1]) relax_at<DIM, double>(fp, L, c, first, h, y, blockIdx.z);
}

// Full-grid sweep: each thread takes position h of rows R*yp .. R*yp+R-1
// (n1 is a multiple of R), loading all its cells' data before any is stored
// so that R times the loads are in flight per thread.
template <int DIM, int R = 2, int MINB = 8>
__global__ void __launch_bounds__(256, MINB) k_bx_relax(float* __restrict__ fp, BoxLev L, int c, int first) {
  int h = blockIdx.x * blockDim.x + threadIdx.x;
  int yp = blockIdx.y * blockDim.y + threadIdx.y;
  int z = blockIdx.z;
  if (h >= L.hh || R * yp >= L.n[1]) return;
  V2 E = var2(fp, L.oe, L.half), G = var2(fp, L.og, L.half);
  const float* PB = fp + L.opb;
  unsigned own[R];
  float pb[R], xv[R], s0[R], s1[R], g0[R], g1[R];
  for (int k = 0; k < R; k++) {
    int y = R * yp + k;
    int x = 2 * h + ((c + y + z + (DIM == 3 ? 1 : 0)) & 1);
    Loc<DIM> l(L, x, y, z);
    own[k] = l.own;
    pb[k] = PB[l.own];
    s0[k] = s1[k] = xv[k] = 0.f;
    if (first != 1) {
      s0[k] = nsum<DIM>(E.v0, l);
      s1[k] = nsum<DIM>(E.v1, l);
      if (first == 0) xv[k] = E.v0[l.own];
    }
    g0[k] = G.v0[l.own];
    g1[k] = G.v1[l.own];
  }
  for (int k = 0; k < R; k++) {
    float r0, r1;
    newton_cell(L, pb[k], xv[k], s0[k], s1[k], g0[k], g1[k], r0, r1);
    E.v0[own[k]] = r0;
    E.v1[own[k]] = r1;
  }
}

// ---------------------------------------------------------------------------
// The same colour sweep (3D) with its rows staged in shared memory by bulk
// asynchronous copies (cp.async.bulk, completion counted on an mbarrier).
// A tile is kTileRows consecutive rows y of one plane z of the own colour; it
// needs the own rows of pb, g0, g1 (and e0 unless first) and the other
// colour's e0, e1 rows y-1..y+kTileRows at z and y..y+kTileRows-1 at z-1 and
// z+1 (periodic wrap).  Persistent CTAs walk the tiles plane by plane, the
// next tile's rows in flight while the current one is computed, so the
// memory system always has whole rows outstanding instead of one word per
// thread.  The cell update is relax_at's (newton_cell); the six neighbours
// are summed left to right, where relax_at adds the two z-neighbours as a
// pair, so the values agree to rounding, not bit for bit.
constexpr int kTileThreads = 256;
constexpr long long kWaitLimit = 1ll << 24;  // mbarrier polls before giving up

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity) {
  for (long long it = 0; it < kWaitLimit; it++) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

// floats of one stage: own pb, g0, g1, e0 (4 T rows), other e0/e1 at z
// (2 (T+2) rows), at z-1 and z+1 (4 T rows)
__host__ __device__ __forceinline__ int tile_stage_floats(int T, int hh) { return (10 * T + 4) * hh; }

// T rows per tile, NS stages (NS - 1 tiles in flight ahead of the one computed)
template <int T, int NS>
__global__ void __launch_bounds__(kTileThreads) k_bx_relax_tiled(float* __restrict__ fp, BoxLev L, int c, int first) {
  extern __shared__ __align__(128) float tsm[];
  __shared__ __align__(8) unsigned long long bar[NS];
  const int hh = L.hh, n1 = L.n[1], n2 = L.n[2];
  const int SF = tile_stage_floats(T, hh);
  const int tiles_per_plane = n1 / T, ntiles = tiles_per_plane * n2;
  const unsigned rowb = (unsigned)hh * 4u;
  const long long half = L.half;
  // bases of the colour-split arrays (variable v, colour k): off + (2v+k)*half
  const float* E = fp + L.oe;
  const float* G = fp + L.og;
  const float* PB = fp + L.opb;
  const int o = 1 - c;  // the other colour
  if (threadIdx.x == 0) {
    for (int b = 0; b < NS; b++)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&bar[b])));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  // rows of a tile into stage buffer sb: consecutive rows of one array are
  // contiguous in memory, so each array's rows go as one bulk copy (two or
  // three where the rows wrap around the plane); thread 0 issues them
  auto issue = [&](int tile, int sb) {
    if (threadIdx.x != 0) return;
    int z = tile / tiles_per_plane, y0 = (tile % tiles_per_plane) * T;
    int nrows = first == 1 ? 3 * T : (first == 2 ? 3 * T + 2 * (T + 2) + 4 * T : 4 * T + 2 * (T + 2) + 4 * T);
    unsigned b = smem_addr(&bar[sb]);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"((unsigned)nrows * rowb)
                 : "memory");
    float* base = tsm + sb * SF;
    // rows y .. y+n-1 (wrapping in the plane) of plane zz of array a -> slots from `slot`
    auto rows = [&](const float* a, int zz, int y, int n, int slot) {
      while (n > 0) {
        int yy = y < 0 ? y + n1 : (y >= n1 ? y - n1 : y);
        int run = n1 - yy < n ? n1 - yy : n;
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                smem_addr(base + (long long)slot * hh)),
            "l"(a + ((long long)zz * n1 + yy) * hh), "r"((unsigned)run * rowb), "r"(b)
            : "memory");
        y += run;
        n -= run;
        slot += run;
      }
    };
    rows(PB + (long long)c * half, z, y0, T, 0);
    rows(G + (long long)c * half, z, y0, T, T);
    rows(G + (long long)(2 + c) * half, z, y0, T, 2 * T);
    if (first == 0) rows(E + (long long)c * half, z, y0, T, 3 * T);
    if (first != 1) {
      int zm = z ? z - 1 : n2 - 1, zp = z + 1 < n2 ? z + 1 : 0;
      for (int v = 0; v < 2; v++) {
        const float* a = E + (long long)(2 * v + o) * half;
        rows(a, z, y0 - 1, T + 2, 4 * T + v * (T + 2));
        rows(a, zm, y0, T, 4 * T + 2 * (T + 2) + v * T);
        rows(a, zp, y0, T, 4 * T + 2 * (T + 2) + 2 * T + v * T);
      }
    }
  };
  int it = 0;
  int tile = blockIdx.x;
  for (int k = 0; k < NS - 1; k++)
    if (tile + k * (int)gridDim.x < ntiles) issue(tile + k * gridDim.x, k);
  bool ok = true;
  for (; tile < ntiles; tile += gridDim.x, it++) {
    int sb = it % NS;
    int next = tile + (NS - 1) * gridDim.x;  // its buffer was released by the barrier ending the last iteration
    if (next < ntiles) issue(next, (it + NS - 1) % NS);
    ok = mbar_wait(smem_addr(&bar[sb]), (unsigned)((it / NS) & 1)) && ok;
    const float* st = tsm + sb * SF;
    const float* sPB = st;
    const float* sG0 = st + T * hh;
    const float* sG1 = st + 2 * T * hh;
    const float* sE0 = st + 3 * T * hh;
    const float* sO0 = st + 4 * T * hh;          // other e0 at z, rows y0-1..y0+T
    const float* sO1 = sO0 + (T + 2) * hh;       // other e1 at z
    const float* sZ = sO1 + (T + 2) * hh;        // z-1: e0, e1; z+1: e0, e1 (T rows each)
    int z = tile / tiles_per_plane, y0 = (tile % tiles_per_plane) * T;
    for (int q = threadIdx.x; q < T * hh; q += kTileThreads) {
      int yl = q / hh, h = q - yl * hh;
      int y = y0 + yl;
      int bb = (c + y + z + 1) & 1;  // x = 2h + bb
      int xm = bb ? h : (h ? h - 1 : hh - 1);
      int xp = bb ? (h + 1 < hh ? h + 1 : 0) : h;
      float pb = sPB[q];
      float s0 = 0.f, s1 = 0.f, xv = 0.f;
      if (first != 1) {
        const float* a0 = sO0 + (yl + 1) * hh;
        const float* a1 = sO1 + (yl + 1) * hh;
        s0 = a0[xm] + a0[xp] + a0[h - hh] + a0[h + hh] + sZ[q] + sZ[2 * T * hh + q];
        s1 = a1[xm] + a1[xp] + a1[h - hh] + a1[h + hh] + sZ[T * hh + q] + sZ[3 * T * hh + q];
        if (first == 0) xv = sE0[q];
      }
      float r0, r1;
      newton_cell(L, pb, xv, s0, s1, sG0[q], sG1[q], r0, r1);
      if (!ok) r0 = r1 = __int_as_float(0x7fc00000);  // a copy that never landed: poison the sweep
      long long row = ((long long)z * n1 + y) * hh + h;
      float* Ew = fp + L.oe;
      Ew[(long long)c * half + row] = r0;
      Ew[(long long)(2 + c) * half + row] = r1;
    }
    __syncthreads();  // every thread is done with buffer sb before it is refilled
  }
  if (!ok)  // a wait gave up: give the copies still in flight a bounded time to land before the block exits
    for (int b = 0; b < NS; b++) mbar_wait(smem_addr(&bar[b]), 0u), mbar_wait(smem_addr(&bar[b]), 1u);
}

// ---------------------------------------------------------------------------
// One smoothing of a 3D level's V-cycle visit (nsmooth = 2: colour
// half-sweeps 0, 1, 0, 1) in one pass over memory.  A CTA owns TY rows y0 ..
// y0+TY-1 of the planes z0 .. z1-1 and streams the planes z0-NS .. z1+NS-1
// through a ring of NS+3 shared-memory slots, each holding the four
// colour-split e arrays of rows y0-NS .. y0+TY+NS-1 of one plane (TMA tensor
// copies of four rows of one array, at row chunks wrapped around the plane).
// Once plane i has landed, stage
// s (half-sweep s) updates plane i-s: it needs the other colour of planes
// i-s-1 .. i-s+1 at stage s-1, which stage s-1 produced in this pass or the
// last.  Each stage's rows shrink by one at both ends (its neighbours must
// be at the previous stage), so stage NS leaves rows y0 .. y0+TY-1 final,
// and the planes outside z0 .. z1-1 are computed only as halo.  Colour
// updates read only the other colour and their own cell, so the result is
// the NS separate half-sweeps' bit for bit.  g and pb come from global
// memory into registers one plane ahead of the stage that uses them.  The
// output goes to a second e array (oe_out): the input rows of a tile's halo
// belong to other CTAs' outputs.  DRAM bytes per cell for NS = 4: 8 (e,
// none when fresh) + 8 (g) + 4 (pb) read, 8 written, against 4 x 18 for four
// separate half-sweeps.
constexpr int kSmStages = 4;      // half-sweeps per pass
constexpr int kSmThreads = 512;
constexpr int kSmMinPlanes = 16;  // smallest z range of a CTA (the halo costs 2 NS planes)

__host__ __device__ constexpr int smooth_slots(int ns) { return ns + 3; }  // planes i-ns-1 .. i, i+1 in flight
__host__ __device__ constexpr long long smooth_slot_floats(int ty, int hh, int ns = kSmStages) {
  return 4LL * (ty + 2 * ns) * hh;
}
__host__ __device__ constexpr int ilog2(int n) { return n <= 1 ? 0 : 1 + ilog2(n / 2); }

// CPT consecutive cells of a colour row as one vector access (4: float4,
// 2: float2)
template <int CPT>
__device__ __forceinline__ void ldv(const float* p, float* v) {
  if constexpr (CPT == 4) {
    const float4 t = *reinterpret_cast<const float4*>(p);
    v[0] = t.x, v[1] = t.y, v[2] = t.z, v[3] = t.w;
  } else {
    const float2 t = *reinterpret_cast<const float2*>(p);
    v[0] = t.x, v[1] = t.y;
  }
}
template <int CPT>
__device__ __forceinline__ void stv(float* p, const float* v) {
  if constexpr (CPT == 4) *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
  else *reinterpret_cast<float2*>(p) = make_float2(v[0], v[1]);
}

// TY rows a tile, HH cells a colour row, FRESH: the old e counts as zero (the
// finest level's pre-smoothing), NS stages, CPT consecutive cells of a row a
// thread, NT threads a CTA.  The library runs CPT = 4 at 512 threads (two
// cells a thread at 1024 threads measured no faster: the kernel is bound by
// its instructions, not by the warps it has to hide latency).
template <int TY, int HH, bool FRESH, int NS = kSmStages, int CPT = 4, int NT = kSmThreads>
__global__ void __launch_bounds__(NT, 1) k_bx_smooth(float* __restrict__ fp, BoxLev L, long long oe_out, int nz,
                                                   const __grid_constant__ CUtensorMap emap) {
  extern __shared__ __align__(128) float ssm[];
  constexpr int NSL = smooth_slots(NS);
  constexpr int R = TY + 2 * NS, AR = R * HH, SL = 4 * AR, LG = ilog2(HH);
  constexpr int W = HH / CPT;               // threads of a colour row: CPT consecutive cells each
  constexpr int RK = NT / W;                // rows between a thread's row segments
  constexpr int KQ = (R + RK - 1) / RK;     // row segments of a thread (the same rows in every stage)
  constexpr bool CARRY = CPT == 4;          // registers for the carried in-plane values
  static_assert((1 << LG) == HH && HH % 4 == 0 && RK % 2 == 0 && (CPT == 2 || CPT == 4), "rows of 2^k cells");
  static_assert(R % 4 == 0 && TY % 4 == 0, "slots fill in chunks of four rows");
  __shared__ __align__(8) unsigned long long bar[NSL];
  const int n1 = L.n[1], n2 = L.n[2];
  const unsigned half = (unsigned)L.half;  // a level's cells are fewer than 2^31
  const int ytiles = n1 / TY;
  const int y0 = (blockIdx.x % ytiles) * TY, zc = blockIdx.x / ytiles;
  const int z0 = (int)((long long)zc * n2 / nz), z1 = (int)((long long)(zc + 1) * n2 / nz);
  const int P = z1 - z0 + 2 * NS;  // local plane j is z0 - NS + j
  const float* G = fp + L.og;
  const float* PB = fp + L.opb;
  float* EO = fp + oe_out;
  auto wrap = [](int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); };
  // this thread's cells hc .. hc+CPT-1 of rows rb + k RK: the same in every
  // stage, so that a stage's z+1 values are the ones the thread computed in
  // the stage before it, and no other thread writes what a stage reads in
  // the same pass but the rows y+-1 and the row neighbours beyond the
  // thread's cells, which were written in the pass before
  const int li = threadIdx.x % W, rb = threadIdx.x / W, hc = CPT * li;
  const int hm = (hc - 1) & (HH - 1), hp = (hc + CPT) & (HH - 1);  // the row's periodic wrap
  unsigned goff[KQ];  // the cells' offset within a plane of a colour-split array
#pragma unroll
  for (int k = 0; k < KQ; k++) goff[k] = (unsigned)(wrap(y0 - NS + rb + k * RK, n1) * HH + hc);
  if (threadIdx.x == 0) {
    for (int b = 0; b < NSL; b++) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&bar[b])));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  // lane 0 of warps 0-3: the rows y0-NS .. y0+TY+NS-1 of the four e arrays
  // of local plane j into slot k, by tensor copies of four rows of one array
  // (emap: the input e as [array][z][y][h], a box of 4 x HH cells); warp w
  // copies the row chunks w, w+4, ..., whose start rows, wrapped around the
  // plane, are whole chunks (n1 is a multiple of 4); warp 0 arms the barrier
  // with the plane's bytes.  Nothing when fresh: the first half-sweeps count
  // the old e as zero.
  auto issue = [&](int j, int k) {
    const int w = threadIdx.x >> 5;
    if (FRESH || (threadIdx.x & 31) || w >= 4 || j >= P) return;
    const unsigned b = smem_addr(&bar[k]);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    if (w == 0)
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"((unsigned)SL * 4u)
                   : "memory");
    const int zw = wrap(z0 - NS + j, n2);
    for (int ck = w; ck < R / 4; ck += 4) {
      const int yc = wrap(y0 - NS + 4 * ck, n1);
      for (int a = 0; a < 4; a++)
        asm volatile(
            "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
            "[%6];" ::"r"(smem_addr(ssm + k * SL + a * AR + ck * 4 * HH)),
            "l"(reinterpret_cast<unsigned long long>(&emap)), "r"(0), "r"(yc), "r"(zw), "r"(a), "r"(b)
            : "memory");
    }
  };
  // pb, g0, g1 of this thread's cells of stage s for the pass over local
  // plane j, in registers before that pass
  float v[NS][KQ][3][CPT];
  auto load = [&](int s, int j) {
    if (j < s || j > P - 1 - s) return;  // uniform over the CTA
    const unsigned c = (s - 1) & 1;
    const unsigned zoff = (unsigned)(wrap(z0 - NS + j, n2) * n1 * HH);
#pragma unroll
    for (int k = 0; k < KQ; k++) {
      const int r = rb + k * RK;
      if (r >= s && r <= R - 1 - s) {
        const unsigned gi = zoff + goff[k];
        ldv<CPT>(PB + (c * half + gi), v[s - 1][k][0]);
        ldv<CPT>(G + (c * half + gi), v[s - 1][k][1]);
        ldv<CPT>(G + ((2 + c) * half + gi), v[s - 1][k][2]);
      }
    }
  };
  // per stage, the other colour of the thread's cells in the plane after the
  // one last passed
  float cz[NS][CARRY ? KQ : 1][2][CPT];
  issue(0, 0);
  issue(1, 1);
  bool ok = true;
  int si = 0;               // the slot of plane i: i mod NSL
  unsigned phase = 0;       // its barrier's phase parity: (i / NSL) & 1
  auto slot = [&](int d) {  // the slot of plane i - d (0 <= d < NSL)
    const int t = si - d;
    return t < 0 ? t + NSL : t;
  };
  for (int i = 0; i < P; i++) {
    if (!FRESH) ok = mbar_wait(smem_addr(&bar[si]), phase) && ok;
    float fw[KQ][2][CPT];  // the last stage's new values: the z+1 values of the next stage
#pragma unroll
    for (int s = 1; s <= NS; s++) {
      const int j = i - s;
      if (j >= s && j <= P - 1 - s) {  // uniform over the CTA
        const int c = (s - 1) & 1, o = 1 - c;
        const int first = FRESH ? (s <= 2 ? s : 0) : 0;
        // x = 2h + bb: the parity is the same for all of the thread's rows (RK is even)
        const int bb = (c + y0 - NS + rb + z0 - NS + j + 1) & 1;
        float* S = ssm + slot(s) * SL + (rb << LG);
        const float* Sm = ssm + slot(s + 1) * SL + (rb << LG);
        const float* Sp = ssm + slot(s - 1) * SL + (rb << LG);
#pragma unroll
        for (int k = 0; k < KQ; k++) {
          const int r = rb + k * RK;
          if (r >= s && r <= R - 1 - s) {
            const int ro = k * RK * HH;
            float s0[CPT], s1[CPT], xv[CPT];
#pragma unroll
            for (int q = 0; q < CPT; q++) s0[q] = s1[q] = xv[q] = 0.f;
            if (first != 1) {
#pragma unroll
              for (int var = 0; var < 2; var++) {
                const int ao = (2 * var + o) * AR + ro;
                float a[CPT], zp[CPT], zm[CPT], ym[CPT], yp[CPT];
                // the other colour of this plane was the z+1 value of the
                // pass over plane j-1, unchanged since
                if (CARRY && j > s) {
#pragma unroll
                  for (int q = 0; q < CPT; q++) a[q] = cz[s - 1][CARRY ? k : 0][var][q];
                } else {
                  ldv<CPT>(S + ao + hc, a);
                }
                if (s == 1) {
                  ldv<CPT>(Sp + ao + hc, zp);
                } else {
#pragma unroll
                  for (int q = 0; q < CPT; q++) zp[q] = fw[k][var][q];
                }
                if (CARRY) {
#pragma unroll
                  for (int q = 0; q < CPT; q++) cz[s - 1][CARRY ? k : 0][var][q] = zp[q];
                }
                ldv<CPT>(Sm + ao + hc, zm);
                ldv<CPT>(S + ao - HH + hc, ym);
                ldv<CPT>(S + ao + HH + hc, yp);
                // a[xm] + a[xp] with xm, xp = h, h+1 (bb = 1) or h-1, h (bb = 0)
                const float edge = S[ao + (bb ? hp : hm)];
                float* acc = var ? s1 : s0;
#pragma unroll
                for (int q = 0; q < CPT; q++) {
                  const float lft = bb ? a[q] : (q ? a[q - 1] : edge);
                  const float rgt = bb ? (q + 1 < CPT ? a[q + 1] : edge) : a[q];
                  float t = lft + rgt + ym[q] + yp[q];
                  t += zm[q] + zp[q];
                  acc[q] = t;
                }
              }
              if (first == 0) ldv<CPT>(S + c * AR + ro + hc, xv);
            }
            float r0[CPT], r1[CPT];
#pragma unroll
            for (int q = 0; q < CPT; q++) {
              newton_cell(L, v[s - 1][k][0][q], xv[q], s0[q], s1[q], v[s - 1][k][1][q], v[s - 1][k][2][q], r0[q],
                          r1[q]);
              if (!ok) r0[q] = r1[q] = nanf("");  // a copy that never landed: poison the pass
              fw[k][0][q] = r0[q], fw[k][1][q] = r1[q];
            }
            stv<CPT>(S + c * AR + ro + hc, r0);
            stv<CPT>(S + (2 + c) * AR + ro + hc, r1);
          }
        }
      }
      load(s, i + 1 - s);  // the next pass's cells of this stage, in flight while the others compute
    }
    __syncthreads();  // rows y+-1 of this pass are read by the next; the slot below is free
    issue(i + 2, slot(NSL - 2));  // plane i + 2 into the slot of plane i - NS - 1, which stage NS read last
    const int j = i - NS;
    if (j >= NS && j <= P - 1 - NS) {  // plane j is final: rows NS .. NS+TY-1 of the slot
      const float* S = ssm + slot(NS) * SL + NS * HH;
      float* D = EO + (unsigned)(((z0 - NS + j) * n1 + y0) * HH);
      constexpr int n4 = (TY * HH) >> 2;
#pragma unroll
      for (int q = threadIdx.x; q < 4 * n4; q += NT) {
        const int a = q / n4, t = q - a * n4;
        reinterpret_cast<float4*>(D + (unsigned)a * half)[t] = reinterpret_cast<const float4*>(S + a * AR)[t];
      }
    }
    if (++si == NSL) si = 0, phase ^= 1u;
  }
  if (!ok)  // a wait gave up: give the copies still in flight a bounded time to land before the block exits
    for (int b = 0; b < NSL; b++) mbar_wait(smem_addr(&bar[b]), 0u), mbar_wait(smem_addr(&bar[b]), 1u);
}

// RestrictSolution on e and on the base field: coarse e = ec = R(e_fine),
// coarse pb = R(pb_fine); one coarse cell
template <int DIM>
__device__ __forceinline__ void restrict_at(float* __restrict__ fp, const BoxLev& F, const BoxLev& C, int X, int Y,
                                            int Z) {
  V2 Ef = var2(fp, F.oe, F.half);
  const float* PBf = fp + F.opb;
  float s[3] = {0.f, 0.f, 0.f};
  const int nz = DIM == 3 ? 2 : 1;
  for (int dz = 0; dz < nz; dz++)
    for (int dy = 0; dy < 2; dy++) {
      unsigned y = 2 * Y + dy, z = DIM == 3 ? 2 * Z + dz : 0;
      unsigned r = (z * (unsigned)F.n[1] + y) * (unsigned)F.hh + (unsigned)X;  // both fine cells sit at x/2 = X
      for (int c = 0; c < 2; c++) {
        unsigned i = r + (c ? (unsigned)F.half : 0u);
        s[0] += Ef.v0[i];
        s[1] += Ef.v1[i];
        s[2] += PBf[i];
      }
    }
  const float w = DIM == 2 ? 0.25f : 0.125f;
  Loc<DIM> lc(C, X, Y, Z);
  V2 Ec = var2(fp, C.oe, C.half), ECc = var2(fp, C.oec, C.half);
  Ec.v0[lc.own] = ECc.v0[lc.own] = s[0] * w;
  Ec.v1[lc.own] = ECc.v1[lc.own] = s[1] * w;
  fp[C.opb + lc.own] = s[2] * w;
}

// CoarseLoadingFunction on the correction: coarse g = R(g - M(e)) + M_c(ec)
template <int DIM>
__device__ __forceinline__ void coarse_load_at(float* __restrict__ fp, const BoxLev& F, const BoxLev& C, int X, int Y,
                                               int Z) {
  V2 Ef = var2(fp, F.oe, F.half), Gf = var2(fp, F.og, F.half);
  const float* PBf = fp + F.opb;
  float R0 = 0.f, R1 = 0.f;
  const int nz = DIM == 3 ? 2 : 1;
  for (int dz = 0; dz < nz; dz++)
    for (int dy = 0; dy < 2; dy++)
      for (int dx = 0; dx < 2; dx++) {
        Loc<DIM> l(F, 2 * X + dx, 2 * Y + dy, DIM == 3 ? 2 * Z + dz : 0);
        float m0, m1;
        mop<DIM>(Ef, F, l, PBf[l.own], m0, m1);
        R0 += Gf.v0[l.own] - m0;
        R1 += Gf.v1[l.own] - m1;
      }
  const float w = DIM == 2 ? 0.25f : 0.125f;
  Loc<DIM> lc(C, X, Y, Z);
  // M_c(ec): the coarse operator on the restricted correction
  V2 ECc = var2(fp, C.oec, C.half), Gc = var2(fp, C.og, C.half);
  float m0, m1;
  mop<DIM>(ECc, C, lc, fp[C.opb + lc.own], m0, m1);
  Gc.v0[lc.own] = R0 * w + m0;
  Gc.v1[lc.own] = R1 * w + m1;
}

// RestrictSolution and the fine half of CoarseLoadingFunction in one pass
// over the fine cells: coarse e = ec = R(e), coarse pb = R(pb) and coarse
// g = R(g - M(e)); the coarse operator M_c(ec) needs the neighbours' ec, so
// k_bx_coarse_op adds it in a second (coarse-sized) pass.  Every fine value
// is loaded before the first store; six blocks per SM (40 registers, no
// spills) against five uncapped: 30 vs 37 us averaged over the levels.
template <int DIM>
__device__ __forceinline__ void restrict_load_at(float* __restrict__ fp, const BoxLev& F, const BoxLev& C, int X,
                                                 int Y, int Z) {
  V2 Ef = var2(fp, F.oe, F.half), Gf = var2(fp, F.og, F.half);
  const float* PBf = fp + F.opb;
  float s0 = 0.f, s1 = 0.f, s2 = 0.f, R0 = 0.f, R1 = 0.f;
  const int nz = DIM == 3 ? 2 : 1;
  for (int dz = 0; dz < nz; dz++)
    for (int dy = 0; dy < 2; dy++)
      for (int dx = 0; dx < 2; dx++) {
        Loc<DIM> l(F, 2 * X + dx, 2 * Y + dy, DIM == 3 ? 2 * Z + dz : 0);
        float pb = PBf[l.own];
        s0 += Ef.v0[l.own];
        s1 += Ef.v1[l.own];
        s2 += pb;
        float m0, m1;
        mop<DIM>(Ef, F, l, pb, m0, m1);
        R0 += Gf.v0[l.own] - m0;
        R1 += Gf.v1[l.own] - m1;
      }
  const float w = DIM == 2 ? 0.25f : 0.125f;
  Loc<DIM> lc(C, X, Y, Z);
  V2 Ec = var2(fp, C.oe, C.half), ECc = var2(fp, C.oec, C.half), Gc = var2(fp, C.og, C.half);
  Ec.v0[lc.own] = ECc.v0[lc.own] = s0 * w;
  Ec.v1[lc.own] = ECc.v1[lc.own] = s1 * w;
  fp[C.opb + lc.own] = s2 * w;
  Gc.v0[lc.own] = R0 * w;
  Gc.v1[lc.own] = R1 * w;
}
template <int DIM>
__global__ void __launch_bounds__(256, 6) k_bx_restrict_load(float* __restrict__ fp, BoxLev F, BoxLev C) {
  int X = blockIdx.x * blockDim.x + threadIdx.x;
  int Y = blockIdx.y * blockDim.y + threadIdx.y;
  if (X < C.n[0] && Y < C.n[1]) restrict_load_at<DIM>(fp, F, C, X, Y, blockIdx.z);
}
// coarse g += M_c(ec), the coarse operator on the restricted correction
template <int DIM>
__global__ void __launch_bounds__(256) k_bx_coarse_op(float* __restrict__ fp, BoxLev C) {
  int X = blockIdx.x * blockDim.x + threadIdx.x;
  int Y = blockIdx.y * blockDim.y + threadIdx.y;
  if (X >= C.n[0] || Y >= C.n[1]) return;
  Loc<DIM> lc(C, X, Y, blockIdx.z);
  V2 ECc = var2(fp, C.oec, C.half), Gc = var2(fp, C.og, C.half);
  float g0 = Gc.v0[lc.own], g1 = Gc.v1[lc.own];
  float m0, m1;
  mop<DIM>(ECc, C, lc, fp[C.opb + lc.own], m0, m1);
  Gc.v0[lc.own] = g0 + m0;
  Gc.v1[lc.own] = g1 + m1;
}

// CorrectFine on e: e_fine += P(e_c - ec), per-direction (3,1)/4 weights
// (Bi/TriLinProlongationP1, gridutilities.f90:156-195, :510-566).  Thread T
// (per dimension 0..nc-1) owns fine cells 2T-1 (wrapped) and 2T, between
// coarse cells T-1 (wrapped) and T.
template <int DIM>
__device__ __forceinline__ void prolong_at(float* __restrict__ fp, const BoxLev& F, const BoxLev& C, int T0, int T1,
                                           int T2) {
  const int T[3] = {T0, T1, T2};
  int cx[2][3], fx[2][3];
  for (int d = 0; d < 3; d++) {
    int n = C.n[d];
    cx[0][d] = T[d] ? T[d] - 1 : n - 1;
    cx[1][d] = T[d];
    fx[0][d] = T[d] ? 2 * T[d] - 1 : 2 * n - 1;
    fx[1][d] = 2 * T[d];
  }
  constexpr int NZ = DIM == 3 ? 2 : 1;
  V2 Ec = var2(fp, C.oe, C.half), ECc = var2(fp, C.oec, C.half), Ef = var2(fp, F.oe, F.half);
  // corrections e_c - ec at the 2x2(x2) coarse corners, both variables
  float a[2][NZ][2][2];
  for (int dz = 0; dz < NZ; dz++)
    for (int dy = 0; dy < 2; dy++)
      for (int dx = 0; dx < 2; dx++) {
        Loc<DIM> l(C, cx[dx][0], cx[dy][1], DIM == 3 ? cx[dz][2] : 0);
        a[0][dz][dy][dx] = Ec.v0[l.own] - ECc.v0[l.own];
        a[1][dz][dy][dx] = Ec.v1[l.own] - ECc.v1[l.own];
      }
  // weight 3/4 on the near coarse cell (f = 0: the first, f = 1: the second)
  auto w1 = [](float lo, float hi, int f) { return f == 0 ? 3.0f * lo + hi : lo + 3.0f * hi; };
  // every fine value is loaded before the first store, so the loads of one
  // thread are in flight together (a store to fp could alias a later load)
  constexpr int NF = 4 * NZ;
  unsigned own[NF];
  float val[NF][2];
  for (int m = 0; m < NF; m++) {
    int fxi = m & 1, fy = (m >> 1) & 1, fz = m >> 2;
    Loc<DIM> l(F, fx[fxi][0], fx[fy][1], DIM == 3 ? fx[fz][2] : 0);
    own[m] = l.own;
    val[m][0] = Ef.v0[l.own];
    val[m][1] = Ef.v1[l.own];
  }
  for (int m = 0; m < NF; m++) {
    int fxi = m & 1, fy = (m >> 1) & 1, fz = m >> 2;
    for (int v = 0; v < 2; v++) {
      float r0 = w1(w1(a[v][0][0][0], a[v][0][0][1], fxi), w1(a[v][0][1][0], a[v][0][1][1], fxi), fy);
      float add;
      if (DIM == 2) {
        add = r0 * (1.0f / 16.0f);
      } else {
        float r1 =
            w1(w1(a[v][NZ - 1][0][0], a[v][NZ - 1][0][1], fxi), w1(a[v][NZ - 1][1][0], a[v][NZ - 1][1][1], fxi), fy);
        add = w1(r0, r1, fz) * (1.0f / 64.0f);
      }
      val[m][v] += add;
    }
  }
  for (int m = 0; m < NF; m++) {
    Ef.v0[own[m]] = val[m][0];
    Ef.v1[own[m]] = val[m][1];
  }
}
template <int DIM>
__global__ void __launch_bounds__(256) k_bx_prolong(float* __restrict__ fp, BoxLev F, BoxLev C) {
  int X = blockIdx.x * blockDim.x + threadIdx.x;
  int Y = blockIdx.y * blockDim.y + threadIdx.y;
  if (X < C.n[0] && Y < C.n[1]) prolong_at<DIM>(fp, F, C, X, Y, blockIdx.z);
}

// The V-cycle on the coarse end of the hierarchy (levels with at most
// kSmallCells cells) in one CTA: the same phases as bx_vcycle, separated by
// __syncthreads() instead of kernel boundaries, so a cycle spends one launch
// instead of eleven per level on grids too small to fill the GPU.
constexpr int kSmallCells = 8192;
constexpr int kSmallThreads = 512;
struct SmallLevels {
  BoxLev L[kNLev];  // L[0] the top (finest) small level, then coarser
  int n;
};

// q = i / n, r = i % n for i >= 0: a shift and a mask when n is a power of
// two (every extent of a periodic box level here; the branch is uniform
// across the CTA), the division otherwise
__device__ __forceinline__ void divmod(int i, int n, int& q, int& r) {
  if ((n & (n - 1)) == 0) {
    q = i >> (__ffs(n) - 1);
    r = i & (n - 1);
  } else {
    q = i / n;
    r = i - q * n;
  }
}
// linear index j of an n0 x n1 x n2 grid -> (x, y, z)
__device__ __forceinline__ void unflatten(int j, int n0, int n1, int& x, int& y, int& z) {
  int r;
  divmod(j, n0, r, x);
  divmod(r, n1, z, y);
}

template <int DIM, typename T = float>
__device__ __forceinline__ void small_relax(float* fp, const BoxLev& L, int nsmooth, bool fresh) {
  int cnt = L.hh * L.n[1] * L.n[2];
  for (int pass = 1; pass <= nsmooth; pass++)
    for (int c = 0; c < 2; c++) {
      int first = (fresh && pass == 1) ? c + 1 : 0;
      for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
        int h, y, z;
        unflatten(i, L.hh, L.n[1], h, y, z);
        relax_at<DIM, T>(fp, L, c, first, h, y, z);
      }
      __syncthreads();
    }
}

template <int DIM>
__device__ __forceinline__ void small_cycle(float* fp, const SmallLevels& S, int nsmooth, int fresh) {
  for (int i = 0; i < S.n; i++) {
    const BoxLev& F = S.L[i];
    if (i == S.n - 1) {  // the coarsest level: FP64 arithmetic
      small_relax<DIM, double>(fp, F, nsmooth, fresh && i == 0);
      break;
    }
    small_relax<DIM>(fp, F, nsmooth, fresh && i == 0);
    const BoxLev& C = S.L[i + 1];
    int cnt = C.n[0] * C.n[1] * C.n[2];
    for (int j = threadIdx.x; j < cnt; j += blockDim.x) {
      int X, Y, Z;
      unflatten(j, C.n[0], C.n[1], X, Y, Z);
      restrict_at<DIM>(fp, F, C, X, Y, Z);
    }
    __syncthreads();
    for (int j = threadIdx.x; j < cnt; j += blockDim.x) {
      int X, Y, Z;
      unflatten(j, C.n[0], C.n[1], X, Y, Z);
      coarse_load_at<DIM>(fp, F, C, X, Y, Z);
    }
    __syncthreads();
  }
  for (int i = S.n - 2; i >= 0; i--) {
    const BoxLev &F = S.L[i], &C = S.L[i + 1];
    int cnt = C.n[0] * C.n[1] * C.n[2];
    for (int j = threadIdx.x; j < cnt; j += blockDim.x) {
      int X, Y, Z;
      unflatten(j, C.n[0], C.n[1], X, Y, Z);
      prolong_at<DIM>(fp, F, C, X, Y, Z);
    }
    __syncthreads();
    small_relax<DIM>(fp, F, nsmooth, false);
  }
}

template <int DIM>
__global__ void __launch_bounds__(kSmallThreads) k_bx_small_vcycle(float* __restrict__ fp, SmallLevels S, int nsmooth,
                                                                   int fresh) {
  small_cycle<DIM>(fp, S, nsmooth, fresh);
}

// The same cycle on a copy in shared memory: the small levels' arrays are
// one contiguous range of the pool, fp[lo, lo + nf) (levels are laid out
// finest first, every array start a multiple of 64 floats), so the CTA
// copies the range in, cycles on it with S's offsets taken relative to lo,
// and copies it back.  Every phase then waits on shared memory instead of
// L2.
constexpr int kSmallSmemMax = 200 * 1024;
template <int DIM>
__global__ void __launch_bounds__(kSmallThreads) k_bx_small_vcycle_smem(float* __restrict__ fp, SmallLevels S,
                                                                        long long lo, int nf, int nsmooth, int fresh) {
  extern __shared__ float4 sm4[];
  float4* g4 = reinterpret_cast<float4*>(fp + lo);
  for (int i = threadIdx.x; i < nf / 4; i += blockDim.x) sm4[i] = g4[i];
  __syncthreads();
  small_cycle<DIM>(reinterpret_cast<float*>(sm4), S, nsmooth, fresh);
  __syncthreads();
  for (int i = threadIdx.x; i < nf / 4; i += blockDim.x) g4[i] = sm4[i];
}

// The pool range [lo, hi) of the small levels' arrays, S rebased to lo.
// False when it does not fit kSmallSmemMax.
bool small_in_smem(SmallLevels& S, long long& lo, int& nf) {
  lo = S.L[0].oe;
  long long hi = 0;
  for (int i = 0; i < S.n; i++) {
    const BoxLev& L = S.L[i];
    long long ends[4] = {L.oe + 4 * L.half, L.og + 4 * L.half,
                         L.opb + (L.oec < 0 ? 4 : 2) * L.half, L.oec < 0 ? 0 : L.oec + 4 * L.half};
    for (long long e : ends) hi = std::max(hi, e);
    lo = std::min({lo, L.oe, L.og, L.opb, L.oec < 0 ? lo : L.oec});
  }
  hi = (hi + 63) & ~63LL;
  if (lo % 4 || (hi - lo) * (long long)sizeof(float) > kSmallSmemMax) return false;
  nf = (int)(hi - lo);
  for (int i = 0; i < S.n; i++) {
    BoxLev& L = S.L[i];
    L.oe -= lo;
    L.og -= lo;
    L.opb -= lo;
    if (L.oec >= 0) L.oec -= lo;
  }
  return true;
}

// After a cycle on the finest level: tracked residual g <- g - M(e) (M at
// this cycle's base field), its per-CTA sums of squares, then qbar += e as
// double-float.  One row (2D) or two rows (3D) per thread; every load
// precedes every store.  Two rows fit 48 registers without spills, five
// blocks per SM (61 registers at four blocks took 185 us at 256^3, 174 us
// capped).
template <int DIM, int R = 1>
__global__ void __launch_bounds__(256, R == 1 ? 6 : 5) k_bx_track_update(float* __restrict__ fp, BoxLev L,
                                                                       long long oqlo, double* __restrict__ partial) {
  // R rows per thread (y = R yp .. R yp + R - 1): every load of the R cells
  // is issued before the first store, R times the loads in flight
  int x = blockIdx.x * blockDim.x + threadIdx.x;
  int yp = blockIdx.y * blockDim.y + threadIdx.y;
  int z = blockIdx.z;
  float s0 = 0.f, s1 = 0.f;
  if (x < L.n[0] && R * yp < L.n[1]) {
    V2 E = var2(fp, L.oe, L.half), G = var2(fp, L.og, L.half);
    V2 QH = var2(fp, L.opb, L.half), QL = var2(fp, oqlo, L.half);  // the base field is qhi(phi)
    unsigned own[R];
    float a0[R], a1[R], th0[R], tl0[R], th1[R], tl1[R];
    for (int k = 0; k < R; k++) {
      Loc<DIM> l(L, x, R * yp + k, z);
      unsigned i = l.own;
      own[k] = i;
      float h0 = QH.v0[i], h1 = QH.v1[i], lo0 = QL.v0[i], lo1 = QL.v1[i];
      float e0 = E.v0[i], e1 = E.v1[i];
      float m0, m1;
      mop_track<DIM>(E, L, l, h0, m0, m1);
      a0[k] = G.v0[i] - m0;
      a1[k] = G.v1[i] - m1;
      DF t0 = two_sum(h0, e0);
      t0 = fast_two_sum(t0.h, t0.l + lo0);
      DF t1 = two_sum(h1, e1);
      t1 = fast_two_sum(t1.h, t1.l + lo1);
      th0[k] = t0.h, tl0[k] = t0.l, th1[k] = t1.h, tl1[k] = t1.l;
    }
    for (int k = 0; k < R; k++) {
      unsigned i = own[k];
      G.v0[i] = a0[k];
      G.v1[i] = a1[k];
      QH.v0[i] = th0[k];
      QL.v0[i] = tl0[k];
      QH.v1[i] = th1[k];
      QL.v1[i] = tl1[k];
      s0 += a0[k] * a0[k];
      s1 += a1[k] * a1[k];
    }
  }
  cta_sum2(s0, s1, partial);
}

// The true residual r = f - N(qbar) of the finest level in double-float
// (ErrorAFAS, afasroutines.f90:113-233, with f = (phi_old, -phi_old)); g is
// set to r and the per-CTA sums of r^2 go to partial.
template <int DIM>
__global__ void __launch_bounds__(256) k_bx_resid(float* __restrict__ fp, BoxLev L, long long oqlo, long long ofhi,
                                                  long long oflo, double* __restrict__ partial) {
  int x = blockIdx.x * blockDim.x + threadIdx.x;
  int y = blockIdx.y * blockDim.y + threadIdx.y;
  int z = blockIdx.z;
  float s0 = 0.f, s1 = 0.f;
  if (x < L.n[0] && y < L.n[1]) {
    const DF c0 = {L.c0h, L.c0l}, c1 = {L.c1h, L.c1l};
    V2 QH = var2(fp, L.opb, L.half), QL = var2(fp, oqlo, L.half), G = var2(fp, L.og, L.half);
    Loc<DIM> l(L, x, y, z);
    const unsigned nbi[6] = {l.xm, l.xp, l.ym, l.yp, l.zm, l.zp};
    DF v[2], nb[2][6];
    for (int q = 0; q < 2; q++) {
      const float* hi = q ? QH.v1 : QH.v0;
      const float* lo = q ? QL.v1 : QL.v0;
      v[q] = {hi[l.own], lo[l.own]};
      for (int m = 0; m < 2 * DIM; m++) nb[q][m] = {hi[nbi[m]], lo[nbi[m]]};
    }
    DF f1 = {fp[ofhi + l.own], fp[oflo + l.own]};
    DF lphi = df_lap<DIM>(nb[0], v[0]);
    DF lmu = df_lap<DIM>(nb[1], v[1]);
    // r1 = f1 - (phi - c0 lap(mu)); r2 = -f1 - (mu - phi^3 + c1 lap(phi))
    DF r1 = df_add(df_add(f1, df_neg(v[0])), df_mul(c0, lmu));
    DF p3 = df_mul(df_mul(v[0], v[0]), v[0]);
    DF r2 = df_add(df_add(df_neg(df_add(f1, v[1])), p3), df_neg(df_mul(c1, lphi)));
    float a0 = r1.h + r1.l, a1 = r2.h + r2.l;
    G.v0[l.own] = a0;
    G.v1[l.own] = a1;
    s0 = a0 * a0;
    s1 = a1 * a1;
  }
  cta_sum2(s0, s1, partial);
}

// FP64 q (ghosted Fortran layout) -> qhi/qlo, and f = (phi_old, -phi_old) as
// fhi/flo, on the finest level; two cells (x = 2h, 2h+1) per thread
template <int DIM>
__global__ void __launch_bounds__(256) k_bx_split(const double* __restrict__ pool, long long oq, long long oqold,
                                                  long long sq, int qn0, int qn1, float* __restrict__ fp, BoxLev L,
                                                  long long oqlo, long long ofhi, long long oflo) {
  int h = blockIdx.x * blockDim.x + threadIdx.x;
  int y = blockIdx.y * blockDim.y + threadIdx.y;
  int z = blockIdx.z;
  if (h >= L.hh || y >= L.n[1]) return;
  long long g = (2 * h + 1) + (long long)(y + 1) * qn0 + (DIM == 3 ? (long long)(z + 1) * qn0 * qn1 : 0);
  double in[2][3];  // the two cells' phi, mu, phi_old, loaded before any store
  for (int b = 0; b < 2; b++) {
    in[b][0] = pool[oq + g + b];
    in[b][1] = pool[oq + sq + g + b];
    in[b][2] = pool[oqold + g + b];
  }
  V2 QH = var2(fp, L.opb, L.half), QL = var2(fp, oqlo, L.half);
  for (int b = 0; b < 2; b++) {
    Loc<DIM> l(L, 2 * h + b, y, z);
    DF s0 = split64(in[b][0]), s1 = split64(in[b][1]), f = split64(in[b][2]);
    QH.v0[l.own] = s0.h;
    QL.v0[l.own] = s0.l;
    QH.v1[l.own] = s1.h;
    QL.v1[l.own] = s1.l;
    fp[ofhi + l.own] = f.h;
    fp[oflo + l.own] = f.l;
  }
}

// k_bx_split for a step that follows a box solve on the same q: with g the
// true residual r_old = f_old - N(q) and f_old in fhi/flo, the residual for
// the new f = (phi_old, -phi_old) is r_old + (f_new - f_old), so g becomes
// g + (d, -d) with d = f_new - f_old in double-float, and the per-CTA sums
// of g^2 go to partial (what k_bx_resid would give, without its
// double-float operator evaluation).
template <int DIM>
__global__ void __launch_bounds__(256) k_bx_split_warm(const double* __restrict__ pool, long long oq, long long oqold,
                                                       long long sq, int qn0, int qn1, float* __restrict__ fp,
                                                       BoxLev L, long long oqlo, long long ofhi, long long oflo,
                                                       double* __restrict__ partial) {
  int h = blockIdx.x * blockDim.x + threadIdx.x;
  int y = blockIdx.y * blockDim.y + threadIdx.y;
  int z = blockIdx.z;
  float s0 = 0.f, s1 = 0.f;
  if (h < L.hh && y < L.n[1]) {
    long long g = (2 * h + 1) + (long long)(y + 1) * qn0 + (DIM == 3 ? (long long)(z + 1) * qn0 * qn1 : 0);
    V2 QH = var2(fp, L.opb, L.half), QL = var2(fp, oqlo, L.half), G = var2(fp, L.og, L.half);
    double in[2][3];
    unsigned own[2];
    float fo[2][2], go[2][2];  // old f (hi, lo) and g, loaded before any store
    for (int b = 0; b < 2; b++) {
      in[b][0] = pool[oq + g + b];
      in[b][1] = pool[oq + sq + g + b];
      in[b][2] = pool[oqold + g + b];
      Loc<DIM> l(L, 2 * h + b, y, z);
      own[b] = l.own;
      fo[b][0] = fp[ofhi + l.own];
      fo[b][1] = fp[oflo + l.own];
      go[b][0] = G.v0[l.own];
      go[b][1] = G.v1[l.own];
    }
    for (int b = 0; b < 2; b++) {
      unsigned i = own[b];
      DF s0v = split64(in[b][0]), s1v = split64(in[b][1]), f = split64(in[b][2]);
      DF d = df_add(f, df_neg(DF{fo[b][0], fo[b][1]}));
      DF r1 = df_add(DF{go[b][0], 0.f}, d), r2 = df_add(DF{go[b][1], 0.f}, df_neg(d));
      float a0 = r1.h + r1.l, a1 = r2.h + r2.l;
      QH.v0[i] = s0v.h;
      QL.v0[i] = s0v.l;
      QH.v1[i] = s1v.h;
      QL.v1[i] = s1v.l;
      fp[ofhi + i] = f.h;
      fp[oflo + i] = f.l;
      G.v0[i] = a0;
      G.v1[i] = a1;
      s0 += a0 * a0;
      s1 += a1 * a1;
    }
  }
  cta_sum2(s0, s1, partial);
}

// qhi + qlo -> FP64 q (interior of the finest level)
template <int DIM>
__global__ void __launch_bounds__(256) k_bx_merge(double* __restrict__ pool, long long oq, long long sq, int qn0,
                                                  int qn1, float* __restrict__ fp, BoxLev L, long long oqlo) {
  int h = blockIdx.x * blockDim.x + threadIdx.x;
  int y = blockIdx.y * blockDim.y + threadIdx.y;
  int z = blockIdx.z;
  if (h >= L.hh || y >= L.n[1]) return;
  long long g = (2 * h + 1) + (long long)(y + 1) * qn0 + (DIM == 3 ? (long long)(z + 1) * qn0 * qn1 : 0);
  V2 QH = var2(fp, L.opb, L.half), QL = var2(fp, oqlo, L.half);
  float hi[2][2], lo[2][2];  // loaded before any store
  for (int b = 0; b < 2; b++) {
    Loc<DIM> l(L, 2 * h + b, y, z);
    hi[b][0] = QH.v0[l.own];
    hi[b][1] = QH.v1[l.own];
    lo[b][0] = QL.v0[l.own];
    lo[b][1] = QL.v1[l.own];
  }
  for (int b = 0; b < 2; b++)
    for (int v = 0; v < 2; v++) pool[oq + v * sq + g + b] = f2d(hi[b][v]) + f2d(lo[b][v]);
}

// ---------------------------------------------------------------------------
// host side

struct Launch {
  dim3 g, b;
};
// threads over (nx, ny, nz) with up to 128 along x and 256 per block
Launch shape(int nx, int ny, int nz) {
  int tx = nx >= 128 ? 128 : nx;
  int ty = std::max(1, 256 / tx);
  if (ty > ny) ty = ny;
  return {dim3((nx + tx - 1) / tx, (ny + ty - 1) / ty, nz), dim3(tx, ty, 1)};
}
long long ctas(const Launch& s) { return (long long)s.g.x * s.g.y * s.g.z; }

#define BX_LAUNCH(H, SH, KER, ...)                                            \
  do {                                                                        \
    if ((H).ndims == 2) KER<2><<<(SH).g, (SH).b, 0, (H).s>>>(__VA_ARGS__);    \
    else KER<3><<<(SH).g, (SH).b, 0, (H).s>>>(__VA_ARGS__);                   \
    int r__ = after_launch(H, 1);                                             \
    if (r__) return r__;                                                      \
  } while (0)

BoxLev& B(Hier& H, int level) { return H.blev[level + kMaxDepth]; }

// The staged sweep (box_sweep 2) applies to 3D levels whose rows are whole
// 16-byte units and whose planes split into whole 8-row tiles, large enough
// to fill the GPU; two stages of 8 rows measured fastest of the staged forms.
constexpr int kTileT = 8, kTileNS = 2;
bool staged_relax(const Hier& H, const BoxLev& L) {
  if (H.box_sweep != 2 || H.ndims != 3) return false;
  long long smem = (long long)kTileNS * tile_stage_floats(kTileT, L.hh) * 4;
  return L.hh % 4 == 0 && L.hh >= 64 && smem <= 200 * 1024 && L.n[1] % kTileT == 0 &&
         (kTileT * L.hh) % kTileThreads == 0;
}

int launch_staged(Hier& H, const BoxLev& L, int c, int first) {
  int occ = 0;
  int smem = kTileNS * tile_stage_floats(kTileT, L.hh) * (int)sizeof(float);
  auto ker = k_bx_relax_tiled<kTileT, kTileNS>;
  cudaError_t e = cudaFuncSetAttribute(ker, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(k_bx_relax_tiled)");
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, ker, kTileThreads, smem);
  if (e != cudaSuccess || occ < 1) return cuda_fail(e, "occupancy(k_bx_relax_tiled)");
  int ntiles = (L.n[1] / kTileT) * L.n[2];
  int grid = std::min(ntiles, occ * H.box_sms);
  ker<<<grid, kTileThreads, smem, H.s>>>(H.fpool, L, c, first);
  return after_launch(H, 1);
}

// The one-pass smoothing (box_sweep 3): 3D levels whose colour rows hold 128
// cells (tiles of 8 rows; the ring fills 224 KB of shared memory), at least
// one tile and its halo per plane.  Levels of 64-cell rows (tiles of 16 rows)
// compile but measured slower than four sweeps on a GB300 (128^3: 62 against
// 36 us: 64 CTAs), so they keep the sweeps.
int smooth_rows(const BoxLev& L) {
  const int ty = L.hh == 128 ? 8 : 0;
  return ty && L.n[1] % ty == 0 && L.n[1] >= ty + 2 * kSmStages ? ty : 0;
}
bool smooth_fits(const Hier& H, const BoxLev& L) {
  return H.ndims == 3 && L.n[2] >= kSmStages && smooth_rows(L) > 0;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library); null when the driver does not provide it
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }();
  return fn;
}

// the tensor map of a level's e arrays at offset oe: [array][z][y][h] with
// h innermost, a box of four rows of one array
int e_tensor_map(Hier& H, const BoxLev& L, long long oe, CUtensorMap* m) {
  const PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc) return cuda_fail(cudaErrorNotSupported, "cuTensorMapEncodeTiled entry point");
  const cuuint64_t dims[4] = {(cuuint64_t)L.hh, (cuuint64_t)L.n[1], (cuuint64_t)L.n[2], 4};
  const cuuint64_t strides[3] = {(cuuint64_t)L.hh * 4, (cuuint64_t)L.hh * L.n[1] * 4, (cuuint64_t)L.half * 4};
  const cuuint32_t box[4] = {(cuuint32_t)L.hh, 4, 1, 1};
  const cuuint32_t es[4] = {1, 1, 1, 1};
  CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, H.fpool + oe, dims, strides, box, es,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return cuda_fail(cudaErrorInvalidValue, "cuTensorMapEncodeTiled");
  return BSAMG_OK;
}

// out_oe = e after two red-black passes from e at in.oe (fresh: from zero)
int bx_smooth(Hier& H, const BoxLev& in, long long out_oe, bool fresh) {
  const int ty = smooth_rows(in);
  const int ytiles = in.n[1] / ty;
  int nz = std::max(1, std::min(H.box_sms / ytiles, in.n[2] / kSmMinPlanes));
  size_t smem = (size_t)smooth_slots(kSmStages) * smooth_slot_floats(ty, in.hh) * sizeof(float);
  static std::atomic<unsigned long long> attr;  // the kernels' shared-memory limit, per device
  if (needs_setup(attr, H.ctx->device)) {
    for (auto kf : {k_bx_smooth<8, 128, true>, k_bx_smooth<8, 128, false>}) {
      cudaError_t e = cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(k_bx_smooth)");
    }
    mark_setup(attr, H.ctx->device);
  }
  CUtensorMap emap;
  int r = e_tensor_map(H, in, in.oe, &emap);
  if (r) return r;
  auto ker = fresh ? k_bx_smooth<8, 128, true> : k_bx_smooth<8, 128, false>;
  ker<<<ytiles * nz, kSmThreads, smem, H.s>>>(H.fpool, in, out_oe, nz, emap);
  return after_launch(H, 1);
}
bool smooth_applies(const Hier& H, const BoxLev& L, int nsmooth) {
  return H.box_sweep == 3 && nsmooth == 2 && L.oe2 >= 0;
}

int bx_relax(Hier& H, int level, int c, int first) {
  BoxLev& L = B(H, level);
  if (staged_relax(H, L)) return launch_staged(H, L, c, first);
  if ((H.box_sweep == 1 || H.box_sweep == 3) && H.ndims == 3 && L.n[1] % 4 == 0) {
    // four rows per thread at five blocks per SM (40 registers): four
    // cells' loads in flight per thread
    Launch sh = shape(L.hh, L.n[1] / 4, L.n[2]);
    k_bx_relax<3, 4, 5><<<sh.g, sh.b, 0, H.s>>>(H.fpool, L, c, first);
    return after_launch(H, 1);
  }
  Launch sh = shape(L.hh, L.n[1] / 2, L.n[2]);
  BX_LAUNCH(H, sh, k_bx_relax, H.fpool, L, c, first);
  return BSAMG_OK;
}

// coarse: the V-cycle's coarsest level, smoothed in FP64 arithmetic
int bx_level_relax(Hier& H, int level, int nsmooth, bool fresh, bool coarse = false) {
  for (int pass = 1; pass <= nsmooth; pass++)
    for (int c = 0; c < 2; c++) {
      const int first = (fresh && pass == 1) ? c + 1 : 0;
      if (coarse) {
        BoxLev& L = B(H, level);
        Launch sh = shape(L.hh, L.n[1], L.n[2]);
        BX_LAUNCH(H, sh, k_bx_relax64, H.fpool, L, c, first);
        continue;
      }
      int r = bx_relax(H, level, c, first);
      if (r) return r;
    }
  return BSAMG_OK;
}

// AFASVcycle (afasroutines.f90:495-529) on the correction
int bx_vcycle(Hier& H, int level, int minlevel, int nsmooth, bool fresh) {
  if (2 * B(H, level).half <= kSmallCells) {
    SmallLevels S{};
    for (int l = level; l >= minlevel; l--) S.L[S.n++] = B(H, l);
    long long lo;
    int nf;
    if (small_in_smem(S, lo, nf)) {
      static std::atomic<unsigned long long> attr[2];  // the kernels' shared-memory limit, per device
      if (needs_setup(attr[H.ndims - 2], H.ctx->device)) {
        cudaError_t e = H.ndims == 2 ? cudaFuncSetAttribute(k_bx_small_vcycle_smem<2>,
                                                            cudaFuncAttributeMaxDynamicSharedMemorySize, kSmallSmemMax)
                                     : cudaFuncSetAttribute(k_bx_small_vcycle_smem<3>,
                                                            cudaFuncAttributeMaxDynamicSharedMemorySize, kSmallSmemMax);
        if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(k_bx_small_vcycle_smem)");
        mark_setup(attr[H.ndims - 2], H.ctx->device);
      }
      size_t smem = (size_t)nf * sizeof(float);
      if (H.ndims == 2)
        k_bx_small_vcycle_smem<2><<<1, kSmallThreads, smem, H.s>>>(H.fpool, S, lo, nf, nsmooth, fresh ? 1 : 0);
      else
        k_bx_small_vcycle_smem<3><<<1, kSmallThreads, smem, H.s>>>(H.fpool, S, lo, nf, nsmooth, fresh ? 1 : 0);
      return after_launch(H, 1);
    }
    if (H.ndims == 2) k_bx_small_vcycle<2><<<1, kSmallThreads, 0, H.s>>>(H.fpool, S, nsmooth, fresh ? 1 : 0);
    else k_bx_small_vcycle<3><<<1, kSmallThreads, 0, H.s>>>(H.fpool, S, nsmooth, fresh ? 1 : 0);
    return after_launch(H, 1);
  }
  if (level > minlevel && smooth_applies(H, B(H, level), nsmooth)) {
    // one-pass smoothings: e to the level's second array before the
    // coarse correction and back after it
    BoxLev F = B(H, level), Fb = F;
    Fb.oe = F.oe2;
    const BoxLev& C = B(H, level - 1);
    Launch sc = shape(C.n[0], C.n[1], C.n[2]);
    int r = bx_smooth(H, F, F.oe2, fresh);
    if (r) return r;
    BX_LAUNCH(H, sc, k_bx_restrict_load, H.fpool, Fb, C);
    BX_LAUNCH(H, sc, k_bx_coarse_op, H.fpool, C);
    if ((r = bx_vcycle(H, level - 1, minlevel, nsmooth, false))) return r;
    BX_LAUNCH(H, sc, k_bx_prolong, H.fpool, Fb, C);
    return bx_smooth(H, Fb, F.oe, false);
  }
  int r = bx_level_relax(H, level, nsmooth, fresh, level == minlevel);
  if (r) return r;
  if (level > minlevel) {
    BoxLev &F = B(H, level), &C = B(H, level - 1);
    Launch sc = shape(C.n[0], C.n[1], C.n[2]);
    BX_LAUNCH(H, sc, k_bx_restrict_load, H.fpool, F, C);
    BX_LAUNCH(H, sc, k_bx_coarse_op, H.fpool, C);
    if ((r = bx_vcycle(H, level - 1, minlevel, nsmooth, false))) return r;
    BX_LAUNCH(H, sc, k_bx_prolong, H.fpool, F, C);
    if ((r = bx_level_relax(H, level, nsmooth, false))) return r;
  }
  return BSAMG_OK;
}

int bx_finish(Hier& H, int finest, long long nparts, int errortype, bool to_host = true) {
  int r = after_launch(H, launch_norm_finish(H.s, H.d_partial, (int)nparts, H.nrvars, H.L(finest).count, errortype,
                                             H.d_norm, H.d_nonfinite));
  if (r || !to_host) return r;
  cudaError_t ce = cudaMemcpyAsync(H.h_norm, H.d_norm, 2 * sizeof(double), cudaMemcpyDeviceToHost, H.s);
  if (ce != cudaSuccess) return cuda_fail(ce, "cudaMemcpyAsync(norm)");
  ce = cudaMemcpyAsync(H.h_nonfinite, H.d_nonfinite, sizeof(int), cudaMemcpyDeviceToHost, H.s);
  if (ce != cudaSuccess) return cuda_fail(ce, "cudaMemcpyAsync(nonfinite)");
  return BSAMG_OK;
}

int bx_resid(Hier& H, int finest, int errortype, bool to_host = true) {
  BoxLev& L = B(H, finest);
  Launch sh = shape(L.n[0], L.n[1], L.n[2]);
  BX_LAUNCH(H, sh, k_bx_resid, H.fpool, L, H.b_oqlo, H.b_ofhi, H.b_oflo, H.d_partial);
  return bx_finish(H, finest, ctas(sh), errortype, to_host);
}

int bx_cycle(Hier& H, int finest, int minlevel, int nsmooth, int errortype, bool to_host = true) {
  int r = bx_vcycle(H, finest, minlevel, nsmooth, true);
  if (r) return r;
  BoxLev& L = B(H, finest);
  if (H.ndims == 3 && L.n[1] % 2 == 0) {  // two rows per thread
    Launch sh = shape(L.n[0], L.n[1] / 2, L.n[2]);
    k_bx_track_update<3, 2><<<sh.g, sh.b, 0, H.s>>>(H.fpool, L, H.b_oqlo, H.d_partial);
    if ((r = after_launch(H, 1))) return r;
    return bx_finish(H, finest, ctas(sh), errortype, to_host);
  }
  Launch sh = shape(L.n[0], L.n[1], L.n[2]);
  BX_LAUNCH(H, sh, k_bx_track_update, H.fpool, L, H.b_oqlo, H.d_partial);
  return bx_finish(H, finest, ctas(sh), errortype, to_host);
}

// ---------------------------------------------------------------------------
// The solve as one graph launch.  MultigridIterations' loop (afasroutines.f90:
// 81-107) with this path's exit test runs on the device: a WHILE node whose
// body is one cycle (V-cycle, tracked-residual update, norm) and a decision
// kernel, followed by an IF node that evaluates the true residual when the
// decision asks for it.  The host enqueues the loop and reads the control
// block once, instead of waiting for every cycle's norm.

constexpr int kLoopMaxCycles = 64;
struct BoxCtl {
  double tol, r_sync;
  int maxv, it, conv, status, nconfirm, pad;
  double res[kLoopMaxCycles];
};
constexpr int kCtlSlotOffset = 16;  // doubles into the hierarchy's pinned slot
static_assert(sizeof(BoxCtl) <= (128 - kCtlSlotOffset) * sizeof(double), "pinned slot too small");

// after a cycle: the tracked norm decides whether to confirm on the true
// residual (the host loop's test: below the tolerance, 1e5 below the last
// true residual, or the last cycle)
__global__ void k_bx_decide_cycle(BoxCtl* c, const double* __restrict__ norm, const int* __restrict__ nonfinite,
                                  cudaGraphConditionalHandle hw, cudaGraphConditionalHandle hi) {
  int it = ++c->it;
  if (c->status || nonfinite[0]) {
    c->status = 1;
    cudaGraphSetConditional(hi, 0);
    cudaGraphSetConditional(hw, 0);
    return;
  }
  double tracked = norm[0];
  bool confirm = tracked < c->tol || tracked < 1e-5 * c->r_sync || it >= c->maxv;
  cudaGraphSetConditional(hi, confirm ? 1u : 0u);
  if (!confirm) c->res[it - 1] = tracked;
}

// after a true residual: converged or the last cycle ends the loop
__global__ void k_bx_decide_true(BoxCtl* c, const double* __restrict__ norm, const int* __restrict__ nonfinite,
                                 cudaGraphConditionalHandle hw) {
  int it = c->it;
  c->nconfirm++;
  if (nonfinite[0]) {
    c->status = 1;
    cudaGraphSetConditional(hw, 0);
    return;
  }
  double res = norm[0];
  c->r_sync = res;
  c->res[it - 1] = res;
  if (res < c->tol) {
    c->conv = 1;
    cudaGraphSetConditional(hw, 0);
  } else if (it >= c->maxv) {
    cudaGraphSetConditional(hw, 0);
  }
}

// capture what body() enqueues into graph g (a conditional node's body)
int capture_into(Hier& H, cudaGraph_t g, const std::function<int()>& body, long long* nlaunch) {
  cudaError_t e = cudaStreamBeginCaptureToGraph(H.s, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamBeginCaptureToGraph");
  H.capturing = true;
  H.capture_launches = 0;
  int r = body();
  H.capturing = false;
  *nlaunch = H.capture_launches;
  cudaGraph_t out = nullptr;
  e = cudaStreamEndCapture(H.s, &out);
  if (r) return r;
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
  return BSAMG_OK;
}

int box_loop_graph(Hier& H, int finest, int minlevel, int nsmooth, int errortype) {
  auto key = std::make_tuple(finest, minlevel, nsmooth, errortype);
  if (H.box_loop && H.box_loop_key == key) return BSAMG_OK;
  if (H.box_loop) cudaGraphExecDestroy(H.box_loop);
  H.box_loop = nullptr;
  if (!H.box_ctl) {
    cudaError_t e = dev_alloc(H, &H.box_ctl, sizeof(BoxCtl));
    if (e != cudaSuccess) return cuda_fail(e, "device allocation (loop control)");
  }
  BoxCtl* ctl = static_cast<BoxCtl*>(H.box_ctl);
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaGraphCreate(&g, 0);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGraphCreate");
  int r = BSAMG_OK;
  cudaGraphConditionalHandle hw, hi;
  cudaGraphNodeParams wp = {}, ip = {};
  cudaGraphNode_t wn = nullptr;
  do {
    if ((e = cudaGraphConditionalHandleCreate(&hw, g, 1, cudaGraphCondAssignDefault)) != cudaSuccess) break;
    if ((e = cudaGraphConditionalHandleCreate(&hi, g, 0, cudaGraphCondAssignDefault)) != cudaSuccess) break;
    wp.type = cudaGraphNodeTypeConditional;
    wp.conditional.handle = hw;
    wp.conditional.type = cudaGraphCondTypeWhile;
    wp.conditional.size = 1;
    if ((e = cudaGraphAddNode(&wn, g, nullptr, nullptr, 0, &wp)) != cudaSuccess) break;
    cudaGraph_t body = wp.conditional.phGraph_out[0];
    // the cycle, its decision, then the IF node on what was captured
    r = capture_into(H, body, [&]() -> int {
      int rr = bx_cycle(H, finest, minlevel, nsmooth, errortype, false);
      if (rr) return rr;
      k_bx_decide_cycle<<<1, 1, 0, H.s>>>(ctl, H.d_norm, H.d_nonfinite, hw, hi);
      if ((rr = after_launch(H, 1))) return rr;
      cudaStreamCaptureStatus st;
      cudaGraph_t cg = nullptr;
      const cudaGraphNode_t* deps = nullptr;
      size_t nd = 0;
      cudaError_t ce = cudaStreamGetCaptureInfo(H.s, &st, nullptr, &cg, &deps, nullptr, &nd);
      if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamGetCaptureInfo");
      ip.type = cudaGraphNodeTypeConditional;
      ip.conditional.handle = hi;
      ip.conditional.type = cudaGraphCondTypeIf;
      ip.conditional.size = 1;
      cudaGraphNode_t in = nullptr;
      ce = cudaGraphAddNode(&in, cg, deps, nullptr, nd, &ip);
      if (ce != cudaSuccess) return cuda_fail(ce, "cudaGraphAddNode(if)");
      ce = cudaStreamUpdateCaptureDependencies(H.s, &in, nullptr, 1, cudaStreamSetCaptureDependencies);
      if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamUpdateCaptureDependencies");
      return BSAMG_OK;
    }, &H.box_loop_n1);
    if (r) break;
    r = capture_into(H, ip.conditional.phGraph_out[0], [&]() -> int {
      int rr = bx_resid(H, finest, errortype, false);
      if (rr) return rr;
      k_bx_decide_true<<<1, 1, 0, H.s>>>(ctl, H.d_norm, H.d_nonfinite, hw);
      return after_launch(H, 1);
    }, &H.box_loop_n2);
    if (r) break;
    e = cudaGraphInstantiate(&H.box_loop, g, 0);
  } while (0);
  cudaGraphDestroy(g);
  if (r) return r;
  if (e != cudaSuccess) {
    cudaGetLastError();
    H.box_loop = nullptr;
    return cuda_fail(e, "conditional solve graph");
  }
  H.box_loop_key = key;
  return BSAMG_OK;
}

}  // namespace

bool box_eligible(const Hier& H, bool periodic_single) {
  // the box path's split/merge address q with one ghost layer
  // the box kernels carry CH's equations: only a plugin that declares the
  // box path (CH) takes it
  const Plugin* pl = find_plugin(H.problem);
  if (!pl || !pl->box || !periodic_single || H.mbc != 1) return false;
  for (int l = H.minlevel; l <= H.maxlevel; l++) {
    const HostPatch& P = H.patches[H.L(l).patches[0]];
    for (int d = 0; d < H.ndims; d++) {
      if (P.mx[d] % 2) return false;
      if (l > H.minlevel && P.mx[d] != 2 * H.patches[P.parent].mx[d]) return false;
    }
    // cell indices (both colours) are 32-bit
    if ((long long)P.mx[0] * P.mx[1] * P.mx[2] >= (1LL << 31)) return false;
  }
  return true;
}

// float pool of the box path: per level e, g, pb (not on the finest level,
// where pb is qhi(phi)), ec (below the finest); on the finest level qhi,
// qlo, fhi, flo
void box_coefficients(Hier& H) {
  for (int l = H.maxlevel; l >= H.minlevel; l--) {
    const HostPatch& P = H.patches[H.L(l).patches[0]];
    BoxLev& L = H.blev[l + kMaxDepth];
    double c[4];
    coefficients(H, P.dx[0], c);
    L.c0 = (float)c[0];
    L.c1 = (float)c[1];
    L.tmp3 = (float)c[2];
    L.a12 = (float)c[3];
    L.c0h = (float)c[0];
    L.c0l = (float)(c[0] - (double)L.c0h);
    L.c1h = (float)c[1];
    L.c1l = (float)(c[1] - (double)L.c1h);
    for (int x = 0; x < 4; x++) L.cd[x] = c[x];
  }
}

size_t box_layout(Hier& H) {
  if (cudaDeviceGetAttribute(&H.box_sms, cudaDevAttrMultiProcessorCount, H.ctx->device) != cudaSuccess ||
      H.box_sms <= 0)
    H.box_sms = 1;
  long long o = 0;
  auto al = [](long long x) { return (x + 63) & ~63LL; };
  for (int l = H.maxlevel; l >= H.minlevel; l--) {
    const HostPatch& P = H.patches[H.L(l).patches[0]];
    BoxLev& L = H.blev[l + kMaxDepth];
    for (int d = 0; d < 3; d++) L.n[d] = P.mx[d];
    L.hh = P.mx[0] / 2;
    L.half = (long long)P.mx[0] * P.mx[1] * P.mx[2] / 2;
    L.oe = o; o = al(o + 4 * L.half);
    L.og = o; o = al(o + 4 * L.half);
    if (l == H.maxlevel) {
      L.opb = o; o = al(o + 4 * L.half);    // qhi (both variables)
      H.b_oqlo = o; o = al(o + 4 * L.half);
      H.b_ofhi = o; o = al(o + 2 * L.half);
      H.b_oflo = o; o = al(o + 2 * L.half);
      L.oec = -1;
    } else {
      L.opb = o; o = al(o + 2 * L.half);
      L.oec = o; o = al(o + 4 * L.half);
    }
    L.oe2 = -1;
    if (l > H.minlevel && smooth_fits(H, L)) {  // the one-pass smoothing's output
      L.oe2 = o;
      o = al(o + 4 * L.half);
    }
  }
  box_coefficients(H);
  const BoxLev& F = H.blev[H.maxlevel + kMaxDepth];
  H.b_partials = (size_t)ctas(shape(F.n[0], F.n[1], F.n[2]));
  return (size_t)o;
}

int box_enq_relax(Hier& H, int level, int ipass) { return bx_relax(H, level, ipass - 1, 0); }

int box_smoother_colours(const Hier& H, int level) {
  return level > H.minlevel && smooth_applies(H, H.blev[level + kMaxDepth], 2) ? 4 : 1;
}

int box_enq_smoother(Hier& H, int level, int ipass) {
  if (box_smoother_colours(H, level) == 4) return bx_smooth(H, B(H, level), B(H, level).oe2, false);
  return bx_relax(H, level, ipass - 1, 0);
}

int box_iterations(Hier& H, int finest, int minlevel, int nsmooth, int maxvcycles, double tol, int errortype,
                   int strict, int* ncycles, double* residuals) {
  if (finest != H.maxlevel || minlevel < H.minlevel) return BSAMG_ERR_UNSUPPORTED;
  const HostPatch& P = H.patches[H.L(finest).patches[0]];
  BoxLev& L = B(H, finest);
  Launch sh = shape(L.hh, L.n[1], L.n[2]);
  bool warm = H.box_g_valid;  // g is the residual at this q: update it for the new f
  H.box_g_valid = false;
  // the whole solve as one graph launch when the loop fits its control block
  bool loop = maxvcycles >= 1 && maxvcycles <= kLoopMaxCycles && !H.box_loop_off;
  if (loop) {
    int rl = box_loop_graph(H, finest, minlevel, nsmooth, errortype);
    if (rl == BSAMG_ERR_CUDA && !H.box_loop) {
      H.box_loop_off = true;  // conditional graphs unavailable: the host loop below
      loop = false;
    } else if (rl) {
      return rl;
    }
  }
  int r;
  if (warm) {
    BX_LAUNCH(H, sh, k_bx_split_warm, H.pool, P.oq, P.oqold, P.sq, P.qn[0], P.qn[1], H.fpool, L, H.b_oqlo, H.b_ofhi,
              H.b_oflo, H.d_partial);
    r = bx_finish(H, finest, ctas(sh), errortype, !loop);
  } else {
    BX_LAUNCH(H, sh, k_bx_split, H.pool, P.oq, P.oqold, P.sq, P.qn[0], P.qn[1], H.fpool, L, H.b_oqlo, H.b_ofhi,
              H.b_oflo);
    r = bx_resid(H, finest, errortype, !loop);
  }
  if (r) return r;
  bool conv = false;
  int it = 0;
  if (loop) {
    // control block: the tolerance and cycle limit from the host, the
    // starting residual and its finiteness from the device
    BoxCtl* hc = reinterpret_cast<BoxCtl*>(H.h_norm + kCtlSlotOffset);
    BoxCtl* dc = static_cast<BoxCtl*>(H.box_ctl);
    hc->tol = tol;
    hc->maxv = maxvcycles;
    hc->it = hc->conv = hc->status = hc->nconfirm = 0;
    cudaError_t ce = cudaMemcpyAsync(dc, hc, offsetof(BoxCtl, res), cudaMemcpyHostToDevice, H.s);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(&dc->r_sync, H.d_norm, sizeof(double), cudaMemcpyDeviceToDevice, H.s);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(&dc->status, H.d_nonfinite, sizeof(int), cudaMemcpyDeviceToDevice, H.s);
    if (ce == cudaSuccess) ce = cudaGraphLaunch(H.box_loop, H.s);
    if (ce != cudaSuccess) return cuda_fail(ce, "solve graph");
    // leave the state as the FP64 path leaves it (see below), then read
    // the control block once
    BX_LAUNCH(H, sh, k_bx_merge, H.pool, P.oq, P.sq, P.qn[0], P.qn[1], H.fpool, L, H.b_oqlo);
    if ((r = enq_set_ghost(H, finest, 0))) return r;
    if ((r = enq_fill_down(H, 2, finest, minlevel))) return r;
    ce = cudaMemcpyAsync(hc, dc, sizeof(BoxCtl), cudaMemcpyDeviceToHost, H.s);
    if (ce != cudaSuccess) return cuda_fail(ce, "cudaMemcpyAsync(loop control)");
    if (int rw = stream_wait(H)) return rw;
    H.launches += hc->it * H.box_loop_n1 + hc->nconfirm * H.box_loop_n2;
    if (hc->status) return BSAMG_ERR_NONFINITE;
    it = hc->it;
    conv = hc->conv != 0;
    if (residuals)
      for (int n = 0; n < it; n++) residuals[n] = hc->res[n];
    if (ncycles) *ncycles = conv ? it : maxvcycles;
    H.box_g_valid = true;
    if (!conv && strict) return BSAMG_ERR_NOT_CONVERGED;
    return BSAMG_OK;
  }
  if (int rw = stream_wait(H)) return rw;
  if (*H.h_nonfinite) return BSAMG_ERR_NONFINITE;
  double r_sync = H.h_norm[0];
  Hier::GraphRec *gc = nullptr, *gv = nullptr;
  auto key = [&](int m) { return std::make_tuple(m, finest, minlevel, nsmooth, errortype); };
  if ((r = capture_graph(H, key(21), [&] { return bx_cycle(H, finest, minlevel, nsmooth, errortype); }, &gc)))
    return r;
  if ((r = capture_graph(H, key(22), [&] { return bx_resid(H, finest, errortype); }, &gv))) return r;
  for (it = 1; it <= maxvcycles; it++) {
    if ((r = replay(H, gc))) return r;
    if (*H.h_nonfinite) return BSAMG_ERR_NONFINITE;
    double tracked = H.h_norm[0], res = tracked;
    // confirm on the true residual when the tracked one says converged, on
    // the last cycle, and once the tracked value is 1e5 below the residual
    // it started from (where FP32 rounding of g - M(e) stops being negligible)
    if (tracked < tol || tracked < 1e-5 * r_sync || it == maxvcycles) {
      if ((r = replay(H, gv))) return r;
      if (*H.h_nonfinite) return BSAMG_ERR_NONFINITE;
      res = H.h_norm[0];
      r_sync = res;
      if (residuals) residuals[it - 1] = res;
      if (res < tol) {
        conv = true;
        break;
      }
      continue;
    }
    if (residuals) residuals[it - 1] = res;
  }
  if (ncycles) *ncycles = conv ? it : maxvcycles;
  // leave the state as the FP64 path leaves it: q in FP64 with fresh ghosts
  // and the coarse levels restricted from the finest (FillDown,
  // afasroutines.f90:83)
  BX_LAUNCH(H, sh, k_bx_merge, H.pool, P.oq, P.sq, P.qn[0], P.qn[1], H.fpool, L, H.b_oqlo);
  if ((r = enq_set_ghost(H, finest, 0))) return r;
  if ((r = enq_fill_down(H, 2, finest, minlevel))) return r;
  // the loop ends on a true residual (converged, or the last cycle's check)
  H.box_g_valid = true;
  if (!conv && strict) return BSAMG_ERR_NOT_CONVERGED;
  return BSAMG_OK;
}

}  // namespace bsamg
