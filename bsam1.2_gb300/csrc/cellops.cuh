// Cell addressing and the undivided Laplacian, shared by the kernels of both
// paths and by the plugins' device code.
#pragma once
#include "internal.h"

namespace bsamg {

// offset of Fortran cell (i,j,k) (lower bound 0) in a ghosted plane of
// extents n
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
template <int DIM, typename T>
__device__ __forceinline__ T ulap(const T* a, long long c, long long sy, long long sz) {
  if (DIM == 2) return a[c + 1] + a[c - 1] + a[c + sy] + a[c - sy] - T(4) * a[c];
  return a[c + 1] + a[c - 1] + a[c + sy] + a[c - sy] + a[c + sz] + a[c - sz] - T(6) * a[c];
}

// The quotients a0/b and a1/b, each bit-identical to the IEEE
// round-to-nearest division, from one correctly rounded reciprocal
// y = RN(1/b) (the __drcp_rn intrinsic): q = RN(a*y) is within one ulp of
// a/b, the remainder r = a - b*q is exact in one fused multiply-add, and
// RN(q + r*y) is the correctly rounded quotient (P. Markstein, "Computation
// of elementary functions on the IBM RISC System/6000 processor", IBM J.
// Res. Dev. 34(1), 1990).  The argument needs every intermediate in the
// normal range: the fast form is taken for 1 <= b < 2^400 and
// 2^-400 <= |a| < 2^400 (exponent tests on the integer pipe), and `/` for
// everything else (zeros, tiny or huge values, NaN and Inf).  A zero
// remainder returns q, which is then exact.  One reciprocal and three
// operations per quotient replace two full divisions; bit-identity with `/`
// is checked on the GPU over random and edge-case operands.
__device__ __forceinline__ bool mk_fast_num(double a) {
  unsigned e = ((unsigned)__double2hiint(a) >> 20) & 0x7ffu;
  return e - (1023u - 400u) <= 800u;
}
__device__ __forceinline__ bool mk_fast_den(double b) {
  return ((unsigned)__double2hiint(b) >> 20) - 1023u < 400u;  // sign bit set: huge, slow form
}
__device__ __forceinline__ double mk_quot(double a, double b, double y) {
  double q = __dmul_rn(a, y);
  double r = __fma_rn(-b, q, a);
  return (__double_as_longlong(r) << 1) ? __fma_rn(r, y, q) : q;
}
__device__ __forceinline__ void div2_rn(double a0, double a1, double b, double& q0, double& q1) {
  if (mk_fast_den(b) && mk_fast_num(a0) && mk_fast_num(a1)) {
    double y = __drcp_rn(b);
    q0 = mk_quot(a0, b, y);
    q1 = mk_quot(a1, b, y);
  } else {
    q0 = a0 / b;
    q1 = a1 / b;
  }
}

__device__ __forceinline__ double cube(double c) { return c * c * c; }  // CH/problem.f90:918
__device__ __forceinline__ double sqr(double c) { return c * c; }       // CH/problem.f90:931

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

// cell t of a ghosted array of extents n whose indices start at -gs
template <int DIM>
__device__ __forceinline__ bool ghosted_cell(const int* n, int gs, int t, int& i, int& j, int& k) {
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

}  // namespace bsamg
