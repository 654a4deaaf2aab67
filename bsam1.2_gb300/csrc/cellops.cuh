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
