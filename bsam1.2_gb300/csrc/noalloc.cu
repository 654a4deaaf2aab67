// Convergence norm of one CH patch on caller-owned device buffers, with no
// allocation of any kind.
//
// Some callers cannot let a library call cudaMalloc: a host whose device
// memory is owned by its own allocator (a PyTorch caching allocator, a
// Fortran code with a fixed device-memory plan), or a serving loop that must
// not trigger the device-wide synchronisation cudaMalloc/cudaFree imply while
// other streams are busy.  This entry point computes ErrorAFAS
// (afasroutines.f90:113-233) of one CH patch from q and f the caller already
// has on the device and writes the norm to a device double the caller owns.
// Its only scratch -- one partial sum per block plus the final reduction's
// stage sums -- lives in a file-scope __device__ array of fixed size, so a
// patch may have at most BSAMG_NOALLOC_MAX_CELLS interior cells (256^3).
//
// The array exists once per device for the life of the process and every
// call on that device shares it: two calls whose kernels overlap on the GPU
// (different streams, no ordering between them) race on it.  Each call
// writes every partial it later reads, so nothing needs clearing between
// calls.  The first call on a device looks the array's device address up
// (cudaGetSymbolAddress, with that device current) and keeps it for the
// rest of the process; make that first call before any stream capture that
// includes this entry point.  The kept address does not survive
// cudaDeviceReset (the module is loaded again, possibly elsewhere): a host
// that resets a device must not call this entry point on it afterwards.
//
// Same arithmetic, block decomposition and final reduction as the
// hierarchy's norm (the partial kernel below is k_norm_partial's for one CH
// patch, built with --fmad=false like it, and the final sum is
// launch_norm_finish itself), so the two agree bit for bit.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/bsamg.h"
#include "hier.h"
#include "internal.h"
#include "launch.h"

namespace {

using namespace bsamg;

constexpr int kMaxBlocks = BSAMG_NOALLOC_MAX_CELLS / (kBlock * kNormGroup);

// [0, 2*kMaxBlocks): per-CTA partial sums of rf^2 (two variables);
// [2*kMaxBlocks, 2*kMaxBlocks + kNormOutLen): the final reduction's output
// and stage sums (launch_norm_finish's `out`)
__device__ __align__(256) double g_norm_scratch[2 * kMaxBlocks + kNormOutLen];

std::mutex g_mu;
constexpr int kMaxDevices = 256;
double* g_scratch_ptr[kMaxDevices] = {};

int scratch_on_current_device(double** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return BSAMG_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_norm_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_norm_scratch)");
    g_scratch_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_scratch_ptr[dev];
  return BSAMG_OK;
}

template <int DIM>
__device__ __forceinline__ double ulap(const double* a, long long c, long long sy, long long sz) {
  if (DIM == 2) return a[c + 1] + a[c - 1] + a[c + sy] + a[c - sy] - 4.0 * a[c];
  return a[c + 1] + a[c - 1] + a[c + sy] + a[c - sy] + a[c + sz] + a[c - sz] - 6.0 * a[c];
}

// rf = f - Operator(q) (CH/problem.f90:393-422, :638-669) per interior cell,
// sums of rf^2 over kNormGroup consecutive runs of kBlock cells per CTA, in
// the order of the hierarchy's k_norm_partial on a one-patch level (whose
// work-list blocks are the same runs of cells)
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_norm_single(const double* __restrict__ q, const double* __restrict__ f,
                                                        int mx0, int mx1, int mx2, double c0, double c1,
                                                        double* __restrict__ partial) {
  __shared__ double red[2][kBlock / 32];
  double s0 = 0.0, s1 = 0.0;
  for (int sub = 0; sub < kNormGroup; sub++) {
    long long t = ((long long)blockIdx.x * kNormGroup + sub) * kBlock + threadIdx.x;
    int i = (int)(t % mx0) + 1, j, k;
    long long r = t / mx0;
    if (DIM == 2) {
      j = (int)r + 1;
      k = 1;
      if (j > mx1) break;
    } else {
      j = (int)(r % mx1) + 1;
      k = (int)(r / mx1) + 1;
      if (k > mx2) break;
    }
    long long n0 = mx0 + 2, n1 = mx1 + 2;
    long long sy = n0, sz = n0 * n1;
    long long sq = DIM == 2 ? n0 * n1 : n0 * n1 * (mx2 + 2);
    long long sf = (long long)mx0 * mx1 * (DIM == 2 ? 1 : mx2);
    long long c = DIM == 2 ? (long long)j * n0 + i : ((long long)k * n1 + j) * n0 + i;
    long long fc = DIM == 2 ? (long long)(j - 1) * mx0 + (i - 1) : ((long long)(k - 1) * mx1 + (j - 1)) * mx0 + (i - 1);
    const double* a0 = q;
    const double* a1 = q + sq;
    double r0 = a0[c] - c0 * ulap<DIM>(a1, c, sy, sz);
    double r1 = a1[c] - a0[c] * a0[c] * a0[c] + c1 * ulap<DIM>(a0, c, sy, sz);
    double e0 = f[fc] - r0;
    double e1 = f[sf + fc] - r1;
    s0 = s0 + e0 * e0;
    s1 = s1 + e1 * e1;
  }
  for (int o = 16; o > 0; o >>= 1) {
    s0 = s0 + __shfl_down_sync(0xffffffffu, s0, o);
    s1 = s1 + __shfl_down_sync(0xffffffffu, s1, o);
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
      t0 = t0 + red[0][n];
      t1 = t1 + red[1][n];
    }
    partial[2 * blockIdx.x] = t0;
    partial[2 * blockIdx.x + 1] = t1;
  }
}

}  // namespace

extern "C" int bsamg_ch_residual_norm_noalloc(const double* q, const double* f, int ndims, const int mx[3],
                                              double h, double dt, double eps, int errortype, double* norm_out,
                                              void* stream) {
  if (!q || !f || !mx || !norm_out || (ndims != 2 && ndims != 3) || (errortype != 1 && errortype != 2) ||
      !(h > 0.0))
    return BSAMG_ERR_ARG;
  long long cells = 1;
  for (int d = 0; d < ndims; d++) {
    if (mx[d] < 1) return BSAMG_ERR_ARG;
    cells *= mx[d];
  }
  if (cells > BSAMG_NOALLOC_MAX_CELLS) {
    cuda_fail(cudaSuccess, "bsamg_ch_residual_norm_noalloc: patch larger than BSAMG_NOALLOC_MAX_CELLS");
    return BSAMG_ERR_ARG;
  }
  double* scratch = nullptr;
  int rc = scratch_on_current_device(&scratch);
  if (rc != BSAMG_OK) return rc;
  // plugin coefficients exactly as the hierarchy computes them
  double h2 = h * h;
  double eps2 = eps * eps;
  double c0 = dt / h2, c1 = eps2 / h2;
  int nblk = norm_partials((int)((cells + kBlock - 1) / kBlock));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (ndims == 2)
    k_norm_single<2><<<nblk, kBlock, 0, s>>>(q, f, mx[0], mx[1], 1, c0, c1, scratch);
  else
    k_norm_single<3><<<nblk, kBlock, 0, s>>>(q, f, mx[0], mx[1], mx[2], c0, c1, scratch);
  // the hierarchy's own final reduction (two stages above 2048 blocks);
  // no non-finite flag: a NaN or Inf input shows as a NaN or Inf norm
  double* out = scratch + 2 * kMaxBlocks;
  launch_norm_finish(s, scratch, nblk, 2, 2.0 * (double)cells, errortype, out, nullptr);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "bsamg_ch_residual_norm_noalloc launch");
  e = cudaMemcpyAsync(norm_out, out, sizeof(double), cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) return cuda_fail(e, "bsamg_ch_residual_norm_noalloc copy");
  return BSAMG_OK;
}
