// Test-only kernel: div2_rn (one reciprocal, Markstein-corrected quotients;
// cellops.cuh) against the IEEE division `/`, bit for bit, over seeded
// random operand pairs drawn the way the CH smoother's operands fall
// (denominator det >= 1, numerators of either sign over a wide exponent
// range) and over a table of edge cases.  Built and run by
// tests/test_div_gpu.py.
#include <cstdint>

#include "cellops.cuh"

namespace {

__device__ __forceinline__ unsigned long long splitmix(unsigned long long x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// a double with the given sign, unbiased exponent and 52 mantissa bits
__device__ __forceinline__ double make(unsigned long long sign, int e, unsigned long long mant) {
  return __longlong_as_double((long long)((sign << 63) | ((unsigned long long)(e + 1023) << 52) |
                                          (mant & 0xFFFFFFFFFFFFFull)));
}

__device__ void check(double a0, double a1, double b, unsigned long long* bad, double* first) {
  double q0, q1;
  bsamg::div2_rn(a0, a1, b, q0, q1);
  double r0 = a0 / b, r1 = a1 / b;
  bool ok = __double_as_longlong(q0) == __double_as_longlong(r0) &&
            __double_as_longlong(q1) == __double_as_longlong(r1);
  if (!ok) {
    if (atomicAdd(bad, 1ull) == 0) {
      first[0] = a0;
      first[1] = a1;
      first[2] = b;
    }
  }
}

__global__ void k_random(unsigned long long n, unsigned long long seed, unsigned long long* bad, double* first) {
  for (unsigned long long t = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; t < n;
       t += (unsigned long long)gridDim.x * blockDim.x) {
    unsigned long long u = splitmix(seed ^ (t * 0xD1B54A32D192ED03ull));
    unsigned long long v = splitmix(u), w = splitmix(v), z = splitmix(w);
    // denominator in [1, 2^40): random exponent and mantissa, a quarter of
    // them with a mantissa of all ones or all zeros in its low 20 bits
    int eb = (int)(u % 41);
    unsigned long long mb = v;
    if ((u >> 40) % 4 == 0) mb = (u >> 45) & 1 ? (mb | 0xFFFFFull) : (mb & ~0xFFFFFull);
    double b = make(0, eb, mb);
    // numerators: either sign, exponents over [-120, 120], a tenth of them
    // exact multiples of b
    int ea0 = (int)((w >> 8) % 241) - 120, ea1 = (int)((z >> 8) % 241) - 120;
    double a0 = make(w >> 63, ea0, z);
    double a1 = make(z >> 63, ea1, w ^ v);
    if ((w % 10) == 0) a0 = b * (double)((long long)(z % 2001) - 1000);
    check(a0, a1, b, bad, first);
  }
}

__global__ void k_table(const double* a, int na, const double* b, int nb, unsigned long long* bad, double* first) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= na * nb) return;
  check(a[t % na], a[(t / 7) % na], b[t / na], bad, first);
}

}  // namespace

extern "C" int div_check_random(unsigned long long n, unsigned long long seed, unsigned long long* bad_host,
                                double* first_host) {
  unsigned long long* bad;
  double* first;
  if (cudaMalloc(&bad, 8) != cudaSuccess || cudaMalloc(&first, 24) != cudaSuccess) return -1;
  cudaMemset(bad, 0, 8);
  k_random<<<152 * 16, 256>>>(n, seed, bad, first);
  cudaError_t e = cudaDeviceSynchronize();
  cudaMemcpy(bad_host, bad, 8, cudaMemcpyDeviceToHost);
  cudaMemcpy(first_host, first, 24, cudaMemcpyDeviceToHost);
  cudaFree(bad);
  cudaFree(first);
  return e == cudaSuccess ? 0 : -2;
}

extern "C" int div_check_table(const double* a_host, int na, const double* b_host, int nb,
                               unsigned long long* bad_host, double* first_host) {
  unsigned long long* bad;
  double *first, *a, *b;
  if (cudaMalloc(&bad, 8) != cudaSuccess || cudaMalloc(&first, 24) != cudaSuccess ||
      cudaMalloc(&a, 8 * na) != cudaSuccess || cudaMalloc(&b, 8 * nb) != cudaSuccess)
    return -1;
  cudaMemset(bad, 0, 8);
  cudaMemcpy(a, a_host, 8 * na, cudaMemcpyHostToDevice);
  cudaMemcpy(b, b_host, 8 * nb, cudaMemcpyHostToDevice);
  int n = na * nb;
  k_table<<<(n + 255) / 256, 256>>>(a, na, b, nb, bad, first);
  cudaError_t e = cudaDeviceSynchronize();
  cudaMemcpy(bad_host, bad, 8, cudaMemcpyDeviceToHost);
  cudaMemcpy(first_host, first, 24, cudaMemcpyDeviceToHost);
  cudaFree(bad);
  cudaFree(first);
  cudaFree(a);
  cudaFree(b);
  return e == cudaSuccess ? 0 : -2;
}
