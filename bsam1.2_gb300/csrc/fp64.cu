// Plain FP64 kernels: the drop-in path.  This file holds the kernels that do
// not depend on the problem plugin (restriction, coarse rings, CorrectFine,
// FillDown, UpdateSourceFunction, the final norm reduction, ghost programs)
// and the launchers, which reach the plugin-dependent kernels (relaxation,
// coarse loading, residual, source, coarse tails) through the plugin
// registry (plugin.h).
//
// This translation unit is compiled with --fmad=false, like the FP64 part
// of every plugin (see kern_fp64.cuh).
//
// On GB300 these kernels are bounded by the FP64 pipe, not by HBM: the CH
// smoother needs ~22 FP64 operations and 2 divisions per cell update against
// 32 bytes of algorithmic traffic, and the part issues FP64 at ~1.2 TFLOP/s.
#include <cuda_runtime.h>

#include <algorithm>

#include "kern_fp64.cuh"

namespace bsamg {

template <int DIM>
__global__ void __launch_bounds__(kBlock) k_restrict_q(const PatchDev* __restrict__ P, double* __restrict__ pool,
                                                       const Blk* __restrict__ blk, int nrvars) {
  u_restrict_q<DIM>(P, pool, blk[blockIdx.x], threadIdx.x, nrvars);
}


template <int DIM>
__global__ void __launch_bounds__(kBlock) k_coarse_ghost(const PatchDev* __restrict__ P, double* __restrict__ pool,
                                                         const Blk* __restrict__ blk, int nrvars) {
  u_coarse_ghost<DIM>(P, pool, blk[blockIdx.x], threadIdx.x, nrvars);
}


template <int DIM>
__global__ void __launch_bounds__(kBlock) k_correct_a(const PatchDev* __restrict__ P, double* __restrict__ pool,
                                                      const Blk* __restrict__ blk, int nrvars) {
  u_correct_a<DIM>(P, pool, blk[blockIdx.x], threadIdx.x, nrvars);
}

// InitFields' first statement (bsamroutines.f90:1815-1818, :1834-1837):
// child qc(1-mbc:cmx+mbc) = parent%q(mb-mbc:mb+mbc), on a new patch
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_qc_from_parent(const PatchDev* __restrict__ P, double* __restrict__ pool,
                                                           const Blk* __restrict__ blk, int nrvars) {
  const Blk b = blk[blockIdx.x];
  const PatchDev& p = P[b.patch];
  int i, j, k;
  if (!ghosted_cell<DIM>(p.cn, p.gs, b.start + threadIdx.x, i, j, k)) return;
  const PatchDev& par = P[p.parent];
  long long src = gofs<DIM>(par.qn, p.mb[0] - 1 + i, p.mb[1] - 1 + j, DIM == 3 ? p.mb[2] - 1 + k : 0);
  long long dst = gofs<DIM>(p.cn, i, j, k);
  for (int v = 0; v < nrvars; v++) pool[p.oqc + v * p.sc + dst] = pool[par.oq + v * par.sq + src];
}


template <int DIM>
__global__ void __launch_bounds__(kBlock) k_correct_b(const PatchDev* __restrict__ P, double* __restrict__ pool,
                                                      const Blk* __restrict__ blk, int nrvars) {
  u_correct_b<DIM>(P, pool, blk[blockIdx.x], threadIdx.x, nrvars);
}

template <int DIM>
__global__ void __launch_bounds__(kBlock) k_fill_down(const PatchDev* __restrict__ P, double* __restrict__ pool,
                                                      const Blk* __restrict__ blk, int nrvars, int field) {
  u_fill_down<DIM>(P, pool, blk[blockIdx.x], threadIdx.x, nrvars, field);
}


// Final deterministic reduction of the block partials in block order.
// First stage of a long final sum: CTA g adds the partial pairs
// [g*chunk, min((g+1)*chunk, nblk)) in a fixed order and writes one pair to
// stage[2g], stage[2g+1].  Spreading the FP64 additions over many SMs
// matters on GB300, whose FP64 rate is two additions per clock per SM.
constexpr int kStageBlocks = (kNormOutLen - 8) / 3;
template <int NV>
__global__ void __launch_bounds__(kBlock) k_norm_stage(const double* __restrict__ partial, int nblk, int chunk,
                                                       double* __restrict__ stage) {
  __shared__ double red[NV][kBlock];
  int lo = blockIdx.x * chunk, hi = min(lo + chunk, nblk);
  double a[NV];
  for (int v = 0; v < NV; v++) a[v] = 0.0;
  for (int n = lo + threadIdx.x; n < hi; n += kBlock)
    for (int v = 0; v < NV; v++) a[v] = a[v] + partial[NV * n + v];
  for (int v = 0; v < NV; v++) red[v][threadIdx.x] = a[v];
  __syncthreads();
  for (int w = kBlock / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int v = 0; v < NV; v++) red[v][threadIdx.x] = red[v][threadIdx.x] + red[v][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int v = 0; v < NV; v++) stage[NV * blockIdx.x + v] = red[v][0];
}

// One CTA of 1024 threads; each thread keeps eight independent partial sums
// per variable so that eight loads are in flight, then a fixed-shape tree.
// The order of the additions depends only on nblk, so the result is
// deterministic.  Partials hold NV values per block.
constexpr int kFinishThreads = 1024;
template <int NV>
__global__ void __launch_bounds__(kFinishThreads) k_norm_finish(const double* __restrict__ partial, int nblk,
                                                                double count, int errortype, double* out,
                                                                int* nonfinite) {
  __shared__ double red[NV][kFinishThreads / 32];
  double a[NV][8];
  for (int v = 0; v < NV; v++)
    for (int u = 0; u < 8; u++) a[v][u] = 0.0;
  int n = threadIdx.x;
  for (; n + 7 * kFinishThreads < nblk; n += 8 * kFinishThreads)
    for (int u = 0; u < 8; u++)
      for (int v = 0; v < NV; v++) a[v][u] = a[v][u] + partial[NV * (n + u * kFinishThreads) + v];
  // the remaining (at most seven) partials of this thread; a constant index
  // keeps a[][] in registers
  for (; n < nblk; n += kFinishThreads)
    for (int v = 0; v < NV; v++) a[v][0] = a[v][0] + partial[NV * n + v];
  double t[NV];
  for (int v = 0; v < NV; v++)
    t[v] = ((a[v][0] + a[v][1]) + (a[v][2] + a[v][3])) + ((a[v][4] + a[v][5]) + (a[v][6] + a[v][7]));
  for (int o = 16; o > 0; o >>= 1)
    for (int v = 0; v < NV; v++) t[v] = t[v] + __shfl_down_sync(0xffffffffu, t[v], o);
  int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0)
    for (int v = 0; v < NV; v++) red[v][w] = t[v];
  __syncthreads();
  if (w == 0) {
    for (int v = 0; v < NV; v++) t[v] = red[v][threadIdx.x];
    for (int o = 16; o > 0; o >>= 1)
      for (int v = 0; v < NV; v++) t[v] = t[v] + __shfl_down_sync(0xffffffffu, t[v], o);
    if (threadIdx.x == 0)
      for (int v = 0; v < NV; v++) red[v][0] = t[v];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double sum = red[0][0];
    for (int v = 1; v < NV; v++) sum = sum + red[v][0];
    double r;
    if (errortype == 1) {
      r = sqrt(sum / count);  // integralresult(1)/integralresult(2), :135
    } else {
      double cells = count / NV;
      r = sqrt(red[0][0] / cells);
      for (int v = 1; v < NV; v++) {  // MAXVAL of component errors, :146-153
        double e = sqrt(red[v][0] / cells);
        r = e > r ? e : r;
      }
    }
    out[0] = r;
    out[1] = sum;
    if (nonfinite) nonfinite[0] = isfinite(r) ? 0 : 1;
  }
}

__global__ void __launch_bounds__(kBlock) k_ghost_stage(const PatchDev* __restrict__ P, double* __restrict__ pool,
                                                        const GhostOp* __restrict__ ops, int n, ProbParams pp) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  GhostOp g = ops[t];
  ghost_apply(P, pool, g, pp);
}

// whole program in one block: stages separated by __syncthreads
__global__ void __launch_bounds__(kBlock) k_ghost_program(const PatchDev* __restrict__ P, double* __restrict__ pool,
                                                          const GhostOp* __restrict__ ops,
                                                          const int* __restrict__ stage_off, int nstages,
                                                          ProbParams pp) {
  for (int s = 0; s < nstages; s++) {
    int lo = stage_off[s], hi = stage_off[s + 1];
    for (int t = lo + threadIdx.x; t < hi; t += blockDim.x) {
      GhostOp g = ops[t];
      ghost_apply(P, pool, g, pp);
    }
    __syncthreads();
  }
}

// The coarse tail of the V-cycle in one block (see TailPhase): the
// operations the separate launches would run, phase by phase, each phase's
// work-list blocks executed in turn by the block's 256 threads with a
// barrier between phases.  Per-cell arithmetic and the order of dependent
// ---------------------------------------------------------------------------
// launchers

#define DISPATCH_DIM(c, KER, ...)                            \
  do {                                                       \
    if ((c).ndims == 2) KER<2><<<nblk, kBlock, 0, (c).s>>>(__VA_ARGS__); \
    else KER<3><<<nblk, kBlock, 0, (c).s>>>(__VA_ARGS__);    \
  } while (0)

// the plugin's FP64 launchers; a hierarchy is created only for a registered
// plugin, so the lookup cannot fail here
static const PluginFp64& ops_of(const LaunchCtx& c) { return *find_plugin(c.pp.problem)->fp64; }

int launch_relax(const LaunchCtx& c, const Blk* blk, int nblk, int ipass) {
  return ops_of(c).relax(c, blk, nblk, ipass);
}
int launch_restrict_q(const LaunchCtx& c, const Blk* blk, int nblk) {
  if (nblk <= 0) return 0;
  DISPATCH_DIM(c, k_restrict_q, c.P, c.pool, blk, c.pp.nrvars);
  return 1;
}
int launch_coarse_ghost(const LaunchCtx& c, const Blk* blk, int nblk) {
  if (nblk <= 0) return 0;
  DISPATCH_DIM(c, k_coarse_ghost, c.P, c.pool, blk, c.pp.nrvars);
  return 1;
}
int launch_coarse_load(const LaunchCtx& c, const Blk* blk, int nblk) { return ops_of(c).coarse_load(c, blk, nblk); }
int launch_correct_a(const LaunchCtx& c, const Blk* blk, int nblk) {
  if (nblk <= 0) return 0;
  DISPATCH_DIM(c, k_correct_a, c.P, c.pool, blk, c.pp.nrvars);
  return 1;
}
int launch_qc_from_parent(const LaunchCtx& c, const Blk* blk, int nblk) {
  if (nblk <= 0) return 0;
  DISPATCH_DIM(c, k_qc_from_parent, c.P, c.pool, blk, c.pp.nrvars);
  return 1;
}
int launch_correct_b(const LaunchCtx& c, const Blk* blk, int nblk) {
  if (nblk <= 0) return 0;
  DISPATCH_DIM(c, k_correct_b, c.P, c.pool, blk, c.pp.nrvars);
  return 1;
}
int launch_fill_down(const LaunchCtx& c, const Blk* blk, int nblk, int field) {
  if (nblk <= 0) return 0;
  DISPATCH_DIM(c, k_fill_down, c.P, c.pool, blk, c.pp.nrvars, field);
  return 1;
}
int launch_get_source(const LaunchCtx& c, const Blk* blk, int nblk) { return ops_of(c).get_source(c, blk, nblk); }
int launch_update_source(const LaunchCtx& c, const Blk* blk, int nblk) {
  return ops_of(c).update_source(c, blk, nblk);
}
int launch_norm_partial(const LaunchCtx& c, const Blk* blk, int nblk, double* partial, int store_rf) {
  return ops_of(c).norm_partial(c, blk, nblk, partial, store_rf);
}
int launch_norm_finish(cudaStream_t s, const double* partial, int nblk, int nrvars, double count, int errortype,
                       double* out, int* nonfinite) {
  int n = 1;
  if (nblk > 2048) {
    // two stages; out[8 ..] holds the stage sums
    int g = std::min(kStageBlocks, (nblk + 511) / 512);
    int chunk = (nblk + g - 1) / g;
    g = (nblk + chunk - 1) / chunk;
    if (nrvars == 3) k_norm_stage<3><<<g, kBlock, 0, s>>>(partial, nblk, chunk, out + 8);
    else k_norm_stage<2><<<g, kBlock, 0, s>>>(partial, nblk, chunk, out + 8);
    partial = out + 8;
    nblk = g;
    n = 2;
  }
  if (nrvars == 3) k_norm_finish<3><<<1, kFinishThreads, 0, s>>>(partial, nblk, count, errortype, out, nonfinite);
  else k_norm_finish<2><<<1, kFinishThreads, 0, s>>>(partial, nblk, count, errortype, out, nonfinite);
  return n;
}
int launch_ghost_stage(const LaunchCtx& c, const GhostOp* ops, int n) {
  if (n <= 0) return 0;
  int nb = (n + kBlock - 1) / kBlock;
  k_ghost_stage<<<nb, kBlock, 0, c.s>>>(c.P, c.pool, ops, n, c.pp);
  return 1;
}
int launch_ghost_program_1cta(const LaunchCtx& c, const GhostOp* ops, const int* stage_off, int nstages) {
  if (nstages <= 0) return 0;
  k_ghost_program<<<1, kBlock, 0, c.s>>>(c.P, c.pool, ops, stage_off, nstages, c.pp);
  return 1;
}
int launch_tail(const LaunchCtx& c, const TailPhase* ph, int nph) { return ops_of(c).tail(c, ph, nph); }
int launch_tail_smem(const LaunchCtx& c, const PatchDev* shadow, const TailPhase* ph, int nph, const StageSeg* segs,
                     int nsegs, int smem_bytes) {
  return ops_of(c).tail_smem(c, shadow, ph, nph, segs, nsegs, smem_bytes);
}
int tail_smem_attributes(int problem) { return find_plugin(problem)->fp64->tail_smem_attributes(); }

}  // namespace bsamg
