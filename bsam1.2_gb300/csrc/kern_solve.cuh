// The mixed-precision solve of an adaptive hierarchy in one launch of one
// thread-block cluster (included by kern_mixed.cuh; templates over the
// plugin struct).
//
// On an adaptive mesh every level is small (a few thousand cells on patches
// of 8-64 cells per side) and a V-cycle is a chain of some 300 dependent
// operations: colour sweeps, ghost programs, restriction, the FAS loading,
// prolongation.  As separate launches each costs a launch and a drain of the
// whole GPU for microseconds of work.  Here the host records the solve once
// per mesh as a program of phases over the same device work lists, and one
// cluster of up to 16 CTAs executes it: every phase is spread over all
// threads of the cluster and phases are separated by the cluster's hardware
// barrier (barrier.cluster arrive.release / wait.acquire, which orders the
// global-memory writes of one phase before the reads of the next for every
// thread of the cluster, about 0.25 us on GB300).  The coarse end of the
// V-cycle runs in CTA 0 alone, with CTA barriers, while the other CTAs wait.
// The loop of MultigridIterations (afasroutines.f90:78-104) runs on the
// device too: each outer iteration ends with the FP64 residual norm of the
// finest level, reduced in the same order as launch_norm_finish, and CTA 0
// records it and decides whether to stop (norm below the tolerance, a
// non-finite norm, or the last allowed V-cycle).  The host reads one control
// block after the launch.
//
// Every unit computes what the stand-alone kernel of the same operation
// computes, in the same order, so a solve gives bit for bit the iterates of
// the per-launch mixed path.  FP64 ghost programs and FillDown are written
// with explicitly rounded products and sums (this file is compiled with
// contraction on, the FP64 path's kernels without it).
#pragma once
#include <cuda_runtime.h>

namespace bsamg {
namespace mx {

__device__ __forceinline__ unsigned cluster_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ unsigned cluster_ctas() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
  return r;
}
// every thread of every CTA of the cluster; the release/acquire pair makes
// all memory writes before it visible to all threads of the cluster after it
__device__ __forceinline__ void cluster_barrier() {
  __syncwarp();  // the aligned forms want the warp converged
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// the 256 threads of group g of this CTA (hardware barrier 1 + g)
__device__ __forceinline__ void group_barrier(int g) { asm volatile("bar.sync %0, 256;" ::"r"(1 + g) : "memory"); }

// C/F interpolation weights, LIBRARY/boundary.f90:54-63
constexpr double dA1 = -01.0 / 05.0, dA2 = 02.0 / 03.0, dA3 = 08.0 / 15.0;
constexpr double dB1 = 05.0 / 32.0, dB2 = 15.0 / 16.0, dB3 = -03.0 / 32.0;
constexpr double dC1 = 09.0 / 16.0, dC2 = 03.0 / 16.0, dC3 = 03.0 / 16.0, dC4 = 01.0 / 16.0;

// An FP64 ghost operation (the FP64 path's ghost_apply), each product and
// sum rounded on its own in the same order.  The variable loop has the
// plugin's constant bound: a runtime index into pp.qpo would place the
// parameters in local memory, which every cluster barrier evicts from L1.
template <int NV>
__device__ __forceinline__ void s_ghost64(const PatchDev* __restrict__ P, double* pool, const GhostOp& g,
                                          const ProbParams& pp) {
  const PatchDev& d = P[g.dp];
  const PatchDev& s = P[g.sp];
#pragma unroll
  for (int v = 0; v < NV; v++) {
    double* dq = pool + d.oq + v * d.sq;
    const double* sq = pool + s.oq + v * s.sq;
    double val;
    switch (g.type) {
      case kGCopy: val = sq[g.s0]; break;
      case kGCopyAdd: val = __dadd_rn(sq[g.s0], pp.qpo[v]); break;
      case kGCopySub: val = __dsub_rn(sq[g.s0], pp.qpo[v]); break;
      case kGBC:
        val = ((g.mask >> v) & 1) ? __dsub_rn(2.0, sq[g.s0]) : (((g.mask >> (8 + v)) & 1) ? -sq[g.s0] : sq[g.s0]);
        break;
      case kGCfA:
        val = __dadd_rn(__dadd_rn(__dmul_rn(dA1, dq[g.s0]), __dmul_rn(dA2, dq[g.s1])), __dmul_rn(dA3, sq[g.c0]));
        break;
      case kGCfAB: {
        double c = __dadd_rn(__dadd_rn(__dmul_rn(dB1, sq[g.c0]), __dmul_rn(dB2, sq[g.c1])), __dmul_rn(dB3, sq[g.c2]));
        val = __dadd_rn(__dadd_rn(__dmul_rn(dA1, dq[g.s0]), __dmul_rn(dA2, dq[g.s1])), __dmul_rn(dA3, c));
        break;
      }
      default: {
        double c = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(dC1, sq[g.c0]), __dmul_rn(dC2, sq[g.c1])),
                                       __dmul_rn(dC3, sq[g.c2])),
                             __dmul_rn(dC4, sq[g.c3]));
        val = __dadd_rn(__dadd_rn(__dmul_rn(dA1, dq[g.s0]), __dmul_rn(dA2, dq[g.s1])), __dmul_rn(dA3, c));
        break;
      }
    }
    dq[g.dcell] = val;
  }
}

// FillDownLevel of q (afasroutines.f90:257-327, field 2): parent q(mb) =
// Restriction2D/3D (gridutilities.f90:103-126, :437-466) of the child's q,
// the sum left to right and then the product, as the FP64 path's kernel.
template <int DIM>
__device__ __forceinline__ void s_fill64(const PatchDev* __restrict__ P, double* pool, const Blk b, int tid,
                                         int nrvars) {
  const PatchDev& p = P[b.patch];
  int ci, cj, ck;
  if (!interior_cell<DIM>(p.cmx, b.start + tid, ci, cj, ck)) return;
  const PatchDev& par = P[p.parent];
  const int i = 2 * ci, j = 2 * cj, k = DIM == 3 ? 2 * ck : 0;
  for (int v = 0; v < nrvars; v++) {
    const double* q = pool + p.oq + v * p.sq;
    auto at = [&](int a, int b2, int c) { return q[gofs<DIM>(p.qn, a, b2, c)]; };
    double val;
    if (DIM == 2) {
      double s = __dadd_rn(__dadd_rn(__dadd_rn(at(i, j, 0), at(i - 1, j, 0)), at(i, j - 1, 0)), at(i - 1, j - 1, 0));
      val = __dmul_rn(0.25, s);
    } else {
      double s = at(i, j, k);
      s = __dadd_rn(s, at(i - 1, j, k));
      s = __dadd_rn(s, at(i, j - 1, k));
      s = __dadd_rn(s, at(i - 1, j - 1, k));
      s = __dadd_rn(s, at(i, j, k - 1));
      s = __dadd_rn(s, at(i - 1, j, k - 1));
      s = __dadd_rn(s, at(i, j - 1, k - 1));
      s = __dadd_rn(s, at(i - 1, j - 1, k - 1));
      val = __dmul_rn(0.125, s);
    }
    pool[par.oq + v * par.sq + gofs<DIM>(par.qn, p.mb[0] + ci - 1, p.mb[1] + cj - 1, DIM == 3 ? p.mb[2] + ck - 1 : 0)] =
        val;
  }
}

// the FP64 residual partial sums of k_mx_norm, by one group of 256 threads
// (group g of its CTA) for padded block group b
template <class PL, int DIM>
__device__ __forceinline__ void s_norm(const PatchDev* __restrict__ P, double* pool, const Blk* __restrict__ blk,
                                       int b, int u, int g, const ProbParams& pp, double* partial,
                                       double (*red)[kBlock / 32]) {
  constexpr int NV = PL::kNV;
  double s[NV];
  for (int v = 0; v < NV; v++) s[v] = 0.0;
  for (int sub = 0; sub < kNormCells; sub++) {
    const Blk bb = blk[b * kNormCells + sub];
    if (bb.patch < 0) break;
    const PatchDev& p = P[bb.patch];
    int i, j, k;
    if (!interior_cell<DIM>(p.mx, bb.start + u, i, j, k)) continue;
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
  int w = u >> 5, l = u & 31;
  if (l == 0)
    for (int v = 0; v < NV; v++) red[v][w] = s[v];
  group_barrier(g);
  if (u == 0)
    for (int v = 0; v < NV; v++) {
      double t = 0.0;
      for (int m = 0; m < kBlock / 32; m++) t += red[v][m];
      partial[NV * b + v] = t;
    }
  group_barrier(g);
}

// The final sum of launch_norm_finish (one stage: nb <= 2048 partials) by
// the T threads of one CTA: the 1024 threads of k_norm_finish are emulated,
// their shuffle trees replayed in shared memory on the lanes that reach
// lane 0, so the sum is the same bit for bit.  Thread 0 returns the norm.
template <int NV, int T>
__device__ __forceinline__ void s_finish(const double* partial, int nb, double (*tv)[1024], double (*r2)[32],
                                         double* sum_out, double* red0) {
  constexpr int kF = 1024;
  for (int vt = threadIdx.x; vt < kF; vt += T) {
    double a[NV][8];
    for (int v = 0; v < NV; v++)
      for (int u = 0; u < 8; u++) a[v][u] = 0.0;
    int n = vt;
    for (; n + 7 * kF < nb; n += 8 * kF)
      for (int u = 0; u < 8; u++)
        for (int v = 0; v < NV; v++) a[v][u] = a[v][u] + partial[NV * (n + u * kF) + v];
    for (; n < nb; n += kF)
      for (int v = 0; v < NV; v++) a[v][0] = a[v][0] + partial[NV * n + v];
    for (int v = 0; v < NV; v++)
      tv[v][vt] = ((a[v][0] + a[v][1]) + (a[v][2] + a[v][3])) + ((a[v][4] + a[v][5]) + (a[v][6] + a[v][7]));
  }
  __syncthreads();
  // t = t + shfl_down(t, o) within each warp of 32 emulated lanes: lanes
  // l < o are the ones whose values reach lane 0
  for (int o = 16; o > 0; o >>= 1) {
    for (int x = threadIdx.x; x < 32 * o; x += T) {
      int w = x / o, l = x - w * o;
      for (int v = 0; v < NV; v++) tv[v][w * 32 + l] = tv[v][w * 32 + l] + tv[v][w * 32 + l + o];
    }
    __syncthreads();
  }
  if (threadIdx.x < 32)
    for (int v = 0; v < NV; v++) r2[v][threadIdx.x] = tv[v][threadIdx.x * 32];
  __syncthreads();
  for (int o = 16; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int v = 0; v < NV; v++) r2[v][threadIdx.x] = r2[v][threadIdx.x] + r2[v][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double sum = r2[0][0];
    for (int v = 1; v < NV; v++) sum = sum + r2[v][0];
    *sum_out = sum;
    for (int v = 0; v < NV; v++) red0[v] = r2[v][0];
  }
}

template <class PL, int DIM, int T>
struct SolveRun {
  const PatchDev* __restrict__ P;
  double* pool;
  float* fpool;
  double* partial;
  ProbParams pp;
  MxParams mp;
  const Blk* bpool;   // the image's block pool (shared memory)
  const int* spool;   // the image's stage pool
  const int* ppool;   // the image's part pool
  float* sdata;       // this CTA's FP32 data area (shared memory)
  int lg;             // log2 of the units per tile of the FP32 work lists
  const GhostOp* sops;  // this CTA's FP32 ghost operations in shared memory, or null
  const GhostOp* gops;  // the same in global memory, from this CTA's segment on
  int rank, ctas;

  __device__ __forceinline__ void sync(bool cluster) const {
    if (cluster) cluster_barrier();
    else __syncthreads();
  }

  // the blocks of a partitioned list this CTA works on (all of them in a solo block)
  template <typename F>
  __device__ __forceinline__ void owned(const SolvePhase& f, bool cluster, F&& unit) const {
    const Blk* blk = bpool + f.blk;
    const int* pt = ppool + f.part;
    const int lo = cluster ? pt[rank] : pt[0], hi = cluster ? pt[rank + 1] : pt[ctas];
    const int u = threadIdx.x & ((1 << lg) - 1);
    for (int b = lo + (int)(threadIdx.x >> lg); b < hi; b += T >> lg) unit(blk[b], u);
  }

  // one phase by the threads t0 = 0 .. nt-1 of the scope (the cluster, or
  // this CTA alone)
  __device__ __forceinline__ void exec(const SolvePhase& f, int t0, int nt, bool cluster,
                                       double (*red)[PL::kNV][kBlock / 32]) const {
    constexpr int nr = PL::kNV;
    switch (f.op) {
      case kTRelax:
        owned(f, cluster, [&](const Blk& b, int u) { u_relax_any<PL, DIM, true>(P, fpool, b, u, f.arg, mp); });
        break;
      case kTRestrict:
        owned(f, cluster, [&](const Blk& b, int u) { u_restrict<DIM, true>(P, fpool, b, u, nr); });
        break;
      case kTRing:
        owned(f, cluster, [&](const Blk& b, int u) { u_coarse_ring<DIM, true>(P, fpool, b, u, nr, f.arg); });
        break;
      case kTLoad:
        owned(f, cluster, [&](const Blk& b, int u) { u_coarse_load<PL, DIM, true>(P, fpool, b, u, mp); });
        break;
      case kTProlong:
        owned(f, cluster, [&](const Blk& b, int u) { u_prolong<DIM, true>(P, fpool, b, u, nr); });
        break;
      case kSPrep:
        owned(f, cluster, [&](const Blk& b, int u) { u_prep<PL, DIM, true>(P, pool, fpool, b, u, f.arg, pp); });
        break;
      case kSUpdate:
        owned(f, cluster, [&](const Blk& b, int u) { u_update<DIM, true>(P, pool, fpool, b, u, nr, f.arg); });
        break;
      case kTGhost: {
        // stage s: this CTA's operations st[2*(s*ctas + r)] .. st[2*(s*ctas + r) + 1]
        // of its own list (inside a solo block CTA 0 holds every one)
        const int* st = spool + f.stage;
        for (int s = 0; s < f.nstages; s++) {
          const int lo = st[2 * (s * ctas + rank)], hi = st[2 * (s * ctas + rank) + 1];
          for (int t = lo + (int)threadIdx.x; t < hi; t += T) {
            const GhostOp g = sops ? sops[t] : gops[t];
            ghost32_apply<true>(P, fpool, g, nr);
          }
          if (s + 1 < f.nstages) sync(cluster);
        }
        break;
      }
      case kSGhost64: {
        const int* st = spool + f.stage;
        for (int s = 0; s < f.nstages; s++) {
          for (int t = st[s] + t0; t < st[s + 1]; t += nt) {
            const GhostOp g = f.ops[t];
            s_ghost64<PL::kNV>(P, pool, g, pp);
          }
          if (s + 1 < f.nstages) sync(cluster);
        }
        break;
      }
      case kSClear: {
        // the range of the FP32 pool, and this CTA's part of the e arrays
        // held in shared memory (offset, length) at part[2*rank]
        for (long long t = t0; t < f.len; t += nt) fpool[f.a + t] = 0.0f;
        if (f.part >= 0) {
          const int o = ppool[f.part + 2 * rank], n = ppool[f.part + 2 * rank + 1];
          for (int t = threadIdx.x; t < n; t += T) sdata[o + t] = 0.0f;
        }
        break;
      }
      case kSFill64: {
        const Blk* blk = bpool + f.blk;
        for (int b = t0 >> 8; b < f.n; b += nt >> 8) s_fill64<DIM>(P, pool, blk[b], t0 & 255, nr);
        break;
      }
      case kSNorm: {
        const Blk* blk = bpool + f.blk;
        const int g = threadIdx.x >> 8;
        for (int b = t0 >> 8; b < f.n; b += nt >> 8) s_norm<PL, DIM>(P, pool, blk, b, t0 & 255, g, pp, partial, red[g]);
        break;
      }
      default:
        break;
    }
  }
};

template <class PL, int DIM, int T>
__global__ void __launch_bounds__(T, 1)
    k_mx_solve(const unsigned char* __restrict__ img, SolveImage im, double* pool, float* fpool, SolveCtl* ctl,
               double* res, double* partial, ProbParams pp, MxParams mp) {
  constexpr int NV = PL::kNV;
  __shared__ double red[T / 256][NV][kBlock / 32];
  __shared__ double tv[NV][1024];
  __shared__ double r2[NV][32];
  // every CTA stages the read-only program image after its data area and
  // its ghost operations: phases, patch table, block, stage and part pools
  unsigned char* const simg = solve_smem + im.data + im.ops;
  for (int x = threadIdx.x; x < im.bytes / 16; x += T)
    reinterpret_cast<int4*>(simg)[x] = reinterpret_cast<const int4*>(img)[x];
  __syncthreads();
  const int rank = (int)cluster_rank(), ctas = (int)cluster_ctas();
  const int* seg = reinterpret_cast<const int*>(simg + im.off_part) + im.seg;
  const GhostOp* gops = ctl->ops + seg[rank];
  GhostOp* sops = nullptr;
  if (im.ops_smem) {  // this CTA's FP32 ghost operations, as words
    sops = reinterpret_cast<GhostOp*>(solve_smem + im.data);
    const int nw = (seg[rank + 1] - seg[rank]) * (int)(sizeof(GhostOp) / 4);
    for (int x = threadIdx.x; x < nw; x += T) reinterpret_cast<int*>(sops)[x] = reinterpret_cast<const int*>(gops)[x];
  }
  // the data areas of the other CTAs are written from the first phase on:
  // every CTA of the cluster is running before any of them starts
  cluster_barrier();
  const SolvePhase* ph = reinterpret_cast<const SolvePhase*>(simg);
  const SolveRun<PL, DIM, T> R{reinterpret_cast<const PatchDev*>(simg + im.off_patches),
                               pool,
                               fpool,
                               partial,
                               pp,
                               mp,
                               reinterpret_cast<const Blk*>(simg + im.off_blk),
                               reinterpret_cast<const int*>(simg + im.off_stage),
                               reinterpret_cast<const int*>(simg + im.off_part),
                               reinterpret_cast<float*>(solve_smem),
                               im.tile_log2,
                               sops,
                               gops,
                               rank,
                               ctas};
  const int nt = ctas * T, t0 = rank * T + (int)threadIdx.x;
  const int body = ctl->body, nph = ctl->nph, maxv = ctl->maxv, errortype = ctl->errortype;
  const double tol = ctl->tol, count = ctl->count;
  __shared__ int stop;  // set by thread 0 after each finish
  long long* trace = (rank == 0 && threadIdx.x == 0) ? ctl->trace : nullptr;
  if (trace) trace[nph] = clock64();
  for (int it = 0; it <= maxv; it++) {
    // it = 0: the prologue, phases [0, body); then the loop body once per V-cycle
    const int x0 = it == 0 ? 0 : body, x1 = it == 0 ? body : nph;
    for (int x = x0; x < x1; x++) {
      const SolvePhase f = ph[x];
      if (f.op == kSSolo) {
        if (rank == 0)
          for (int y = x + 1; y <= x + f.n; y++) {
            R.exec(ph[y], threadIdx.x, T, false, red);
            __syncthreads();
          }
        x += f.n;
        cluster_barrier();
        if (trace && it <= 1) trace[x] = clock64();
        continue;
      }
      if (f.op == kSFinish) {
        // every CTA sums the partials in the same order and takes the same
        // decision; CTA 0 records it
        double sum, comp[NV];
        s_finish<NV, T>(partial, f.n, tv, r2, &sum, comp);
        if (threadIdx.x == 0) {
          double r;
          if (errortype == 1) {
            r = sqrt(sum / count);  // ErrorAFAS, afasroutines.f90:135
          } else {
            double cells = count / NV;
            r = sqrt(comp[0] / cells);
            for (int v = 1; v < NV; v++) {  // MAXVAL of the component errors, :146-153
              double e = sqrt(comp[v] / cells);
              r = e > r ? e : r;
            }
          }
          const bool nonfinite = !isfinite(r);
          const bool conv = !nonfinite && r < tol;
          stop = conv || nonfinite || it == maxv;
          if (rank == 0) {
            if (!nonfinite) res[it - 1] = r;
            ctl->norm[0] = r;
            ctl->norm[1] = sum;
            ctl->ncycles = it;
            ctl->converged = conv;
            ctl->nonfinite = nonfinite;
            ctl->stop = stop;
          }
        }
        __syncthreads();
      } else {
        R.exec(f, t0, nt, true, red);
      }
      if (f.bar) cluster_barrier();
      if (trace && it <= 1) trace[x] = clock64();
    }
    if (it > 0 && stop) break;
  }
}

}  // namespace mx
}  // namespace bsamg
