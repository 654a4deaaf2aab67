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

#include "kern_mixed.cuh"
#include "box.h"
#include "mixed.h"

namespace bsamg {

namespace {

using namespace mx;

template <int DIM>
__global__ void __launch_bounds__(kBlock) k_mx_restrict(const PatchDev* __restrict__ P, float* __restrict__ fpool,
                                                        const Blk* __restrict__ blk, int nrvars) {
  u_restrict<DIM>(P, fpool, blk[blockIdx.x], threadIdx.x, nrvars);
}

template <int DIM>
__global__ void __launch_bounds__(kBlock) k_mx_coarse_ring(const PatchDev* __restrict__ P, float* __restrict__ fpool,
                                                           const Blk* __restrict__ blk, int nrvars, int corr) {
  u_coarse_ring<DIM>(P, fpool, blk[blockIdx.x], threadIdx.x, nrvars, corr);
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

// the plugin's correction-form launchers (a mixed hierarchy exists only for
// a plugin that has them) and their common arguments
const PluginMixed& mxp(const Hier& H) { return *find_plugin(H.problem)->mixed; }
MxLaunch mxl(const Hier& H) { return MxLaunch{H.s, H.ndims, H.dP, H.pool, H.fpool, H.pp}; }
bool has_mixed(const Hier& H) {
  const Plugin* p = find_plugin(H.problem);
  return p && p->mixed;
}

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
    case kTRelax: return after_launch(H, mxp(H).relax(mxl(H), L.d_blk[kind], L.nblk[kind], arg));
    case kTRestrict: MX_LAUNCH(H, kind, k_mx_restrict, H.dP, H.fpool, L.d_blk[kind], H.nrvars); break;
    case kTRing: MX_LAUNCH(H, kind, k_mx_coarse_ring, H.dP, H.fpool, L.d_blk[kind], H.nrvars, arg); break;
    case kTLoad: return after_launch(H, mxp(H).coarse_load(mxl(H), L.d_blk[kind], L.nblk[kind]));
    default: MX_LAUNCH(H, kind, k_mx_prolong, H.dP, H.fpool, L.d_blk[kind], H.nrvars); break;
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
      const PatchDev* table = T.smem_bytes ? static_cast<const PatchDev*>(T.shadow) : H.dP;
      return after_launch(H, mxp(H).tail(mxl(H), table, ph, T.nph, static_cast<const StageSeg*>(T.segs), T.nsegs,
                                         T.smem_bytes));
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
  long long nbase = mxp(H).nbase;
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
    // the kernels' shared-memory limit, per plugin, dimension and device
    static std::atomic<unsigned long long> attr[kMaxPlugins][2];
    int a = H.problem & (kMaxPlugins - 1), b = H.ndims - 2;
    if (needs_setup(attr[a][b], H.ctx->device)) {
      if (mxp(H).tail_smem_attributes(H.ndims)) return cuda_fail(cudaGetLastError(), "cudaFuncSetAttribute(tail)");
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
  // the plugin's base planes (CH: phib; growth: phib, nb, G, U)
  long long nbase = mxp(H).nbase;
  for (size_t p = 0; p < np; p++) { off[4 * p + 3] = o; o = al(o + nbase * H.patches[p].sf); }
  *total = (size_t)o;
  return off;
}

int mx_norm(Hier& H, int level, int errortype) {
  LevelT& L = H.L(level);
  int nb = (L.nblk[kKindInterior] + kNormCells - 1) / kNormCells;
  if (nb <= 0) return BSAMG_OK;
  // the interior list is padded with patch = -1 entries to a multiple of
  // kNormCells (see mixed_tables)
  int r = after_launch(H, mxp(H).norm(mxl(H), H.mx_norm_blk[level + kMaxDepth], nb, H.d_partial));
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
    // all levels below the root at once (base fields only)
    if ((r__ = after_launch(H, mxp(H).prep(mxl(H), blk, nb, mode)))) return r__;
    if (all_coarse) break;
  }
  int r = mx_vcycle(H, finest, minlevel, nsmooth);
  if (r) return r;
  // tracked residual g - M(e): M needs this cycle's base field, so it runs
  // before the update pass replaces phib with the new base
  {
    LevelT& L = H.L(finest);
    if ((r = after_launch(H, mxp(H).track(mxl(H), L.d_blk[kKindInterior], L.nblk[kKindInterior], H.d_partial))))
      return r;
    if ((r = after_launch(H, launch_norm_finish(H.s, H.d_partial, L.nblk[kKindInterior], H.nrvars, L.count,
                                                 errortype, H.d_norm, H.d_nonfinite))))
      return r;
  }
  for (int level = finest; level >= 0; level--) {
    LevelT& L = H.L(level);
    MX_LAUNCH(H, kKindFGhost, k_mx_update, H.dP, H.pool, H.fpool, L.d_blk[kKindFGhost], H.nrvars,
              mxp(H).nupdate);
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
  if (!has_mixed(H)) return 0;
  size_t n, ne, ec;
  layout(H, &n, &ne, &ec);
  return n * sizeof(float);
}

int mixed_alloc(Hier& H) {
  if (!has_mixed(H)) return BSAMG_OK;
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
  if (H.box_loop) cudaGraphExecDestroy(H.box_loop);
  H.box_loop = nullptr;
  if (H.box_ctl) cudaFreeAsync(H.box_ctl, H.s);
  H.box_ctl = nullptr;
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
  if (!has_mixed(H) || !H.fpool || H.box) return BSAMG_OK;
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
  if (!has_mixed(H) || !H.fpool) return BSAMG_ERR_UNSUPPORTED;
  if (H.box) return box_enq_relax(H, level, ipass);
  return mx_op(H, level, kKindColor, kTRelax, ipass);
}

int mixed_iterations(Hier& H, int finest, int minlevel, int nsmooth, int maxvcycles, double tol, int errortype,
                     int strict, int* ncycles, double* residuals) {
  if (!has_mixed(H) || !H.fpool) return BSAMG_ERR_UNSUPPORTED;
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
