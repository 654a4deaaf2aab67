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
#include <chrono>
#include <cstring>
#include <functional>
#include <map>
#include <mutex>
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

// step 3: qbar += e (whole ghosted array), base refresh, e = 0 (u_update)
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_mx_update(const PatchDev* __restrict__ P, double* __restrict__ pool,
                                                      float* __restrict__ fpool, const Blk* __restrict__ blk,
                                                      int nrvars, int nbase) {
  u_update<DIM>(P, pool, fpool, blk[blockIdx.x], threadIdx.x, nrvars, nbase);
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

// the one-launch solve's FP32 ghost operations in CTA order: out[i] =
// operation (ref & 0xfffff) of program (ref >> 20)
__global__ void __launch_bounds__(kBlock) k_gather_ops(const GhostOp* const* __restrict__ base,
                                                       const unsigned* __restrict__ ref, int n,
                                                       GhostOp* __restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  unsigned r = ref[i];
  out[i] = base[r >> 20][r & 0xfffffu];
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

// the smoothing of one level; on the V-cycle's coarsest level (coarse) in
// FP64 arithmetic
int mx_level_relax(Hier& H, int level, int nsmooth, bool coarse) {
  for (int pass = 1; pass <= nsmooth; pass++)
    for (int rb = 1; rb <= 2; rb++) {
      int r = mx_op(H, level, kKindColor, kTRelax, coarse ? rb | kRelax64 : rb);
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
  // while a solve program is recorded, CTA 0 alone runs the coarse end from
  // level rec_solo down: a marker counts the phases that follow it
  std::vector<TailPhase>* rec = rec_of(H);
  if (rec && level == H.rec_solo) {
    size_t at = rec->size();
    rec->push_back(TailPhase{kTSolo, 0, 0, 0, nullptr, nullptr, nullptr});
    H.rec_solo = -kMaxDepth - 2;
    int r = mx_vcycle(H, level, minlevel, nsmooth);
    H.rec_solo = level;
    (*rec)[at].nblk = (int)(rec->size() - at - 1);
    return r;
  }
  int r = mx_level_relax(H, level, nsmooth, level == minlevel);
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
    if ((r = mx_level_relax(H, level, nsmooth, false))) return r;
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

// ---------------------------------------------------------------------------
// The whole solve of a hierarchy with refinement levels in one launch of one
// thread-block cluster (kern_solve.cuh).  The program below is the sequence
// mixed_iterations runs on such a hierarchy -- the FP64 residual of the
// finest level, e = 0, then per outer iteration: coarse e = 0, the base
// planes and g of every level, the FP32 V-cycle, qbar += e, FillDown(q),
// the refinement levels' ghosts and the FP64 residual -- recorded from the
// same schedule functions, so the launch computes the same iterates.

// the highest level whose level and every level below it together hold at
// most `cells` interior cells: the coarse end that CTA 0 runs alone
int solo_level(const Hier& H, long long cells) {
  int lvl = -kMaxDepth - 2;
  if (cells <= 0) return lvl;
  long long sum = 0;
  for (int l = H.minlevel; l <= H.maxlevel; l++) {
    for (int p : H.L(l).patches) {
      const HostPatch& P = H.patches[p];
      sum += (long long)P.mx[0] * P.mx[1] * P.mx[2];
    }
    if (sum > cells) break;
    lvl = l;
  }
  return lvl;
}

int solve_norm_groups(const Hier& H, int finest) {
  return (H.L(finest).nblk[kKindInterior] + kNormCells - 1) / kNormCells;
}

// clusters of this shape that fit on the device at once (0: it cannot run);
// asked once per device, plugin, dimension and shape
int solve_fit(const Hier& H, SolveShape sh) {
  if (sh.ctas < 1 || sh.ctas > 16 || (sh.threads != 256 && sh.threads != 512 && sh.threads != 1024)) return 0;
  if (sh.tile != 32 && sh.tile != 64 && sh.tile != 128 && sh.tile != 256) return 0;
  static std::mutex mu;
  static std::map<std::tuple<int, int, int, int, int>, int> fit;
  auto key = std::make_tuple(H.ctx->device, H.problem, H.ndims, sh.ctas, sh.threads);
  {
    std::lock_guard<std::mutex> g(mu);
    auto it = fit.find(key);
    if (it != fit.end()) return it->second;
  }
  int n = mxp(H).solve_setup(H.ndims, sh);
  std::lock_guard<std::mutex> g(mu);
  fit[key] = n;
  return n;
}

bool solve_applies_(const Hier& H, int finest) {
  return H.solve_mode == 1 && !H.box && H.fpool && finest >= 1 && solve_norm_groups(H, finest) <= 2048 &&
         solve_norm_groups(H, finest) <= H.partial_cap && solve_fit(H, H.solve_shape) > 0;
}

// The program, its pools and the FP32 ghost operations, as the builder
// lays them out for one choice of which patches keep their FP32 arrays in
// distributed shared memory.
struct SolveBuild {
  std::vector<SolvePhase> prog;
  std::vector<Blk> bpool;
  std::vector<int> spool, ppool;
  std::vector<std::vector<unsigned>> ops;  // per CTA: program << 20 | operation of the FP32 ghost programs
  std::vector<const GhostOp*> progs;       // the programs' device operation arrays
  std::vector<size_t> clears;             // phases whose shared-memory ranges follow the layout
  int body = 0, bad = 0;
};

// size_only: the pools get their final sizes but the ghost operations are
// not distributed (the image's size depends on neither)
int solve_record(Hier& H, int finest, int minlevel, int nsmooth, int solo, int C, const std::vector<int>& owner,
                 const std::vector<char>& dsm, bool size_only, SolveBuild& B) {
  B = SolveBuild();
  B.ops.assign(C, {});
  // the host copies behind the device lists and ghost programs the schedule
  // functions record
  std::map<const Blk*, const std::vector<Blk>*> lists;
  std::map<const Blk*, int> kinds;
  std::map<const int*, const std::vector<int>*> stages;
  std::map<const GhostOp*, const GhostProg*> progs;
  for (int l = H.minlevel; l <= H.maxlevel; l++) {
    LevelT& L = H.L(l);
    for (int k = 0; k < kNKind; k++)
      if (L.d_blk[k]) {
        lists[L.d_blk[k]] = &L.h_blk[k];
        kinds[L.d_blk[k]] = k;
      }
    for (int ip = 0; ip < 3; ip++) {
      if (L.gp[ip].d_stage_off) stages[L.gp[ip].d_stage_off] = &L.gp[ip].stage_off;
      if (L.gp[ip].d_ops) progs[L.gp[ip].d_ops] = &L.gp[ip];
    }
    if (H.mx_norm_blk[l + kMaxDepth]) lists[H.mx_norm_blk[l + kMaxDepth]] = &H.h_mx_norm_blk[l + kMaxDepth];
  }
  if (H.mx_prep_coarse) {
    lists[H.mx_prep_coarse] = &H.h_mx_prep_coarse;
    kinds[H.mx_prep_coarse] = kKindInterior;
  }
  const int tile = H.solve_shape.tile;
  // the CTA that works on a block or ghost operation of patch p (the i-th of
  // its list or stage): CTA 0 for the levels it runs alone, the owner for
  // arrays in shared memory, else the CTAs in turn
  auto sched = [&](int p, int i) {
    if (H.patches[p].level <= solo) return 0;
    return dsm[p] ? owner[p] : i % C;
  };
  std::map<const Blk*, int> boff;
  std::map<const Blk*, std::pair<int, int>> poff;
  std::map<const int*, int> soff;
  std::map<const GhostOp*, int> goff;
  auto host_list = [&](const Blk* d) -> const std::vector<Blk>* {
    auto h = lists.find(d);
    if (h == lists.end()) {
      B.bad = 1;
      return nullptr;
    }
    return h->second;
  };
  auto blk_at = [&](const Blk* d) {  // a list as it is (FP64 phases)
    if (!d) return 0;
    auto it = boff.find(d);
    if (it != boff.end()) return it->second;
    const std::vector<Blk>* v = host_list(d);
    if (!v) return 0;
    int at = (int)B.bpool.size();
    B.bpool.insert(B.bpool.end(), v->begin(), v->end());
    return boff[d] = at;
  };
  auto part_at = [&](const Blk* d) {  // a list in CTA order, with its ctas+1 offsets
    if (!d) return std::make_pair(0, -1);
    auto it = poff.find(d);
    if (it != poff.end()) return it->second;
    const std::vector<Blk>* v = host_list(d);
    if (!v) return std::make_pair(0, -1);
    // each block of kBlock units as tiles of `tile` units (up to the list's
    // end for its patch), so that the small patches of an adaptive level do
    // not leave most of a block's threads idle
    auto kd = kinds.find(d);
    if (kd == kinds.end()) {
      B.bad = 1;
      return std::make_pair(0, -1);
    }
    std::vector<std::vector<Blk>> by(C);
    for (size_t i = 0; i < v->size(); i++) {
      const Blk bb = (*v)[i];
      long long end = std::min<long long>(bb.start + kBlock, kind_units(H, H.patches[bb.patch], kd->second));
      int q = sched(bb.patch, (int)i);
      for (long long t = bb.start; t < end; t += tile) by[q].push_back(Blk{bb.patch, (int)t});
    }
    int at = (int)B.bpool.size(), pt = (int)B.ppool.size();
    for (int r = 0; r < C; r++) {
      B.ppool.push_back((int)(B.bpool.size() - at));
      B.bpool.insert(B.bpool.end(), by[r].begin(), by[r].end());
    }
    B.ppool.push_back((int)(B.bpool.size() - at));
    return poff[d] = std::make_pair(at, pt);
  };
  auto stage_at = [&](const int* d) {  // plain stage offsets (FP64 ghost programs)
    if (!d) return 0;
    auto it = soff.find(d);
    if (it != soff.end()) return it->second;
    auto h = stages.find(d);
    if (h == stages.end()) {
      B.bad = 1;
      return 0;
    }
    int at = (int)B.spool.size();
    B.spool.insert(B.spool.end(), h->second->begin(), h->second->end());
    return soff[d] = at;
  };
  auto ghost_at = [&](const GhostOp* d) {  // an FP32 ghost program split by CTA within each stage
    auto it = goff.find(d);
    if (it != goff.end()) return it->second;
    auto h = progs.find(d);
    if (h == progs.end()) {
      B.bad = 1;
      return 0;
    }
    const GhostProg& G = *h->second;
    int at = (int)B.spool.size();
    int ns = (int)G.stage_off.size() - 1;
    if (size_only) {
      B.spool.insert(B.spool.end(), 2 * C * ns, 0);
      return goff[d] = at;
    }
    const unsigned pid = (unsigned)B.progs.size();
    if (pid >= 4096 || G.ops.size() >= (1u << 20)) {  // beyond the references' fields
      B.bad = 2;
      return 0;
    }
    B.progs.push_back(d);
    std::vector<std::vector<unsigned>> by(C);
    for (int st = 0; st < ns; st++) {
      for (auto& v : by) v.clear();
      for (int i = G.stage_off[st]; i < G.stage_off[st + 1]; i++)
        by[sched(G.ops[i].dp, i - G.stage_off[st])].push_back(pid << 20 | (unsigned)i);
      for (int r = 0; r < C; r++) {  // (first, end) in CTA r's own operation list
        B.spool.push_back((int)B.ops[r].size());
        B.ops[r].insert(B.ops[r].end(), by[r].begin(), by[r].end());
        B.spool.push_back((int)B.ops[r].size());
      }
    }
    return goff[d] = at;
  };
  auto phase = [&](int op, int arg, int bar) {
    SolvePhase f{};
    f.op = op;
    f.arg = arg;
    f.bar = bar;
    f.part = -1;
    return f;
  };
  auto push_fp64 = [&](int op, int arg, int n, const Blk* blk, int bar) {
    SolvePhase f = phase(op, arg, bar);
    f.n = n;
    f.blk = blk_at(blk);
    B.prog.push_back(f);
  };
  auto push_owned = [&](int op, int arg, int n, const Blk* blk, int bar) {
    SolvePhase f = phase(op, arg, bar);
    f.n = n;
    auto pr = part_at(blk);
    f.blk = pr.first;
    f.part = pr.second;
    B.prog.push_back(f);
  };
  auto clear = [&](long long a, long long len, int bar) {
    SolvePhase f = phase(kSClear, 0, bar);
    f.a = a;
    f.len = len;
    f.part = (int)B.ppool.size();
    B.ppool.insert(B.ppool.end(), 2 * C, 0);
    B.clears.push_back(B.prog.size());
    B.prog.push_back(f);
  };
  // what the schedule functions record, as solve phases (FP64 ghost
  // programs when fp64)
  auto record = [&](const std::function<int()>& body, bool fp64) {
    std::vector<TailPhase> rec;
    H.rec = &rec;
    int r = body();
    H.rec = nullptr;
    for (const TailPhase& t : rec) {
      SolvePhase f = phase(t.op, t.arg, 1);
      f.n = t.nblk;
      f.nstages = t.nstages;
      if (t.op == kTSolo) {
        f.op = kSSolo;
        f.bar = 0;
      } else if (t.op == kTGhost && fp64) {
        f.op = kSGhost64;
        f.ops = t.ops;
        f.stage = stage_at(t.stage_off);
      } else if (t.op == kTGhost) {
        f.stage = ghost_at(t.ops);  // f.ops: the operations by CTA, set after their upload
      } else {
        auto pr = part_at(t.blk);
        f.blk = pr.first;
        f.part = pr.second;
      }
      B.prog.push_back(f);
    }
    return r;
  };
  const int nb = solve_norm_groups(H, finest);
  const Blk* nlist = H.mx_norm_blk[finest + kMaxDepth];
  // prologue (mixed_iterations before its loop)
  push_fp64(kSNorm, 0, nb, nlist, 1);
  clear(0, (long long)H.e_len, 1);
  B.body = (int)B.prog.size();
  // mx_iteration, every cycle from the FP64 residual
  if (H.e_coarse_len) clear((long long)H.e_coarse_off, (long long)H.e_coarse_len, 0);
  for (int level = finest; level >= minlevel; level--) {
    LevelT& L = H.L(level);
    int mode = level < 0 ? 0 : (level == finest ? 1 : 2);
    bool all_coarse = level < 0 && minlevel == H.minlevel && H.mx_prep_coarse_n > 0;
    const Blk* blk = all_coarse ? H.mx_prep_coarse : L.d_blk[kKindInterior];
    int n = all_coarse ? H.mx_prep_coarse_n : L.nblk[kKindInterior];
    if (n > 0) push_owned(kSPrep, mode, n, blk, 0);
    if (all_coarse) break;
  }
  B.prog.back().bar = 1;
  H.rec_solo = solo;
  int r = record([&] { return mx_vcycle(H, finest, minlevel, nsmooth); }, false);
  H.rec_solo = -kMaxDepth - 2;
  if (r) return r;
  for (int level = finest; level >= 0; level--) {
    LevelT& L = H.L(level);
    if (L.nblk[kKindFGhost] > 0) push_owned(kSUpdate, mxp(H).nupdate, L.nblk[kKindFGhost], L.d_blk[kKindFGhost], 0);
  }
  B.prog.back().bar = 1;
  // FillDown(q) (enq_fill_down's order); from the level above the solo
  // level down in CTA 0 alone
  size_t solo_at = (size_t)-1;
  for (int level = finest; level >= minlevel + 1; level--) {
    if (level - 1 <= solo && solo_at == (size_t)-1) {
      solo_at = B.prog.size();
      B.prog.push_back(phase(kSSolo, 0, 0));
    }
    LevelT& L = H.L(level);
    if (L.nblk[kKindCoarse] > 0) push_fp64(kSFill64, 2, L.nblk[kKindCoarse], L.d_blk[kKindCoarse], 1);
    if ((r = record([&] { return enq_set_ghost(H, level - 1, 0); }, true))) return r;
  }
  if (solo_at != (size_t)-1) B.prog[solo_at].n = (int)(B.prog.size() - solo_at - 1);
  for (int level = 1; level <= finest; level++)
    if ((r = record([&] { return enq_set_ghost(H, level, 0); }, true))) return r;
  push_fp64(kSNorm, 0, nb, nlist, 1);
  push_fp64(kSFinish, 0, nb, nullptr, 0);  // every CTA decides alone
  // 2: too many ghost programs or operations for the one-launch solve;
  // 1: a recorded list without a host copy (not expected)
  return B.bad == 2 ? BSAMG_ERR_UNSUPPORTED : B.bad ? BSAMG_ERR_ARG : BSAMG_OK;
}

int solve_build(Hier& H, int finest, int minlevel, int nsmooth) {
  const int C = H.solve_shape.ctas;
  const int solo = solo_level(H, H.solve_solo_cells);
  auto key = std::make_tuple(finest, minlevel, nsmooth, solo, C * 4096 + H.solve_shape.tile);
  if (H.solve_key == key && (H.solve_img || H.solve_nofit)) return H.solve_img ? BSAMG_OK : BSAMG_ERR_UNSUPPORTED;
  const int np = (int)H.patches.size();
  auto cells = [&](int p) {
    const HostPatch& P = H.patches[p];
    return (long long)P.mx[0] * P.mx[1] * P.mx[2];
  };
  const long long nbase = mxp(H).nbase;
  auto al4 = [](long long x) { return (x + 3) & ~3LL; };
  auto floats = [&](int p) {  // a patch's FP32 arrays: e, ec, g, base planes
    const HostPatch& P = H.patches[p];
    return al4(H.nrvars * P.sq) + al4(H.nrvars * P.sc) + al4(H.nrvars * P.sf) + al4(nbase * P.sf);
  };
  // owners: the levels CTA 0 runs alone belong to it; every other level's
  // patches, finest level first, are dealt by size, largest first, each to
  // the CTA with the fewest cells of that level (then the least memory)
  std::vector<int> owner(np, 0);
  std::vector<long long> mem_all(C, 0);
  for (int l = H.maxlevel; l >= H.minlevel; l--) {
    std::vector<int> ps = H.L(l).patches;
    if (l <= solo) {
      for (int p : ps) mem_all[0] += floats(p);
      continue;
    }
    std::stable_sort(ps.begin(), ps.end(), [&](int x, int y) { return cells(x) > cells(y); });
    std::vector<long long> load(C, 0);
    for (int p : ps) {
      int r = 0;
      for (int q = 1; q < C; q++)
        if (load[q] < load[r] || (load[q] == load[r] && mem_all[q] < mem_all[r])) r = q;
      owner[p] = r;
      load[r] += cells(p);
      mem_all[r] += floats(p);
    }
  }
  // the image's size does not depend on where the arrays live: record once
  // to size it, choose the levels kept in distributed shared memory
  // (coarsest first, each level where every CTA's share fits beside the
  // image), then record the final program
  std::vector<char> dsm(np, 0);
  SolveBuild B;
  int r = solve_record(H, finest, minlevel, nsmooth, solo, C, owner, dsm, true, B);
  auto no_fit = [&] {  // the per-launch path runs this hierarchy
    solve_invalidate(H);
    H.solve_key = key;
    H.solve_nofit = true;
    return BSAMG_ERR_UNSUPPORTED;
  };
  if (r == BSAMG_ERR_UNSUPPORTED) return no_fit();
  if (r) return r;
  auto al16 = [](size_t x) { return (x + 15) & ~(size_t)15; };
  SolveImage im{};
  size_t o = al16(sizeof(SolvePhase) * B.prog.size());
  im.off_patches = (int)o;
  o = al16(o + sizeof(PatchDev) * H.hP.size());
  im.off_blk = (int)o;
  o = al16(o + sizeof(Blk) * B.bpool.size());
  im.off_stage = (int)o;
  o = al16(o + sizeof(int) * B.spool.size());
  im.off_part = (int)o;
  o = al16(o + sizeof(int) * (B.ppool.size() + C + 1));  // + the CTAs' operation segments
  im.bytes = (int)o;
  if (o > (size_t)kSolveSmemMax) return no_fit();  // too large to stage
  const long long budget = ((long long)kSolveSmemMax - (long long)o) / 4;
  std::vector<long long> mem(C, 0);
  int dsm_levels = 0;
  for (int l = minlevel; l <= finest; l++) {
    std::vector<long long> add(C, 0);
    for (int p : H.L(l).patches) add[owner[p]] += floats(p);
    bool fits = true;
    for (int q = 0; q < C; q++) fits = fits && mem[q] + add[q] <= budget;
    if (!fits) continue;
    for (int q = 0; q < C; q++) mem[q] += add[q];
    for (int p : H.L(l).patches) dsm[p] = 1;
    dsm_levels++;
  }
  if ((r = solve_record(H, finest, minlevel, nsmooth, solo, C, owner, dsm, false, B)))
    return r == BSAMG_ERR_UNSUPPORTED ? no_fit() : r;
  // each CTA's data area: e of its levels >= 0, e of its levels < 0, then
  // ec, g and the base planes
  std::vector<PatchDev> table = H.hP;
  std::vector<long long> elen(C, 0), ecoarse(C, 0), top(C, 0);
  for (int pass = 0; pass < 2; pass++) {
    for (int q = 0; q < C && pass == 1; q++) ecoarse[q] = top[q];
    for (int p = 0; p < np; p++)
      if (dsm[p] && (H.patches[p].level < 0) == (pass == 1)) {
        const HostPatch& P = H.patches[p];
        table[p].eq = top[owner[p]] + origin_of(H, P.qn);
        top[owner[p]] += al4(H.nrvars * P.sq);
      }
  }
  for (int q = 0; q < C; q++) elen[q] = top[q];
  for (int p = 0; p < np; p++) {
    table[p].owner = owner[p];
    table[p].dsm = dsm[p];
    if (!dsm[p]) continue;
    const HostPatch& P = H.patches[p];
    long long& t = top[owner[p]];
    table[p].ecq = t + origin_of(H, P.cn);
    t += al4(H.nrvars * P.sc);
    table[p].eg = t;
    t += al4(H.nrvars * P.sf);
    table[p].ephi = t;
    t += al4(nbase * P.sf);
  }
  long long dmax = 0;
  for (int q = 0; q < C; q++) dmax = std::max(dmax, top[q]);
  im.data = (int)al16((size_t)dmax * 4);
  for (size_t k = 0; k < B.clears.size(); k++) {
    int* pr = B.ppool.data() + B.prog[B.clears[k]].part;
    for (int q = 0; q < C; q++) {
      long long from = k == 0 ? 0 : ecoarse[q];  // the prologue clears all e, the loop the coarse levels' e
      pr[2 * q] = (int)from;
      pr[2 * q + 1] = (int)(elen[q] - from);
    }
  }
  // the FP32 ghost operations, CTA after CTA; each CTA stages its own in
  // shared memory when every CTA's fit in what the data area leaves
  im.seg = (int)B.ppool.size();
  std::vector<unsigned> perm;  // the operations CTA after CTA, as references into their programs
  size_t opmax = 0;
  for (int q = 0; q < C; q++) {
    B.ppool.push_back((int)perm.size());
    perm.insert(perm.end(), B.ops[q].begin(), B.ops[q].end());
    opmax = std::max(opmax, B.ops[q].size());
  }
  B.ppool.push_back((int)perm.size());
  im.ops = (int)al16(sizeof(GhostOp) * opmax);
  im.tile_log2 = 0;
  while ((1 << im.tile_log2) < H.solve_shape.tile) im.tile_log2++;
  im.ops_smem = (size_t)im.data + im.ops + o <= (size_t)kSolveSmemMax ? 1 : 0;
  if (!im.ops_smem) im.ops = 0;
  if (H.solve_ops) cudaFreeAsync(H.solve_ops, H.s);
  H.solve_ops = nullptr;
  if (!perm.empty()) {  // gathered on the device from the programs' own arrays
    size_t nperm = perm.size(), np8 = B.progs.size();
    void* tmp = nullptr;
    cudaError_t e = dev_alloc(H, (void**)&H.solve_ops, sizeof(GhostOp) * nperm);
    // the programs' base pointers first (8-byte aligned), then the references
    if (e == cudaSuccess) e = dev_alloc(H, &tmp, sizeof(void*) * np8 + sizeof(unsigned) * nperm);
    const GhostOp** dbase = static_cast<const GhostOp**>(tmp);
    unsigned* dperm = reinterpret_cast<unsigned*>(dbase + np8);
    if (e == cudaSuccess)  // staged from pageable memory before it returns
      e = cudaMemcpyAsync(dperm, perm.data(), sizeof(unsigned) * nperm, cudaMemcpyHostToDevice, H.s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(dbase, B.progs.data(), sizeof(void*) * np8, cudaMemcpyHostToDevice, H.s);
    if (e == cudaSuccess) {
      k_gather_ops<<<(unsigned)((nperm + kBlock - 1) / kBlock), kBlock, 0, H.s>>>(dbase, dperm, (int)nperm,
                                                                                 H.solve_ops);
      e = cudaGetLastError();
    }
    if (tmp) cudaFreeAsync(tmp, H.s);
    if (e != cudaSuccess) return cuda_fail(e, "solve ghost operations");
  }
  for (SolvePhase& f : B.prog)
    if (f.op == kTGhost) f.ops = H.solve_ops;
  std::vector<unsigned char> img(o, 0);
  std::memcpy(img.data(), B.prog.data(), sizeof(SolvePhase) * B.prog.size());
  std::memcpy(img.data() + im.off_patches, table.data(), sizeof(PatchDev) * table.size());
  if (!B.bpool.empty()) std::memcpy(img.data() + im.off_blk, B.bpool.data(), sizeof(Blk) * B.bpool.size());
  if (!B.spool.empty()) std::memcpy(img.data() + im.off_stage, B.spool.data(), sizeof(int) * B.spool.size());
  std::memcpy(img.data() + im.off_part, B.ppool.data(), sizeof(int) * B.ppool.size());
  if (H.solve_img) cudaFreeAsync(H.solve_img, H.s);
  H.solve_img = nullptr;
  cudaError_t e = dev_alloc(H, &H.solve_img, img.size());
  if (e == cudaSuccess)  // staged from pageable memory before it returns
    e = cudaMemcpyAsync(H.solve_img, img.data(), img.size(), cudaMemcpyHostToDevice, H.s);
  if (e != cudaSuccess) return cuda_fail(e, "solve program upload");
  H.solve_im = im;
  H.solve_nofit = false;
  H.solve_nph = (int)B.prog.size();
  H.solve_body = B.body;
  H.solve_nb = solve_norm_groups(H, finest);
  H.solve_key = key;
  H.solve_dsm_levels = dsm_levels;
  return BSAMG_OK;
}

// upload the control block and launch the program built for this hierarchy
int solve_launch(Hier& H, int finest, int maxvcycles, double tol, int errortype) {
  if (H.solve_ctl_cap < maxvcycles) {
    if (H.solve_ctl) cudaFreeAsync(H.solve_ctl, H.s);
    H.solve_ctl = nullptr;
    H.solve_ctl_cap = 0;
    cudaError_t e = dev_alloc(H, &H.solve_ctl, sizeof(SolveCtl) + sizeof(double) * (size_t)maxvcycles);
    if (e != cudaSuccess) return cuda_fail(e, "device allocation (solve control)");
    H.solve_ctl_cap = maxvcycles;
  }
  SolveCtl c{};
  c.body = H.solve_body;
  c.nph = H.solve_nph;
  c.maxv = maxvcycles;
  c.errortype = errortype;
  c.tol = tol;
  c.count = H.L(finest).count;
  c.nb = H.solve_nb;
  c.nrvars = H.nrvars;
  if (H.solve_trace_on && H.solve_trace_cap < H.solve_nph) {
    if (H.solve_trace) cudaFreeAsync(H.solve_trace, H.s);
    H.solve_trace = nullptr;
    H.solve_trace_cap = 0;
    cudaError_t e = dev_alloc(H, (void**)&H.solve_trace, sizeof(long long) * (H.solve_nph + 1));
    if (e != cudaSuccess) return cuda_fail(e, "device allocation (solve trace)");
    H.solve_trace_cap = H.solve_nph;
  }
  c.trace = H.solve_trace_on ? H.solve_trace : nullptr;
  c.ops = H.solve_ops;
  if (c.trace) {
    cudaError_t e = cudaMemsetAsync(c.trace, 0, sizeof(long long) * (H.solve_nph + 1), H.s);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(solve trace)");
  }
  SolveCtl* ctl = static_cast<SolveCtl*>(H.solve_ctl);
  double* res = reinterpret_cast<double*>(ctl + 1);
  cudaError_t e = cudaMemcpyAsync(ctl, &c, sizeof(c), cudaMemcpyHostToDevice, H.s);  // staged before it returns
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(solve control)");
  if (mxp(H).solve(mxl(H), H.solve_img, H.solve_im, ctl, res, H.d_partial, H.solve_shape) < 0)
    return cuda_fail(cudaGetLastError(), "solve launch");
  return after_launch(H, 1);
}

int solve_iterations(Hier& H, int finest, int minlevel, int nsmooth, int maxvcycles, double tol, int errortype,
                     int strict, int* ncycles, double* residuals) {
  int r;
  using clk = std::chrono::steady_clock;
  auto ms = [](clk::time_point a, clk::time_point b) { return std::chrono::duration<double, std::milli>(b - a).count(); };
  const clk::time_point t0 = clk::now();
  if ((r = solve_build(H, finest, minlevel, nsmooth))) return r;
  const clk::time_point t1 = clk::now();
  if ((r = solve_launch(H, finest, maxvcycles, tol, errortype))) return r;
  if ((r = stream_wait(H))) return r;
  const clk::time_point t2 = clk::now();
  SolveCtl* ctl = static_cast<SolveCtl*>(H.solve_ctl);
  cudaError_t e;
  std::vector<unsigned char> out(sizeof(SolveCtl) + sizeof(double) * (size_t)maxvcycles);
  e = cudaMemcpy(out.data(), ctl, out.size(), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy(solve control)");
  SolveCtl o;
  std::memcpy(&o, out.data(), sizeof(o));
  if (H.solve_trace_on && H.solve_trace) {
    H.solve_trace_h.assign(H.solve_nph + 1, 0);
    e = cudaMemcpy(H.solve_trace_h.data(), H.solve_trace, sizeof(long long) * (H.solve_nph + 1),
                   cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy(solve trace)");
    std::vector<SolvePhase> ph(H.solve_nph);
    e = cudaMemcpy(ph.data(), H.solve_img, sizeof(SolvePhase) * H.solve_nph, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy(solve program)");
    H.solve_trace_ops.resize(H.solve_nph);
    H.solve_trace_n.resize(H.solve_nph);
    for (int x = 0; x < H.solve_nph; x++) {
      H.solve_trace_ops[x] = ph[x].op;
      H.solve_trace_n[x] = ph[x].op == kTGhost || ph[x].op == kSGhost64 ? ph[x].nstages : ph[x].n;
    }
  }
  const double* rv = reinterpret_cast<const double*>(out.data() + sizeof(SolveCtl));
  int done = o.nonfinite ? o.ncycles - 1 : o.ncycles;
  if (residuals)
    for (int i = 0; i < done && i < maxvcycles; i++) residuals[i] = rv[i];
  H.h_norm[0] = o.norm[0];
  H.h_norm[1] = o.norm[1];
  H.solve_ms[0] = ms(t0, t1);
  H.solve_ms[1] = ms(t1, t2);
  H.solve_ms[2] = ms(t2, clk::now());
  if (o.nonfinite) return BSAMG_ERR_NONFINITE;
  if (ncycles) *ncycles = o.converged ? o.ncycles : maxvcycles;
  if (!o.converged && strict) return BSAMG_ERR_NOT_CONVERGED;
  return BSAMG_OK;
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
  for (void** p : {&H.solve_img, &H.solve_ctl, (void**)&H.solve_trace, (void**)&H.solve_ops}) {
    if (*p) cudaFreeAsync(*p, H.s);
    *p = nullptr;
  }
  H.solve_ctl_cap = 0;
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
    H.h_mx_norm_blk[l + kMaxDepth] = v;
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
    H.h_mx_prep_coarse = v;
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

void solve_invalidate(Hier& H) {
  if (H.solve_img) cudaFreeAsync(H.solve_img, H.s);
  H.solve_img = nullptr;
  H.solve_nofit = false;
  H.solve_key = std::make_tuple(kMaxDepth + 1, 0, 0, 0, 0);  // no program has this key
}

bool solve_shape_runs(const Hier& H, SolveShape sh) { return has_mixed(H) && solve_fit(H, sh) > 0; }

bool solve_applies(const Hier& H, int finest) { return solve_applies_(H, finest); }

int solve_time_one_cycle(Hier& H, int finest, int minlevel, int nsmooth, int errortype, double* ms) {
  int r = solve_build(H, finest, minlevel, nsmooth);
  if (r) return r;
  if ((r = stream_wait(H))) return r;
  auto t0 = std::chrono::steady_clock::now();
  if ((r = solve_launch(H, finest, 1, 0.0, errortype))) return r;
  if ((r = stream_wait(H))) return r;
  *ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return BSAMG_OK;
}

int mixed_enq_relax(Hier& H, int level, int ipass) {
  if (!has_mixed(H) || !H.fpool) return BSAMG_ERR_UNSUPPORTED;
  if (H.box) return box_enq_relax(H, level, ipass);
  return mx_op(H, level, kKindColor, kTRelax, ipass);
}

int mixed_iterations(Hier& H, int finest, int minlevel, int nsmooth, int maxvcycles, double tol, int errortype,
                     int strict, int* ncycles, double* residuals) {
  if (!has_mixed(H) || !H.fpool) return BSAMG_ERR_UNSUPPORTED;
  if (solve_applies(H, finest)) {
    // the autotuner may choose the shape, or the per-launch path
    int rs = !H.solve_tuned && H.ctx->autotune ? solve_autotune(H, finest, minlevel, nsmooth, errortype) : 0;
    if (rs) return rs;
    if (!H.solve_launches) {
      rs = solve_iterations(H, finest, minlevel, nsmooth, maxvcycles, tol, errortype, strict, ncycles, residuals);
      if (rs != BSAMG_ERR_UNSUPPORTED) return rs;  // else its program is too large to stage: per-launch path
    }
  }
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
