// Host side of libbsamg: context, hierarchy tables, device pool, launch
// schedule of the FAS V-cycle, CUDA-graph replay and the C ABI.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <atomic>
#include <thread>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "hier.h"
#include "box.h"
#include "mixed.h"

using namespace bsamg;

namespace {
thread_local std::string g_detail;
}  // namespace

namespace bsamg {

int cuda_fail(cudaError_t e, const char* what) {
  g_detail = std::string(what) + ": " + cudaGetErrorString(e);
  return BSAMG_ERR_CUDA;
}

int io_fail(const char* what) {
  g_detail = what;
  return BSAMG_ERR_IO;
}

#define CK(call)                                   \
  do {                                             \
    cudaError_t e__ = (call);                      \
    if (e__ != cudaSuccess) return cuda_fail(e__, #call); \
  } while (0)

#define RET(x)                 \
  do {                         \
    int r__ = (x);             \
    if (r__ != BSAMG_OK) return r__; \
  } while (0)

// count launches and check the launch status
int after_launch(Hier& H, int n) {
  if (n <= 0) return BSAMG_OK;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
  if (H.capturing) H.capture_launches += n;
  else H.launches += n;
  return BSAMG_OK;
}

int set_device(const Hier& H) {
  CK(cudaSetDevice(H.ctx->device));
  return BSAMG_OK;
}

long long align32(long long x) { return (x + 31) & ~31LL; }

// ---------------------------------------------------------------------------
// schedule pieces (plain FP64)

int launch_fp_tail(Hier& H, const Hier::TailProg& T) {
  const TailPhase* ph = static_cast<const TailPhase*>(T.phases);
  if (T.smem_bytes)
    return after_launch(H, launch_tail_smem(H.lc(), static_cast<const PatchDev*>(T.shadow), ph, T.nph,
                                            static_cast<const StageSeg*>(T.segs), T.nsegs, T.smem_bytes));
  return after_launch(H, launch_tail(H.lc(), ph, T.nph));
}

// the tail program being recorded: the V-cycle schedule records its
// operations instead of launching them
std::vector<TailPhase>* recording(Hier& H) { return static_cast<std::vector<TailPhase>*>(H.rec); }

// one work-list operation of the FP64 V-cycle, launched or recorded
int enq_op(Hier& H, int level, int kind, int op, int arg) {
  LevelT& L = H.L(level);
  if (auto* rec = recording(H)) {
    if (L.nblk[kind] > 0) rec->push_back(TailPhase{op, arg, L.nblk[kind], 0, L.d_blk[kind], nullptr, nullptr});
    return BSAMG_OK;
  }
  LaunchCtx c = H.lc();
  const Blk* b = L.d_blk[kind];
  int n = L.nblk[kind];
  switch (op) {
    case kTRelax: return after_launch(H, launch_relax(c, b, n, arg));
    case kTRestrict: return after_launch(H, launch_restrict_q(c, b, n));
    case kTRing: return after_launch(H, arg ? launch_correct_a(c, b, n) : launch_coarse_ghost(c, b, n));
    case kTLoad: return after_launch(H, launch_coarse_load(c, b, n));
    case kTFill: return after_launch(H, launch_fill_down(c, b, n, arg));
    default: return after_launch(H, launch_correct_b(c, b, n));
  }
}

int enq_relax(Hier& H, int level, int ipass) { return enq_op(H, level, kKindColor, kTRelax, ipass); }

int enq_set_ghost(Hier& H, int level, int ipass) {
  LevelT& L = H.L(level);
  GhostProg& g = L.gp[ipass];
  int nst = (int)g.stage_off.size() - 1;
  if (nst <= 0) return BSAMG_OK;
  if (auto* rec = recording(H)) {
    rec->push_back(TailPhase{kTGhost, 0, 0, nst, nullptr, g.d_ops, g.d_stage_off});
    return BSAMG_OK;
  }
  int nops = g.stage_off[nst];
  LaunchCtx c = H.lc();
  if (nops <= 2048) return after_launch(H, launch_ghost_program_1cta(c, g.d_ops, g.d_stage_off, nst));
  for (int s = 0; s < nst; s++)
    RET(after_launch(H, launch_ghost_stage(c, g.d_ops + g.stage_off[s], g.stage_off[s + 1] - g.stage_off[s])));
  return BSAMG_OK;
}

int enq_level_relax(Hier& H, int level, int nsmooth) {
  for (int pass = 1; pass <= nsmooth; pass++)
    for (int rb = 1; rb <= 2; rb++) {
      RET(enq_relax(H, level, rb));
      RET(enq_set_ghost(H, level, rb));
    }
  return BSAMG_OK;
}

// AFASVcycle, afasroutines.f90:495-529
int enq_vcycle(Hier& H, int level, int minlevel, int nsmooth) {
  if (!H.rec && level <= H.tail_level && level >= minlevel) {
    auto it = H.fp_tail_progs.find(std::make_tuple(level, minlevel, nsmooth));
    if (it != H.fp_tail_progs.end())  // the rest of the V-cycle in one block
      return launch_fp_tail(H, it->second);
  }
  RET(enq_level_relax(H, level, nsmooth));
  if (level > minlevel) {
    RET(enq_op(H, level, kKindCoarse, kTRestrict, 0));
    RET(enq_set_ghost(H, level - 1, 0));
    RET(enq_op(H, level, kKindCGhost, kTRing, 0));
    RET(enq_op(H, level, kKindCoarse, kTLoad, 0));
    RET(enq_vcycle(H, level - 1, minlevel, nsmooth));
    RET(enq_op(H, level, kKindCGhost, kTRing, 1));
    RET(enq_op(H, level, kKindProl, kTProlong, 0));
    RET(enq_set_ghost(H, level, 0));
    RET(enq_level_relax(H, level, nsmooth));
  }
  return BSAMG_OK;
}

int enq_fill_down_from(Hier& H, int field, int finest, int minlevel);

// Record and upload the FP64 tail programs used by a run with these
// levels once, outside any stream capture: the V-cycle (key nsmooth) and
// FillDown of q and f (keys -2, -1) from the first level at or below the
// tail level.
int fp_prepare_tail(Hier& H, int finest, int minlevel, int nsmooth) {
  int start = std::min(finest, H.tail_level);
  if (start < minlevel) return BSAMG_OK;
  for (int which : {nsmooth, -2, -1}) {
    auto key = std::make_tuple(start, minlevel, which);
    if (H.fp_tail_progs.count(key)) continue;
    std::vector<TailPhase> prog;
    H.rec = &prog;
    int r = which > 0 ? enq_vcycle(H, start, minlevel, nsmooth) : enq_fill_down_from(H, -which, start, minlevel);
    H.rec = nullptr;
    if (r) return r;
    Hier::TailProg T;
    T.nph = (int)prog.size();
    if (!prog.empty()) {
      CK(dev_alloc(H, &T.phases, sizeof(TailPhase) * prog.size()));
      CK(cudaMemcpyAsync(T.phases, prog.data(), sizeof(TailPhase) * prog.size(), cudaMemcpyHostToDevice, H.s));
    }
    // shared-memory staging of the tail levels' FP64 arrays when they fit:
    // q, qc, f, rf read and written back, qold read
    std::vector<PatchDev> shadow = H.hP;
    std::vector<StageSeg> segs;
    long long so = 0;
    auto add = [&](long long g, long long n, int out) {
      segs.push_back(StageSeg{g, (int)so, (int)n, out, 0});
      long long at = so;
      so += (n + 1) & ~1LL;
      return at;
    };
    for (size_t p = 0; p < H.patches.size(); p++) {
      const HostPatch& P = H.patches[p];
      if (P.level < minlevel || P.level > start) continue;
      PatchDev& D = shadow[p];
      long long zq = origin_of(H, P.qn), zc = origin_of(H, P.cn);  // staged from the arrays' starts
      D.oq = add(P.oq, (long long)H.nrvars * P.sq, 1) + zq;
      D.oqold = add(P.oqold, (long long)H.nrvars * P.sq, 0) + zq;
      D.oqc = add(P.oqc, (long long)H.nrvars * P.sc, 1) + zc;
      D.of = add(D.of, (long long)H.nrvars * P.sf, 1);
      D.orf = add(D.orf, (long long)H.nrvars * P.sf, 1);
    }
    if (so * (long long)sizeof(double) <= kTailSmemMax && !segs.empty() && !prog.empty()) {
      // the kernels' shared-memory limit, per plugin and device
      static std::atomic<unsigned long long> attr[kMaxPlugins];
      std::atomic<unsigned long long>& a = attr[H.problem & (kMaxPlugins - 1)];
      if (needs_setup(a, H.ctx->device)) {
        if (tail_smem_attributes(H.problem)) return cuda_fail(cudaGetLastError(), "cudaFuncSetAttribute(tail)");
        mark_setup(a, H.ctx->device);
      }
      T.smem_bytes = (int)(so * sizeof(double));
      T.nsegs = (int)segs.size();
      CK(dev_alloc(H, &T.shadow, sizeof(PatchDev) * shadow.size()));
      CK(cudaMemcpyAsync(T.shadow, shadow.data(), sizeof(PatchDev) * shadow.size(), cudaMemcpyHostToDevice, H.s));
      T.hshadow = shadow;
      CK(dev_alloc(H, &T.segs, sizeof(StageSeg) * segs.size()));
      CK(cudaMemcpyAsync(T.segs, segs.data(), sizeof(StageSeg) * segs.size(), cudaMemcpyHostToDevice, H.s));
    }
    H.fp_tail_progs[key] = T;
  }
  return BSAMG_OK;
}

// FillDown, afasroutines.f90:236-254 (field 1 = source, 2 = solution)
int enq_fill_down_from(Hier& H, int field, int finest, int minlevel) {
  for (int level = finest; level >= minlevel + 1; level--) {
    if (!H.rec && level <= H.tail_level) {
      auto it = H.fp_tail_progs.find(std::make_tuple(level, minlevel, -field));
      if (it != H.fp_tail_progs.end())  // the remaining levels in one block
        return launch_fp_tail(H, it->second);
    }
    RET(enq_op(H, level, kKindCoarse, kTFill, field));
    if (field == 2) RET(enq_set_ghost(H, level - 1, 0));
  }
  return BSAMG_OK;
}
int enq_fill_down(Hier& H, int field, int finest, int minlevel) {
  return enq_fill_down_from(H, field, finest, minlevel);
}

int enq_get_source(Hier& H, int finest) {
  for (int level = finest; level >= 0; level--) {
    LevelT& L = H.L(level);
    RET(after_launch(H, launch_get_source(H.lc(), L.d_blk[kKindInterior], L.nblk[kKindInterior])));
  }
  return BSAMG_OK;
}

int enq_update_source(Hier& H, int finest) {
  for (int level = finest; level >= 0; level--) {
    LevelT& L = H.L(level);
    RET(after_launch(H, launch_update_source(H.lc(), L.d_blk[kKindInterior], L.nblk[kKindInterior])));
  }
  return BSAMG_OK;
}

// ErrorAFAS on `level` -> H.d_norm[0] (device)
int enq_norm(Hier& H, int level, int errortype) {
  LevelT& L = H.L(level);
  RET(after_launch(H, launch_norm_partial(H.lc(), L.d_blk[kKindInterior], L.nblk[kKindInterior], H.d_partial, 1)));
  return after_launch(H, launch_norm_finish(H.s, H.d_partial, norm_partials(L.nblk[kKindInterior]), H.nrvars, L.count,
                                            errortype,
                                            H.d_norm, H.d_nonfinite));
}

int enq_copy_q_to_qold(Hier& H, int minlevel, int finest) {
  bool all = minlevel <= H.minlevel && finest >= H.maxlevel;
  if (all) {
    CK(cudaMemcpyAsync(H.pool + H.qold_region, H.pool + H.q_region, sizeof(double) * H.q_len,
                       cudaMemcpyDeviceToDevice, H.s));
    return BSAMG_OK;
  }
  for (int level = minlevel; level <= finest; level++)
    for (int p : H.L(level).patches) {
      HostPatch& P = H.patches[p];
      CK(cudaMemcpyAsync(H.pool + P.oqold, H.pool + P.oq, sizeof(double) * P.sq * H.nrvars,
                         cudaMemcpyDeviceToDevice, H.s));
    }
  return BSAMG_OK;
}

// One V-cycle iteration body of MultigridIterations (afasroutines.f90:81-104)
// followed by a copy of the norm to pinned host memory.
int enq_iteration(Hier& H, int finest, int minlevel, int nsmooth, int errortype) {
  RET(enq_vcycle(H, finest, minlevel, nsmooth));
  RET(enq_fill_down(H, 2, finest, minlevel));
  RET(enq_update_source(H, finest));
  RET(enq_fill_down(H, 1, finest, minlevel));
  RET(enq_norm(H, finest, errortype));
  CK(cudaMemcpyAsync(H.h_norm, H.d_norm, 2 * sizeof(double), cudaMemcpyDeviceToHost, H.s));
  CK(cudaMemcpyAsync(H.h_nonfinite, H.d_nonfinite, sizeof(int), cudaMemcpyDeviceToHost, H.s));
  return BSAMG_OK;
}

int capture_graph(Hier& H, const GraphKey& key, const std::function<int()>& body, Hier::GraphRec** out) {
  auto it = H.graphs.find(key);
  if (it != H.graphs.end()) {
    *out = &it->second;
    return BSAMG_OK;
  }
  CK(cudaStreamBeginCapture(H.s, cudaStreamCaptureModeThreadLocal));
  H.capturing = true;
  H.capture_launches = 0;
  int rc = body();
  H.capturing = false;
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(H.s, &g);
  if (rc != BSAMG_OK) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
  Hier::GraphRec rec;
  // An executable graph inherited from the hierarchy this one was regridded
  // from takes the new parameters in place when the launch sequence has the
  // same shape (same kernels in the same order), which costs far less than
  // instantiating a new one.
  auto donor = H.graph_donors.find(key);
  if (donor != H.graph_donors.end()) {
    cudaGraphExec_t ex = donor->second.exec;
    H.graph_donors.erase(donor);
    cudaGraphExecUpdateResultInfo info;
    if (cudaGraphExecUpdate(ex, g, &info) == cudaSuccess) {
      rec.exec = ex;
      H.graphs_updated++;
    } else {
      cudaGetLastError();  // a failed update is not an error: instantiate instead
      cudaGraphExecDestroy(ex);
    }
  }
  if (!rec.exec) {
    H.graphs_instantiated++;
    e = cudaGraphInstantiate(&rec.exec, g, 0);
    if (e != cudaSuccess) {
      cudaGraphDestroy(g);
      return cuda_fail(e, "cudaGraphInstantiate");
    }
  }
  cudaGraphDestroy(g);
  rec.nlaunch = H.capture_launches;
  H.graphs[key] = rec;
  *out = &H.graphs[key];
  return BSAMG_OK;
}

// Wait for the hierarchy's stream.  With the context's blocking waits on,
// the host thread sleeps on an event instead of spinning, which leaves the
// host cores to the threads that launch work when many hierarchies share
// the GPU.
void free_tail(Hier& H, Hier::TailProg& T) {
  for (void* p : {T.phases, T.shadow, T.segs})
    if (p) cudaFreeAsync(p, H.s);
  T = Hier::TailProg();
}

int stream_wait(Hier& H) {
  if (!H.ctx->blocking_wait) {
    CK(cudaStreamSynchronize(H.s));
    return BSAMG_OK;
  }
  if (!H.done_ev) CK(cudaEventCreateWithFlags(&H.done_ev, cudaEventBlockingSync | cudaEventDisableTiming));
  CK(cudaEventRecord(H.done_ev, H.s));
  CK(cudaEventSynchronize(H.done_ev));
  return BSAMG_OK;
}

// every captured graph of the hierarchy, the box path's solve graph
// included (after a change of what the kernels take as arguments); the
// stream is idle
void drop_graphs(Hier& H) {
  for (auto& kv : H.graphs)
    if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
  H.graphs.clear();
  if (H.box_loop) cudaGraphExecDestroy(H.box_loop);
  H.box_loop = nullptr;
}

int replay(Hier& H, Hier::GraphRec* g) {
  CK(cudaGraphLaunch(g->exec, H.s));
  H.launches += g->nlaunch;
  return stream_wait(H);
}

// plugin coefficients for a spacing h (see PatchDev::c)
void coefficients(const Hier& H, double h, double* c) {
  find_plugin(H.problem)->coefficients(H.pp, H.ndims, h, c);
}

// SetProb: the plugin's parameters from the caller's list (validated
// against the plugin's minimum count by the caller)
void set_problem_params(Hier& H, const double* params, int nparams) {
  double qpo[kMaxVars];
  std::memcpy(qpo, H.pp.qpo, sizeof(qpo));
  H.pp = ProbParams{};
  std::memcpy(H.pp.qpo, qpo, sizeof(qpo));
  H.pp.nrvars = H.nrvars;
  H.pp.problem = H.problem;
  find_plugin(H.problem)->set_params(H.pp, params, nparams);
}

// PeriodicSetup, boundary.f90:805-872
void periodic_setup(Hier& H, const int* mthbc) {
  int m[6];
  for (int f = 0; f < 6; f++) m[f] = f < 2 * H.ndims ? mthbc[f] : 10;
  static const int i13[13] = {1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13};
  static const int i1245[4] = {1, 2, 4, 5}, i1389[4] = {1, 3, 8, 9}, i2367[4] = {2, 3, 6, 7};
  static const int i1[1] = {1}, i2[1] = {2}, i3[1] = {3};
  const int* src = nullptr;
  int n = 0;
  H.periodic = 1;
  if (m[0] == 2) {
    if (m[2] == 2) {
      if (m[4] == 2) { src = i13; n = 13; } else { src = i1245; n = 4; }
    } else {
      if (m[4] == 2) { src = i1389; n = 4; } else { src = i1; n = 1; }
    }
  } else {
    if (m[2] == 2) {
      if (m[4] == 2) { src = i2367; n = 4; } else { src = i2; n = 1; }
    } else {
      if (m[4] == 2) { src = i3; n = 1; } else { H.periodic = 0; }
    }
  }
  H.nperoff = n;
  for (int i = 0; i < n; i++) H.peroffidx[i] = src[i];
}

// Host tables of a hierarchy (no device work): parent links, extents,
// validation, level lists, periodic offsets.  commit() runs it first; the
// regrid runs it on host-only hierarchies to compile their ghost programs.
int build_tables(Hier& H) {
  int root = -1;
  H.minlevel = 0;
  H.maxlevel = 0;
  for (size_t n = 0; n < H.patches.size(); n++) {
    HostPatch& P = H.patches[n];
    if (P.level == 0 && root < 0) root = (int)n;
    H.minlevel = std::min(H.minlevel, P.level);
    H.maxlevel = std::max(H.maxlevel, P.level);
  }
  if (root < 0) return BSAMG_ERR_ARG;
  for (HostPatch& P : H.patches) {
    if (P.parent_id >= 0) {
      auto it = H.id2idx.find(P.parent_id);
      if (it == H.id2idx.end()) return BSAMG_ERR_NOT_FOUND;
      if (H.patches[it->second].level != P.level - 1) return BSAMG_ERR_ARG;
      P.parent = it->second;
    }
    if (P.level > H.minlevel && P.parent < 0) return BSAMG_ERR_ARG;
    for (int d = 0; d < H.ndims; d++)  // RootInit's check, bsamroutines.f90:361-366
      if (P.mglobal[d][1] - P.mglobal[d][0] + 1 != P.mx[d]) return BSAMG_ERR_ARG;
    for (int f = 0; f < 2 * H.ndims; f++)
      if (P.mthbc[f] != 2 && P.mthbc[f] != 10 && P.mthbc[f] != kInternalBC) return BSAMG_ERR_UNSUPPORTED;
    for (int d = 0; d < 3; d++) {
      bool u = d < H.ndims;
      P.cmx[d] = (u && P.mx[d] % 2 == 0) ? P.mx[d] / 2 : 1;
      P.qn[d] = u ? P.mx[d] + 2 * H.mbc : 1;
      P.cn[d] = u ? P.cmx[d] + 2 * H.mbc : 1;
    }
    if (P.parent >= 0) {
      for (int d = 0; d < H.ndims; d++) {
        if (P.mx[d] % 2) return BSAMG_ERR_ARG;
        const HostPatch& Q = H.patches[P.parent];
        if (P.mbounds[d][0] < 1 || P.mbounds[d][1] > Q.mx[d] || P.mbounds[d][1] - P.mbounds[d][0] + 1 != P.cmx[d])
          return BSAMG_ERR_ARG;
      }
    }
    if (P.level > 0 && P.parent >= 0)
      for (int d = 0; d < H.ndims; d++)
        if (P.mx[d] < 4) return BSAMG_ERR_UNSUPPORTED;  // Interpolate2D/3D read cells 1..2 from each side
  }
  // level lists in the reference's visiting order: ApplyOnLevel walks a
  // level from its youngest node to its eldest (treeops.f90:536-550), and
  // each node added is the youngest of its level, so a level is visited in
  // the reverse of the order the patches were added
  for (size_t n = H.patches.size(); n-- > 0;) H.L(H.patches[n].level).patches.push_back((int)n);
  const HostPatch& R = H.patches[root];
  for (int l = 0; l <= kMaxDepth; l++)
    for (int d = 0; d < 3; d++) H.mxmax[l][d] = d < H.ndims ? (R.mx[d] << l) : 1;
  periodic_setup(H, R.mthbc);
  return BSAMG_OK;
}

}  // namespace bsamg

namespace {

int check_nonfinite(Hier& H) { return *H.h_nonfinite ? BSAMG_ERR_NONFINITE : BSAMG_OK; }

int multigrid_iterations(Hier& H, int finest, int minlevel, int nsmooth, int maxvcycles, double tol,
                         int errortype, int mode, int strict, int* ncycles, double* residuals) {
  if (finest > H.maxlevel || minlevel < H.minlevel || finest < 0 || minlevel > 0) return BSAMG_ERR_ARG;
  if (maxvcycles < 1 || nsmooth < 1 || (errortype != 1 && errortype != 2)) return BSAMG_ERR_ARG;
  if (mode != BSAMG_MODE_FP64 && mode != BSAMG_MODE_MIXED) return BSAMG_ERR_ARG;
  RET(set_device(H));
  if (!(mode == BSAMG_MODE_MIXED && H.box)) H.box_g_valid = false;  // the FP64 cycles change q
  // afasroutines.f90:57-76
  // the periodic-box mixed path forms f from qold itself
  if (mode == BSAMG_MODE_MIXED && H.box)
    return box_iterations(H, finest, minlevel, nsmooth, maxvcycles, tol, errortype, strict, ncycles, residuals);
  RET(fp_prepare_tail(H, finest, minlevel, nsmooth));
  RET(enq_fill_down(H, 2, finest, minlevel));
  RET(enq_get_source(H, finest));
  RET(enq_update_source(H, finest));
  RET(enq_fill_down(H, 1, finest, minlevel));
  if (mode == BSAMG_MODE_MIXED)
    return mixed_iterations(H, finest, minlevel, nsmooth, maxvcycles, tol, errortype, strict, ncycles, residuals);
  Hier::GraphRec* gr = nullptr;
  RET(capture_graph(H, std::make_tuple(mode, finest, minlevel, nsmooth, errortype),
                    [&] { return enq_iteration(H, finest, minlevel, nsmooth, errortype); }, &gr));
  int it;
  double r = 0.0;
  for (it = 1; it <= maxvcycles; it++) {
    RET(replay(H, gr));
    r = H.h_norm[0];
    if (residuals) residuals[it - 1] = r;
    RET(check_nonfinite(H));
    if (r < tol) break;
  }
  bool conv = it <= maxvcycles;
  if (ncycles) *ncycles = conv ? it : maxvcycles;
  if (!conv && strict) return BSAMG_ERR_NOT_CONVERGED;
  return BSAMG_OK;
}

// ---------------------------------------------------------------------------
// construction

int add_patch(Hier& H, int level, int id, int parent_id, const int mx[3], const int mglobal[6], const int mbounds[6],
              const int mthbc[6], const double dx[3], const double xlower[3]) {
  if (H.committed || level < -kMaxDepth || level > kMaxDepth) return BSAMG_ERR_ARG;
  if (H.id2idx.count(id)) return BSAMG_ERR_ARG;
  HostPatch P{};
  P.level = level;
  P.id = id;
  P.parent_id = parent_id;
  P.parent = -1;
  for (int d = 0; d < 3; d++) {
    bool u = d < H.ndims;
    P.mx[d] = u ? mx[d] : 1;
    P.mglobal[d][0] = u ? mglobal[2 * d] : 1;
    P.mglobal[d][1] = u ? mglobal[2 * d + 1] : 1;
    P.mbounds[d][0] = u ? mbounds[2 * d] : 1;
    P.mbounds[d][1] = u ? mbounds[2 * d + 1] : 1;
    P.dx[d] = u ? dx[d] : 0.0;
    P.xlower[d] = u ? xlower[d] : 0.0;
    if (u && P.mx[d] < 1) return BSAMG_ERR_ARG;
  }
  for (int f = 0; f < 6; f++) P.mthbc[f] = f < 2 * H.ndims ? mthbc[f] : 10;
  H.id2idx[id] = (int)H.patches.size();
  H.patches.push_back(P);
  return BSAMG_OK;
}

// RootInit + InitSeed, bsamroutines.f90:226-510
int build_uniform(Hier& H, const int mx[3], int minlevel, const int mthbc[6], const double xlower[3],
                  const double xupper[3]) {
  if (H.committed || !H.patches.empty() || minlevel > 0 || minlevel < -kMaxDepth) return BSAMG_ERR_ARG;
  int nd = H.ndims;
  int cmx[3] = {1, 1, 1}, mg[6] = {1, 1, 1, 1, 1, 1}, mb[6] = {1, 1, 1, 1, 1, 1};
  double dx[3] = {0, 0, 0}, xl[3] = {0, 0, 0};
  for (int d = 0; d < nd; d++) {
    if (mx[d] <= 0 || mx[d] % 2) return BSAMG_ERR_ARG;
    if (!(xupper[d] > xlower[d])) return BSAMG_ERR_ARG;
    cmx[d] = mx[d];
    mg[2 * d + 1] = mx[d];
    dx[d] = (xupper[d] - xlower[d]) / (double)mx[d];
    xl[d] = xlower[d];
  }
  for (int d = 1; d < nd; d++)
    if (std::fabs(dx[0] - dx[d]) > 1.0e-10) return BSAMG_ERR_ARG;
  for (int d = 0; d < nd; d++) {
    mb[2 * d] = 1;
    mb[2 * d + 1] = minlevel < 0 ? mx[d] / 2 : mx[d];
  }
  RET(add_patch(H, 0, 0, minlevel < 0 ? 1 : -1, cmx, mg, mb, mthbc, dx, xl));
  H.has_root_xupper = true;
  for (int d = 0; d < 3; d++) H.root_xupper[d] = d < nd ? xupper[d] : 0.0;
  for (int l = -1; l >= minlevel; l--) {
    int nmx[3] = {1, 1, 1}, nmg[6] = {1, 1, 1, 1, 1, 1}, nmb[6] = {1, 1, 1, 1, 1, 1};
    double ndx[3] = {0, 0, 0};
    for (int d = 0; d < nd; d++) {
      if (cmx[d] % 2) return BSAMG_ERR_ARG;
      nmx[d] = cmx[d] / 2;
      ndx[d] = dx[d] * 2.0;
      nmg[2 * d] = 1;
      nmg[2 * d + 1] = mg[2 * d + 1] / 2;
      nmb[2 * d] = 1;
      nmb[2 * d + 1] = l > minlevel ? nmx[d] / 2 : nmx[d];
    }
    RET(add_patch(H, l, -l, l > minlevel ? -l + 1 : -1, nmx, nmg, nmb, mthbc, ndx, xl));
    memcpy(cmx, nmx, sizeof(cmx));
    memcpy(mg, nmg, sizeof(mg));
    memcpy(dx, ndx, sizeof(dx));
  }
  return BSAMG_OK;
}



}  // namespace

namespace bsamg {
long long kind_units(const Hier& H, const HostPatch& P, int kind) {
  switch (kind) {
    case kKindColor: return (long long)((P.mx[0] + 1) / 2) * P.mx[1] * P.mx[2];
    case kKindInterior: return (long long)P.mx[0] * P.mx[1] * P.mx[2];
    case kKindCoarse: return P.parent >= 0 ? (long long)P.cmx[0] * P.cmx[1] * P.cmx[2] : 0;
    case kKindCGhost: return P.parent >= 0 ? (long long)P.cn[0] * P.cn[1] * P.cn[2] : 0;
    case kKindFGhost: return (long long)P.qn[0] * P.qn[1] * P.qn[2];
    case kKindProl: {  // coarse indices -gs..cmx+gs, gs = mbc - 1
      int e = 2 * (H.mbc - 1) + 1;
      return P.parent >= 0 ? (long long)(P.cmx[0] + e) * (P.cmx[1] + e) * (H.ndims == 3 ? P.cmx[2] + e : 1) : 0;
    }
  }
  return 0;
}
}  // namespace bsamg

namespace {

int upload_blocks(Hier& H, LevelT& L, int kind) {
  std::vector<Blk> v;
  for (int p : L.patches) {
    long long units = kind_units(H, H.patches[p], kind);
    for (long long s = 0; s < units; s += kBlock) v.push_back(Blk{p, (int)s});
  }
  L.nblk[kind] = (int)v.size();
  if (v.empty()) return BSAMG_OK;
  CK(dev_alloc(H, (void**)&L.d_blk[kind], sizeof(Blk) * v.size()));
  H.bytes += sizeof(Blk) * v.size();
  // a copy from pageable memory returns once the source has been staged, so
  // v may be freed on return
  CK(cudaMemcpyAsync(L.d_blk[kind], v.data(), sizeof(Blk) * v.size(), cudaMemcpyHostToDevice, H.s));
  L.h_blk[kind] = std::move(v);
  return BSAMG_OK;
}

// every cell an operation touches must lie inside its patch's ghosted
// plane (parent plane for the coarse cells of C/F operations)
// every cell a ghost program touches lies in its patch's q plane (cells are
// counted from cell (0,0,0), which sits origin_of() into the plane)
bool ghost_ops_in_bounds(const Hier& H, const GhostProg& g) {
  int np = (int)H.patches.size();
  for (const GhostOp& o : g.ops) {
    if (o.dp < 0 || o.dp >= np || o.sp < 0 || o.sp >= np) return false;
    const HostPatch &D = H.patches[o.dp], &S = H.patches[o.sp];
    long long zd = origin_of(H, D.qn), zs = origin_of(H, S.qn);
    auto in_d = [&](long long c) { return c + zd >= 0 && c + zd < D.sq; };
    auto in_s = [&](long long c) { return c + zs >= 0 && c + zs < S.sq; };
    if (!in_d(o.dcell)) return false;
    if (o.type <= kGBC) {
      if (!in_s(o.s0)) return false;
    } else {
      if (!in_d(o.s0) || !in_d(o.s1)) return false;
      int nc = o.type == kGCfA ? 1 : (o.type == kGCfAB ? 3 : 4);
      int c[4] = {o.c0, o.c1, o.c2, o.c3};
      for (int x = 0; x < nc; x++)
        if (!in_s(c[x])) return false;
    }
  }
  return true;
}

int upload_ghost(Hier& H, GhostProg& g) {
  if (g.ops.empty()) return BSAMG_OK;
  if (!ghost_ops_in_bounds(H, g)) return BSAMG_ERR_ARG;
  CK(dev_alloc(H, (void**)&g.d_ops, sizeof(GhostOp) * g.ops.size()));
  CK(dev_alloc(H, (void**)&g.d_stage_off, sizeof(int) * g.stage_off.size()));
  H.bytes += sizeof(GhostOp) * g.ops.size() + sizeof(int) * g.stage_off.size();
  CK(cudaMemcpyAsync(g.d_ops, g.ops.data(), sizeof(GhostOp) * g.ops.size(), cudaMemcpyHostToDevice, H.s));
  CK(cudaMemcpyAsync(g.d_stage_off, g.stage_off.data(), sizeof(int) * g.stage_off.size(), cudaMemcpyHostToDevice,
                     H.s));
  return BSAMG_OK;
}

// Pinned host words for the norm read-back come from a per-context pool, so
// hierarchies never call cudaMallocHost/cudaFreeHost (the latter
// synchronises the device) while other hierarchies run.
constexpr int kPinnedSlots = 1024, kSlotDoubles = 128;  // [0, 16): norms; [16, 128): the box loop's control block

int pinned_slot_take(Hier& H) {
  bsamg_ctx* c = H.ctx;
  std::lock_guard<std::mutex> lk(c->mu);
  if (!c->pinned) {
    CK(cudaMallocHost((void**)&c->pinned, sizeof(double) * kSlotDoubles * kPinnedSlots));
    for (int i = kPinnedSlots - 1; i >= 0; i--) c->free_slots.push_back(i);
  }
  if (c->free_slots.empty()) return BSAMG_ERR_BUDGET;
  H.pinned_slot = c->free_slots.back();
  c->free_slots.pop_back();
  H.h_norm = c->pinned + (size_t)H.pinned_slot * kSlotDoubles;
  H.h_nonfinite = reinterpret_cast<int*>(H.h_norm + 8);
  return BSAMG_OK;
}

void pinned_slot_give(Hier& H) {
  if (H.pinned_slot < 0) return;
  std::lock_guard<std::mutex> lk(H.ctx->mu);
  H.ctx->free_slots.push_back(H.pinned_slot);
  H.pinned_slot = -1;
  H.h_norm = nullptr;
  H.h_nonfinite = nullptr;
}

int commit(Hier& H) {
  auto tc0 = std::chrono::steady_clock::now();
  if (H.committed) return BSAMG_ERR_ARG;
  RET(set_device(H));
  RET(build_tables(H));
  {
    bool w = true;
    for (int l = H.minlevel; l <= H.maxlevel; l++) w = w && H.L(l).patches.size() == 1;
    for (const HostPatch& P : H.patches)
      for (int f = 0; f < 2 * H.ndims; f++) w = w && P.mthbc[f] == 2;
    for (int v = 0; v < H.nrvars; v++) w = w && H.pp.qpo[v] == 0.0;
    H.box = box_eligible(H, w);
  }

  // pool layout: [q...][qold...][qc...][f...][rf...][ftmp...]
  long long off = 0;
  for (HostPatch& P : H.patches) {
    P.sq = (long long)P.qn[0] * P.qn[1] * P.qn[2];
    P.sc = (long long)P.cn[0] * P.cn[1] * P.cn[2];
    P.sf = (long long)P.mx[0] * P.mx[1] * P.mx[2];
  }
  H.q_region = off;
  for (HostPatch& P : H.patches) { P.oq = off; off = align32(off + P.sq * H.nrvars); }
  H.q_len = off - H.q_region;
  H.qold_region = off;
  for (HostPatch& P : H.patches) P.oqold = P.oq + H.qold_region - H.q_region;
  off += H.q_len;
  for (HostPatch& P : H.patches) { P.oqc = off; off = align32(off + P.sc * H.nrvars); }
  for (HostPatch& P : H.patches) { P.of = off; off = align32(off + P.sf * H.nrvars); }
  for (HostPatch& P : H.patches) { P.orf = off; off = align32(off + P.sf * H.nrvars); }
  for (HostPatch& P : H.patches) { P.oftmp = off; off = align32(off + P.sf * H.nrvars); }
  H.pool_elems = (size_t)off;
  size_t need = H.pool_elems * sizeof(double) + (H.box ? box_layout(H) * sizeof(float) : mixed_pool_bytes(H));
  {
    std::lock_guard<std::mutex> lk(H.ctx->mu);
    if (H.ctx->budget && H.ctx->used + need > H.ctx->budget) return BSAMG_ERR_BUDGET;
    H.ctx->used += need;
    H.reserved = need;
  }
  H.bytes += need;
  CK(cudaStreamCreateWithFlags(&H.s, cudaStreamNonBlocking));
  // stream-ordered allocations: creating or destroying a hierarchy never
  // synchronises the device, so other hierarchies' work keeps running
  CK(dev_alloc(H, (void**)&H.pool, H.pool_elems * sizeof(double)));
  CK(cudaMemsetAsync(H.pool, 0, H.pool_elems * sizeof(double), H.s));
  RET(mixed_alloc(H));

  std::vector<PatchDev> pd(H.patches.size());
  for (size_t n = 0; n < H.patches.size(); n++) {
    const HostPatch& P = H.patches[n];
    PatchDev& D = pd[n];
    memset(&D, 0, sizeof(D));
    for (int d = 0; d < 3; d++) {
      D.mx[d] = P.mx[d];
      D.qn[d] = P.qn[d];
      D.cmx[d] = P.cmx[d];
      D.cn[d] = P.cn[d];
      D.mb[d] = P.mbounds[d][0];
    }
    D.parent = P.parent;
    D.level = P.level;
    D.gs = H.mbc - 1;
    long long zq = origin_of(H, P.qn), zc = origin_of(H, P.cn);
    D.oq = P.oq + zq; D.oqold = P.oqold + zq; D.oqc = P.oqc + zc; D.of = P.of; D.orf = P.orf; D.oftmp = P.oftmp;
    D.sq = P.sq; D.sc = P.sc; D.sf = P.sf;
    D.eq = P.e_oq + zq; D.ecq = P.e_oqc + zc; D.eg = P.e_of; D.ephi = P.e_ophi;
    D.h = P.dx[0];
    coefficients(H, P.dx[0], D.c);
    for (int x = 0; x < 4; x++) D.cf[x] = (float)D.c[x];
  }
  CK(dev_alloc(H, (void**)&H.dP, sizeof(PatchDev) * pd.size()));
  CK(cudaMemcpyAsync(H.dP, pd.data(), sizeof(PatchDev) * pd.size(), cudaMemcpyHostToDevice, H.s));  // staged
  H.bytes += sizeof(PatchDev) * pd.size();
  H.hP = std::move(pd);

  int maxblk = 1;
  for (int l = H.minlevel; l <= H.maxlevel; l++) {
    LevelT& L = H.L(l);
    for (int k = 0; k < kNKind; k++) RET(upload_blocks(H, L, k));
    maxblk = std::max(maxblk, L.nblk[kKindInterior]);
    L.count = 0.0;
    for (int p : L.patches) {
      const HostPatch& P = H.patches[p];
      L.count = (double)(H.nrvars * P.mx[0] * P.mx[1] * P.mx[2]) + L.count;
    }
  }
  // the ghost programs, compiled on host threads (they only read the tables)
  auto tg0 = std::chrono::steady_clock::now();
  {
    std::vector<std::pair<int, int>> jobs;
    std::vector<std::vector<GhostOp>*> out;
    std::vector<std::vector<int>*> so;
    for (int l = H.minlevel; l <= H.maxlevel; l++)
      for (int ip = 0; ip < (l <= 0 ? 1 : 3); ip++) {
        jobs.emplace_back(l, ip);
        out.push_back(&H.L(l).gp[ip].ops);
        so.push_back(&H.L(l).gp[ip].stage_off);
      }
    compile_set_ghost_all(H, jobs, out, so);
  }
  H.regrid_ms[4] = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tg0).count();
  for (int l = H.minlevel; l <= H.maxlevel; l++) {
    LevelT& L = H.L(l);
    for (int ip = 0; ip < 3; ip++) {
      // below and at the root the program does not depend on the colour
      if (l <= 0 && ip > 0) {
        L.gp[ip].ops = L.gp[0].ops;
        L.gp[ip].stage_off = L.gp[0].stage_off;
        L.gp[ip].d_ops = L.gp[0].d_ops;
        L.gp[ip].d_stage_off = L.gp[0].d_stage_off;
        continue;
      }
      RET(upload_ghost(H, L.gp[ip]));
    }
  }
  RET(mixed_tables(H));
  set_tail(H, H.tail_cells);
  maxblk = std::max(maxblk, (int)H.b_partials);
  H.partial_cap = maxblk;
  CK(dev_alloc(H, (void**)&H.d_partial, sizeof(double) * 2 * (size_t)maxblk * std::max(1, H.nrvars)));
  CK(dev_alloc(H, (void**)&H.d_norm, sizeof(double) * kNormOutLen));
  CK(dev_alloc(H, (void**)&H.d_nonfinite, sizeof(int) * 4));
  RET(pinned_slot_take(H));
  CK(cudaStreamSynchronize(H.s));
  H.committed = true;
  H.regrid_ms[5] = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tc0).count() -
                   H.regrid_ms[4];
  return BSAMG_OK;
}

void release(Hier& H) {
  cudaSetDevice(H.ctx->device);
  if (H.s) cudaStreamSynchronize(H.s);
  for (int m = 0; m < 64; m++)
    if (H.marks[m]) cudaEventDestroy(H.marks[m]);
  if (H.done_ev) cudaEventDestroy(H.done_ev);
  for (auto* gm : {&H.graphs, &H.graph_donors})
    for (auto& kv : *gm)
      if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
  H.graphs.clear();
  for (int l = 0; l < kNLev; l++) {
    LevelT& L = H.lev[l];
    for (int k = 0; k < kNKind; k++)
      if (L.d_blk[k]) cudaFreeAsync(L.d_blk[k], H.s);
    for (int ip = 0; ip < 3; ip++) {
      bool shared = ip > 0 && L.gp[ip].d_ops == L.gp[0].d_ops;
      if (!shared) {
        if (L.gp[ip].d_ops) cudaFreeAsync(L.gp[ip].d_ops, H.s);
        if (L.gp[ip].d_stage_off) cudaFreeAsync(L.gp[ip].d_stage_off, H.s);
      }
    }
  }
  mixed_free(H);
  for (auto& kv : H.fp_tail_progs) free_tail(H, kv.second);
  H.fp_tail_progs.clear();
  if (H.dP) cudaFreeAsync(H.dP, H.s);
  if (H.pool) cudaFreeAsync(H.pool, H.s);
  if (H.d_partial) cudaFreeAsync(H.d_partial, H.s);
  if (H.d_norm) cudaFreeAsync(H.d_norm, H.s);
  if (H.d_nonfinite) cudaFreeAsync(H.d_nonfinite, H.s);
  pinned_slot_give(H);
  if (H.s) {
    cudaStreamSynchronize(H.s);
    cudaStreamDestroy(H.s);
  }
  if (H.reserved) {
    std::lock_guard<std::mutex> lk(H.ctx->mu);
    H.ctx->used -= std::min(H.ctx->used, H.reserved);
    H.reserved = 0;
  }
}

HostPatch* find(Hier& H, int id) {
  auto it = H.id2idx.find(id);
  return it == H.id2idx.end() ? nullptr : &H.patches[it->second];
}

double* field_ptr(Hier& H, HostPatch& P, int field, size_t* n) {
  switch (field) {
    case BSAMG_FIELD_Q: *n = P.sq * H.nrvars; return H.pool + P.oq;
    case BSAMG_FIELD_QOLD: *n = P.sq * H.nrvars; return H.pool + P.oqold;
    case BSAMG_FIELD_QC: *n = P.sc * H.nrvars; return H.pool + P.oqc;
    case BSAMG_FIELD_F: *n = P.sf * H.nrvars; return H.pool + P.of;
    case BSAMG_FIELD_RF: *n = P.sf * H.nrvars; return H.pool + P.orf;
    case BSAMG_FIELD_FTMP: *n = P.sf * H.nrvars; return H.pool + P.oftmp;
  }
  *n = 0;
  return nullptr;
}

bool level_ok(const Hier& H, int level) { return level >= H.minlevel && level <= H.maxlevel; }

}  // namespace

// ---------------------------------------------------------------------------
// C ABI

extern "C" {

int bsamg_init(int device, size_t hbm_budget_bytes, bsamg_ctx** out) {
  if (!out) return BSAMG_ERR_ARG;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDeviceCount");
  if (device < 0 || device >= n) return BSAMG_ERR_ARG;
  e = cudaSetDevice(device);
  if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
  bsamg_ctx* c = new (std::nothrow) bsamg_ctx();
  if (!c) return BSAMG_ERR_ARG;
  c->device = device;
  c->budget = hbm_budget_bytes;
  cudaMemPoolProps props = {};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = device;
  e = cudaMemPoolCreate(&c->mempool, &props);
  if (e == cudaSuccess) {
    unsigned long long keep = ~0ull;
    e = cudaMemPoolSetAttribute(c->mempool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  if (e != cudaSuccess) {
    if (c->mempool) cudaMemPoolDestroy(c->mempool);
    delete c;
    return cuda_fail(e, "cudaMemPoolCreate");
  }
  *out = c;
  return BSAMG_OK;
}

int bsamg_finalize(bsamg_ctx* ctx) {
  if (ctx) cudaSetDevice(ctx->device);
  if (ctx && ctx->pinned) cudaFreeHost(ctx->pinned);
  if (ctx && ctx->mempool) cudaMemPoolDestroy(ctx->mempool);
  delete ctx;
  return BSAMG_OK;
}

int bsamg_ctx_set_blocking_wait(bsamg_ctx* ctx, int on) {
  if (!ctx) return BSAMG_ERR_ARG;
  ctx->blocking_wait = on != 0;
  return BSAMG_OK;
}

int bsamg_ctx_usage(const bsamg_ctx* ctx, size_t* used, size_t* budget) {
  if (!ctx) return BSAMG_ERR_ARG;
  if (used) *used = ctx->used;
  if (budget) *budget = ctx->budget;
  return BSAMG_OK;
}

int bsamg_hier_create(bsamg_ctx* ctx, int ndims, int nrvars, int mbc, int problem_kind, const double* params,
                      int nparams, const double* qpo, bsamg_hier** out) {
  if (!ctx || !out || !params) return BSAMG_ERR_ARG;
  if (ndims < 2 || ndims > 3) return BSAMG_ERR_ARG;
  if (mbc < 1 || mbc > 2) return BSAMG_ERR_UNSUPPORTED;  // RootInit, bsamroutines.f90:305-308
  const Plugin* pl = find_plugin(problem_kind);  // a registered problem plugin
  if (!pl) return BSAMG_ERR_ARG;
  if (nrvars != pl->nvars) return BSAMG_ERR_UNSUPPORTED;  // CH, BioGrowth: 2; growth: 3
  if (nparams < 2 || nparams < pl->nparams) return BSAMG_ERR_ARG;
  bsamg_hier* h = new (std::nothrow) bsamg_hier();
  if (!h) return BSAMG_ERR_ARG;
  h->ctx = ctx;
  h->ndims = ndims;
  h->nrvars = nrvars;
  h->mbc = mbc;
  h->problem = problem_kind;
  h->params.assign(params, params + nparams);
  for (int v = 0; v < kMaxVars; v++) h->pp.qpo[v] = (qpo && v < nrvars) ? qpo[v] : 0.0;
  set_problem_params(*h, params, nparams);
  *out = h;
  return BSAMG_OK;
}

int bsamg_regrid(bsamg_hier* h, const bsamg_regrid_params* prm, bsamg_qinit_fn qinit, void* user, bsamg_hier** out) {
  if (!h || !prm || !out) return BSAMG_ERR_ARG;
  return regrid(*h, *prm, qinit, user, out);
}

int bsamg_hier_destroy(bsamg_hier* h) {
  if (!h) return BSAMG_OK;
  release(*h);
  delete h;
  return BSAMG_OK;
}

int bsamg_patch_add(bsamg_hier* h, int level, int id, int parent_id, const int mx[3], const int mglobal[6],
                    const int mbounds[6], const int mthbc[6], const double dx[3], const double xlower[3]) {
  if (!h || !mx || !mglobal || !mbounds || !mthbc || !dx || !xlower) return BSAMG_ERR_ARG;
  return add_patch(*h, level, id, parent_id, mx, mglobal, mbounds, mthbc, dx, xlower);
}

int bsamg_build_uniform(bsamg_hier* h, const int mx[3], int minlevel, const int mthbc[6], const double xlower[3],
                        const double xupper[3]) {
  if (!h || !mx || !mthbc || !xlower || !xupper) return BSAMG_ERR_ARG;
  return build_uniform(*h, mx, minlevel, mthbc, xlower, xupper);
}

int bsamg_commit(bsamg_hier* h) {
  if (!h) return BSAMG_ERR_ARG;
  return commit(*h);
}

int bsamg_num_patches(const bsamg_hier* h, int* n) {
  if (!h || !n) return BSAMG_ERR_ARG;
  *n = (int)h->patches.size();
  return BSAMG_OK;
}

int bsamg_level_range(const bsamg_hier* h, int* minlevel, int* maxlevel) {
  if (!h || !h->committed) return BSAMG_ERR_ARG;
  if (minlevel) *minlevel = h->minlevel;
  if (maxlevel) *maxlevel = h->maxlevel;
  return BSAMG_OK;
}

int bsamg_patch_info(const bsamg_hier* h, int index, int* out, double* dxl) {
  if (!h || !out || !dxl || index < 0 || index >= (int)h->patches.size()) return BSAMG_ERR_ARG;
  const HostPatch& P = h->patches[index];
  out[0] = P.level;
  out[1] = P.id;
  out[2] = P.parent_id;
  for (int d = 0; d < 3; d++) {
    out[3 + d] = P.mx[d];
    out[6 + 2 * d] = P.mglobal[d][0];
    out[7 + 2 * d] = P.mglobal[d][1];
    out[12 + 2 * d] = P.mbounds[d][0];
    out[13 + 2 * d] = P.mbounds[d][1];
    dxl[d] = P.dx[d];
    dxl[3 + d] = P.xlower[d];
  }
  for (int f = 0; f < 6; f++) out[18 + f] = P.mthbc[f];
  return BSAMG_OK;
}

size_t bsamg_field_size(const bsamg_hier* h, int id, int field) {
  if (!h || !h->committed) return 0;
  bsamg_hier* hh = const_cast<bsamg_hier*>(h);
  HostPatch* P = find(*hh, id);
  if (!P) return 0;
  size_t n;
  field_ptr(*hh, *P, field, &n);
  return n;
}

int bsamg_put_field(bsamg_hier* h, int id, int field, const double* a, size_t n) {
  if (!h || !h->committed || !a) return BSAMG_ERR_ARG;
  h->box_g_valid = false;
  HostPatch* P = find(*h, id);
  if (!P) return BSAMG_ERR_NOT_FOUND;
  size_t nn;
  double* d = field_ptr(*h, *P, field, &nn);
  if (!d || nn != n) return BSAMG_ERR_ARG;
  RET(set_device(*h));
  CK(cudaMemcpyAsync(d, a, n * sizeof(double), cudaMemcpyHostToDevice, h->s));
  return stream_wait(*h);
}

// A box section lo..hi (Fortran indices of the field, variable last) of a
// patch field to or from a host array holding exactly that section in
// Fortran order: one strided 3D copy per variable.
int section_copy(Hier& H, int id, int field, double* a, const int lo[4], const int hi[4], bool to_device) {
  if (!H.committed || !a || !lo || !hi) return BSAMG_ERR_ARG;
  HostPatch* P = find(H, id);
  if (!P) return BSAMG_ERR_NOT_FOUND;
  size_t nn;
  double* d = field_ptr(H, *P, field, &nn);
  if (!d) return BSAMG_ERR_ARG;
  bool ghosted = field == BSAMG_FIELD_Q || field == BSAMG_FIELD_QOLD || field == BSAMG_FIELD_QC;
  const int* ext = field == BSAMG_FIELD_QC ? P->cn : (ghosted ? P->qn : P->mx);
  int low[3];  // Fortran lower bound of each dimension
  for (int k = 0; k < 3; k++) low[k] = (k < H.ndims && ghosted) ? 1 - H.mbc : 1;
  size_t plane = (size_t)ext[0] * ext[1] * ext[2];
  for (int k = 0; k < 3; k++)
    if (lo[k] < low[k] || hi[k] < lo[k] || hi[k] > low[k] + ext[k] - 1) return BSAMG_ERR_ARG;
  if (lo[3] < 1 || hi[3] < lo[3] || hi[3] > H.nrvars) return BSAMG_ERR_ARG;
  size_t sx = (size_t)(hi[0] - lo[0] + 1), sy = (size_t)(hi[1] - lo[1] + 1), sz = (size_t)(hi[2] - lo[2] + 1);
  RET(set_device(H));
  for (int v = lo[3]; v <= hi[3]; v++) {
    double* hv = a + (size_t)(v - lo[3]) * sx * sy * sz;
    double* dv = d + (size_t)(v - 1) * plane;
    cudaMemcpy3DParms m = {};
    cudaPitchedPtr hp = make_cudaPitchedPtr(hv, sx * sizeof(double), sx, sy);
    cudaPitchedPtr dp = make_cudaPitchedPtr(dv, (size_t)ext[0] * sizeof(double), ext[0], ext[1]);
    cudaPos dpos = make_cudaPos((size_t)(lo[0] - low[0]) * sizeof(double), lo[1] - low[1], lo[2] - low[2]);
    if (to_device) {
      m.srcPtr = hp;
      m.dstPtr = dp;
      m.dstPos = dpos;
      m.kind = cudaMemcpyHostToDevice;
    } else {
      m.srcPtr = dp;
      m.srcPos = dpos;
      m.dstPtr = hp;
      m.kind = cudaMemcpyDeviceToHost;
    }
    m.extent = make_cudaExtent(sx * sizeof(double), sy, sz);
    CK(cudaMemcpy3DAsync(&m, H.s));
  }
  return stream_wait(H);
}

int bsamg_put_field_section(bsamg_hier* h, int id, int field, const double* a, const int lo[4], const int hi[4]) {
  if (!h) return BSAMG_ERR_ARG;
  h->box_g_valid = false;
  return section_copy(*h, id, field, const_cast<double*>(a), lo, hi, true);
}

int bsamg_get_field_section(bsamg_hier* h, int id, int field, double* a, const int lo[4], const int hi[4]) {
  if (!h) return BSAMG_ERR_ARG;
  return section_copy(*h, id, field, a, lo, hi, false);
}

int bsamg_get_field(bsamg_hier* h, int id, int field, double* a, size_t n) {
  if (!h || !h->committed || !a) return BSAMG_ERR_ARG;
  HostPatch* P = find(*h, id);
  if (!P) return BSAMG_ERR_NOT_FOUND;
  size_t nn;
  double* d = field_ptr(*h, *P, field, &nn);
  if (!d || nn != n) return BSAMG_ERR_ARG;
  RET(set_device(*h));
  CK(cudaMemcpyAsync(a, d, n * sizeof(double), cudaMemcpyDeviceToHost, h->s));
  return stream_wait(*h);
}

int bsamg_relax_level_color(bsamg_hier* h, int level, int ipass) {
  if (!h || !h->committed || !level_ok(*h, level) || (ipass != 1 && ipass != 2)) return BSAMG_ERR_ARG;
  RET(set_device(*h));
  h->box_g_valid = false;
  return enq_relax(*h, level, ipass);
}

int bsamg_set_ghost(bsamg_hier* h, int level, int ipass) {
  if (!h || !h->committed || !level_ok(*h, level) || ipass < 0 || ipass > 2) return BSAMG_ERR_ARG;
  RET(set_device(*h));
  h->box_g_valid = false;
  return enq_set_ghost(*h, level, ipass);
}

int bsamg_level_relax(bsamg_hier* h, int level, int nsmooth) {
  if (!h || !h->committed || !level_ok(*h, level) || nsmooth < 0) return BSAMG_ERR_ARG;
  RET(set_device(*h));
  h->box_g_valid = false;
  return enq_level_relax(*h, level, nsmooth);
}

int bsamg_fill_down(bsamg_hier* h, int field, int finestlevel, int minlevel) {
  if (!h || !h->committed || (field != 1 && field != 2)) return BSAMG_ERR_ARG;
  if (!level_ok(*h, finestlevel) || !level_ok(*h, minlevel)) return BSAMG_ERR_ARG;
  RET(set_device(*h));
  h->box_g_valid = false;
  return enq_fill_down(*h, field, finestlevel, minlevel);
}

int bsamg_copy_q_to_qold(bsamg_hier* h, int minlevel, int finestlevel) {
  if (!h || !h->committed) return BSAMG_ERR_ARG;
  RET(set_device(*h));
  return enq_copy_q_to_qold(*h, minlevel, finestlevel);
}

int bsamg_vcycle(bsamg_hier* h, int level, int minlevel, int nsmooth) {
  if (!h || !h->committed || !level_ok(*h, level) || !level_ok(*h, minlevel) || minlevel > level)
    return BSAMG_ERR_ARG;
  RET(set_device(*h));
  h->box_g_valid = false;
  return enq_vcycle(*h, level, minlevel, nsmooth);
}

int bsamg_residual_norm(bsamg_hier* h, int level, int errortype, double* out) {
  if (!h || !h->committed || !level_ok(*h, level) || !out || (errortype != 1 && errortype != 2))
    return BSAMG_ERR_ARG;
  RET(set_device(*h));
  RET(enq_norm(*h, level, errortype));
  CK(cudaMemcpyAsync(h->h_norm, h->d_norm, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->s));
  CK(cudaStreamSynchronize(h->s));
  *out = h->h_norm[0];
  return BSAMG_OK;
}

int bsamg_multigrid_iterations(bsamg_hier* h, int finestlevel, int minlevel, int nsmooth, int maxvcycles,
                               double qerrortol, int updateauxfreq, int errortype, int mode, int strict,
                               int* ncycles, double* residuals) {
  if (!h || !h->committed) return BSAMG_ERR_ARG;
  (void)updateauxfreq;  // both plugins have maux = 0: UpdateAuxInVcycle returns at :417
  return multigrid_iterations(*h, finestlevel, minlevel, nsmooth, maxvcycles, qerrortol, errortype, mode, strict,
                              ncycles, residuals);
}

int bsamg_time_step(bsamg_hier* h, int first, int finestlevel, int minlevel, int nsmooth, int maxvcycles,
                    double qerrortol, int updateauxfreq, int errortype, int mode, int strict, int* ncycles,
                    double* residuals) {
  if (!h || !h->committed) return BSAMG_ERR_ARG;
  if (!level_ok(*h, finestlevel) || !level_ok(*h, minlevel)) return BSAMG_ERR_ARG;
  RET(set_device(*h));
  for (int level = 0; level <= finestlevel; level++) RET(enq_set_ghost(*h, level, 0));
  if (first) RET(enq_fill_down(*h, 2, finestlevel, minlevel));
  RET(enq_copy_q_to_qold(*h, minlevel, finestlevel));
  (void)updateauxfreq;
  return multigrid_iterations(*h, finestlevel, minlevel, nsmooth, maxvcycles, qerrortol, errortype, mode, strict,
                              ncycles, residuals);
}

int bsamg_sync(bsamg_hier* h) {
  if (!h || !h->s) return BSAMG_ERR_ARG;
  RET(set_device(*h));
  CK(cudaStreamSynchronize(h->s));
  return BSAMG_OK;
}

int bsamg_stream(bsamg_hier* h, void** stream) {
  if (!h || !stream || !h->committed) return BSAMG_ERR_ARG;
  *stream = (void*)h->s;
  return BSAMG_OK;
}

int bsamg_launch_count(const bsamg_hier* h, long long* n) {
  if (!h || !n) return BSAMG_ERR_ARG;
  *n = h->launches;
  return BSAMG_OK;
}

int bsamg_graph_stats(const bsamg_hier* h, int* instantiated, int* updated) {
  if (!h) return BSAMG_ERR_ARG;
  if (instantiated) *instantiated = h->graphs_instantiated;
  if (updated) *updated = h->graphs_updated;
  return BSAMG_OK;
}

int bsamg_set_params(bsamg_hier* h, const double* params, int nparams) {
  if (!h || !h->committed || !params) return BSAMG_ERR_ARG;
  const Plugin* pl = find_plugin(h->problem);
  if (nparams < 2 || nparams < pl->nparams) return BSAMG_ERR_ARG;
  if ((int)h->params.size() == nparams && std::equal(params, params + nparams, h->params.begin())) return BSAMG_OK;
  h->box_g_valid = false;
  int r = set_device(*h);
  if (r) return r;
  h->params.assign(params, params + nparams);
  set_problem_params(*h, params, nparams);
  for (size_t n = 0; n < h->patches.size(); n++) {
    PatchDev& D = h->hP[n];
    coefficients(*h, h->patches[n].dx[0], D.c);
    for (int x = 0; x < 4; x++) D.cf[x] = (float)D.c[x];
  }
  // stream-ordered after the work already enqueued; staged from pageable
  // memory before the call returns
  cudaError_t e = cudaMemcpyAsync(h->dP, h->hP.data(), sizeof(PatchDev) * h->hP.size(), cudaMemcpyHostToDevice,
                                  h->s);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(patch table)");
  // the staged tails' patch tables carry the coefficients too
  for (auto* progs : {&h->mx_tail_progs, &h->fp_tail_progs})
    for (auto& kv : *progs) {
      Hier::TailProg& T = kv.second;
      if (!T.shadow) continue;
      for (size_t n = 0; n < T.hshadow.size(); n++) {
        std::memcpy(T.hshadow[n].c, h->hP[n].c, sizeof(h->hP[n].c));
        std::memcpy(T.hshadow[n].cf, h->hP[n].cf, sizeof(h->hP[n].cf));
      }
      e = cudaMemcpyAsync(T.shadow, T.hshadow.data(), sizeof(PatchDev) * T.hshadow.size(), cudaMemcpyHostToDevice,
                          h->s);
      if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(tail patch table)");
    }
  // the one-launch solve's program image holds a copy of the patch table
  solve_invalidate(*h);
  // Kernels read the coefficients from the patch table, except those of the
  // periodic-box path and the parameters of plugins whose kernels take them
  // as arguments (captured in graphs): those graphs are captured again.
  if (h->box) box_coefficients(*h);
  bool keep_graphs = pl->coeffs_only && !h->box;
  if (!keep_graphs) {
    e = cudaStreamSynchronize(h->s);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
    drop_graphs(*h);
  }
  return BSAMG_OK;
}

int bsamg_hier_reset(bsamg_hier* h) {
  if (!h || !h->committed) return BSAMG_ERR_ARG;
  h->box_g_valid = false;
  int r = set_device(*h);
  if (r) return r;
  // every field back to the zero fill of bsamg_commit
  cudaError_t e = cudaMemsetAsync(h->pool, 0, h->pool_elems * sizeof(double), h->s);
  if (e == cudaSuccess && h->fpool) e = cudaMemsetAsync(h->fpool, 0, h->fpool_elems * sizeof(float), h->s);
  return e == cudaSuccess ? BSAMG_OK : cuda_fail(e, "cudaMemsetAsync(reset)");
}

int bsamg_set_box_sweep(bsamg_hier* h, int kind) {
  if (!h || kind < 0 || kind > 3) return BSAMG_ERR_ARG;
  h->box_g_valid = false;
  int r = set_device(*h);
  if (r) return r;
  if (h->committed) {  // captured graphs hold the other sweep kernel
    cudaError_t e = cudaStreamSynchronize(h->s);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
    drop_graphs(*h);
  }
  h->box_sweep = kind;
  return BSAMG_OK;
}

int bsamg_set_tail_cells(bsamg_hier* h, long long cells) {
  if (!h || !h->committed || cells < 0) return BSAMG_ERR_ARG;
  int r = set_device(*h);
  if (r) return r;
  cudaError_t e = cudaStreamSynchronize(h->s);
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
  // captured graphs embed the previous tail program
  drop_graphs(*h);
  set_tail(*h, cells);
  return BSAMG_OK;
}

int bsamg_set_solve(bsamg_hier* h, int mode, int ctas, int threads, int tile, long long solo_cells) {
  if (!h || (mode != 0 && mode != 1) || ctas < 1 || ctas > 16 || solo_cells < 0) return BSAMG_ERR_ARG;
  if (threads != 256 && threads != 512 && threads != 1024) return BSAMG_ERR_ARG;
  if (tile != 32 && tile != 64 && tile != 128 && tile != 256) return BSAMG_ERR_ARG;
  int r = set_device(*h);
  if (r) return r;
  if (mode == 1 && h->committed && h->fpool && !solve_shape_runs(*h, SolveShape{ctas, threads, tile}))
    return BSAMG_ERR_UNSUPPORTED;
  h->solve_mode = mode;
  h->solve_shape = SolveShape{ctas, threads, tile};
  h->solve_solo_cells = solo_cells;
  h->solve_tuned = true;
  return BSAMG_OK;
}

int bsamg_get_solve(const bsamg_hier* h, int* mode, int* ctas, int* threads, int* tile, long long* solo_cells) {
  if (!h) return BSAMG_ERR_ARG;
  if (mode) *mode = h->solve_mode;
  if (ctas) *ctas = h->solve_shape.ctas;
  if (threads) *threads = h->solve_shape.threads;
  if (tile) *tile = h->solve_shape.tile;
  if (solo_cells) *solo_cells = h->solve_solo_cells;
  return BSAMG_OK;
}

int bsamg_solve_info(const bsamg_hier* h, long long* info, int n) {
  if (!h || !info || n < 0) return BSAMG_ERR_ARG;
  long long v[11] = {h->solve_nph,
                     h->solve_body,
                     h->solve_dsm_levels,
                     h->solve_im.data,
                     h->solve_im.bytes,
                     h->solve_shape.ctas,
                     h->solve_shape.threads,
                     h->solve_nofit ? 1 : 0,
                     (long long)(1e3 * h->solve_ms[0]),
                     (long long)(1e3 * h->solve_ms[1]),
                     (long long)(1e3 * h->solve_ms[2])};
  for (int x = 0; x < n && x < 11; x++) info[x] = v[x];
  return BSAMG_OK;
}

int bsamg_regrid_timing(const bsamg_hier* h, double* ms, int n) {
  if (!h || !ms || n < 0) return BSAMG_ERR_ARG;
  for (int x = 0; x < n && x < 12; x++) ms[x] = h->regrid_ms[x];
  return BSAMG_OK;
}

int bsamg_solve_trace(bsamg_hier* h, int enable) {
  if (!h) return BSAMG_ERR_ARG;
  h->solve_trace_on = enable != 0;
  return BSAMG_OK;
}

int bsamg_solve_trace_read(const bsamg_hier* h, int cap, int* op, int* n, long long* cycles, int* count) {
  if (!h || !count || cap < 0) return BSAMG_ERR_ARG;
  int np = (int)h->solve_trace_ops.size();
  *count = np;
  if (h->solve_trace_h.size() != (size_t)np + 1) return BSAMG_OK;
  long long prev = h->solve_trace_h[np];
  for (int x = 0; x < np && x < cap; x++) {
    if (op) op[x] = h->solve_trace_ops[x];
    if (n) n[x] = h->solve_trace_n[x];
    // a solo block's clock is taken after its last phase: the block's time
    // goes to that phase, the others read 0
    long long t = h->solve_trace_h[x];
    if (cycles) cycles[x] = t ? t - prev : 0;
    if (t) prev = t;
  }
  return BSAMG_OK;
}

int bsamg_mark(bsamg_hier* h, int slot) {
  if (!h || !h->committed || slot < 0 || slot >= 64) return BSAMG_ERR_ARG;
  RET(set_device(*h));
  if (!h->marks[slot]) CK(cudaEventCreate(&h->marks[slot]));
  CK(cudaEventRecord(h->marks[slot], h->s));
  return BSAMG_OK;
}

int bsamg_elapsed_ms(bsamg_hier* h, int a, int b, double* ms) {
  if (!h || !ms || a < 0 || b < 0 || a >= 64 || b >= 64 || !h->marks[a] || !h->marks[b]) return BSAMG_ERR_ARG;
  RET(set_device(*h));
  CK(cudaEventSynchronize(h->marks[b]));
  float t = 0.f;
  CK(cudaEventElapsedTime(&t, h->marks[a], h->marks[b]));
  *ms = t;
  return BSAMG_OK;
}

int bsamg_time_smoother(bsamg_hier* h, int level, int mode, int reps, double* ms_per_launch) {
  if (!h || !h->committed || !level_ok(*h, level) || reps < 1 || !ms_per_launch) return BSAMG_ERR_ARG;
  if (mode != BSAMG_MODE_FP64 && mode != BSAMG_MODE_MIXED) return BSAMG_ERR_ARG;
  RET(set_device(*h));
  h->box_g_valid = false;  // the sweeps overwrite the box path's e
  RET(bsamg_mark(h, 62));
  for (int r = 0; r < reps; r++)
    RET(mode == BSAMG_MODE_FP64 ? enq_relax(*h, level, 1 + (r & 1))
                                : (h->box && h->fpool ? box_enq_smoother(*h, level, 1 + (r & 1))
                                          : mixed_enq_relax(*h, level, 1 + (r & 1))));
  RET(bsamg_mark(h, 63));
  double ms;
  RET(bsamg_elapsed_ms(h, 62, 63, &ms));
  *ms_per_launch = ms / reps;
  return BSAMG_OK;
}

int bsamg_host_register(void* ptr, size_t bytes) {
  if (!ptr || !bytes) return BSAMG_ERR_ARG;
  CK(cudaHostRegister(ptr, bytes, cudaHostRegisterDefault));
  return BSAMG_OK;
}

int bsamg_host_unregister(void* ptr) {
  if (!ptr) return BSAMG_ERR_ARG;
  CK(cudaHostUnregister(ptr));
  return BSAMG_OK;
}

int bsamg_smoother_colours(bsamg_hier* h, int level, int mode, int* colours) {
  if (!h || !h->committed || !level_ok(*h, level) || !colours) return BSAMG_ERR_ARG;
  *colours = mode == BSAMG_MODE_MIXED && h->box && h->fpool ? box_smoother_colours(*h, level) : 1;
  return BSAMG_OK;
}

const char* bsamg_strerror(int status) {
  switch (status) {
    case BSAMG_OK: return "ok";
    case BSAMG_ERR_ARG: return "bad argument or call order";
    case BSAMG_ERR_CUDA: return "CUDA runtime error";
    case BSAMG_ERR_BUDGET: return "allocation exceeds the context HBM budget";
    case BSAMG_ERR_NOT_CONVERGED: return "maxvcycles reached above qerrortol";
    case BSAMG_ERR_NONFINITE: return "residual norm is not finite";
    case BSAMG_ERR_UNSUPPORTED: return "configuration not supported";
    case BSAMG_ERR_NOT_FOUND: return "unknown patch id";
    case BSAMG_ERR_IO: return "frame file could not be read or written (see bsamg_last_error_detail)";
  }
  return "unknown status";
}

const char* bsamg_last_error_detail(void) { return g_detail.c_str(); }

}  // extern "C"
