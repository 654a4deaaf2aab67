// The problem-plugin interface on the device side.
//
// The reference binds a problem's routines at compile time: `USE Problem,
// ONLY: RelaxGrid2D, RelaxGrid3D` (afasroutines.f90:563), `Operator2D/3D`
// (:677, :743, :819), `Source2D/3D` (:333), `SourceUpdate2D/3D` (:441),
// `UpdateAuxVcycle2D/3D` (:387) and `UserBC2D/3D` (boundary.f90:644, :717)
// come from PROBLEM/<name>/problem.f90.  Fortran routines cannot run on the
// device, so each problem has a device plugin file next to the library's
// plugins (bsam1.2_gb300/plugins/<name>.cu) that restates those routines as
// the static members of one struct, and registers itself here when the
// library loads.  The library's kernels are templates over that struct
// (kern_fp64.cuh, kern_mixed.cuh); the plugin file instantiates them, so
// adding a problem adds one file and changes no library source.
//
// A plugin struct PL provides (see plugins/ch.cu for a complete one):
//
//   static constexpr int kKind;        // problem kind passed to bsamg_hier_create
//   static constexpr const char* kName;
//   static constexpr int kNV;          // nrvars
//   static constexpr int kNParams;     // minimum number of parameters
//   static constexpr bool kCoeffsOnly; // every kernel reads its parameters
//                                      // from the patch table (graphs survive
//                                      // bsamg_set_params)
//   static constexpr bool kBox;        // the periodic-box fast path (box.cu,
//                                      // CH's equations) applies
//   // host: SetProb, the per-patch coefficients (RelaxGrid's tmp constants),
//   // the UserBC Dirichlet masks, which after-step statistics exist
//   static void set_params(ProbParams&, const double* params, int n);
//   static void coefficients(const ProbParams&, int ndims, double h, double c[4]);
//   static int bc_mask(int ndims);     // bits 0-7: 2 - q, bits 8-15: -q
//   static int stats(int ndims);       // bit 0: integral of phi, bit 1: CH energy
//   // device, FP64, evaluated in the reference's order (the FP64 part of a
//   // plugin file is compiled with --fmad=false):
//   template <int DIM> __device__ static void relax(const Cell64&, const double* c, const ProbParams&);
//   template <int DIM> __device__ static void op(const double* a, long long c, long long sy, long long sz,
//                                               long long ps, const QoldView& qold, const double* cf,
//                                               const ProbParams&, double* r);
//   template <int DIM> __device__ static void source(const double* q, long long c, long long sy, long long sz,
//                                                    long long sq, const QoldView& qold, const double* cf,
//                                                    const ProbParams&, double* s);
//   template <int DIM> __device__ static void source_update(...same as source..., double* su);
//   // optional mixed-precision correction form (kMixed = true): FP32
//   // correction smoother and operator M(e) = N(qbar + e) - N(qbar) on
//   // frozen base planes, and the FP32 preparation of those planes
//   static constexpr bool kMixed;
//   static constexpr int kMxBase;      // base planes per interior cell
//   static constexpr int kMxUpdate;    // variables whose base plane the update pass refreshes
//   static MxParams mx_params(const ProbParams&);
//   template <int DIM> __device__ static void mx_prep(const Cell64&, const double* rf, float* base, float* g,
//                                                     int mode, const double* c, const ProbParams&);
//   // the correction smoother in arithmetic T: float on every level, double
//   // on the coarsest (cf: the patch's coefficients in T; e, g and the
//   // base planes are FP32 either way)
//   template <int DIM, typename T> __device__ static void mx_relax(const Cell32&, const T* cf, const MxParams&);
//   template <int DIM> __device__ static void mx_op(const float* e, long long c, long long sy, long long sz,
//                                                  long long ps, const float* base, long long fc, long long sf,
//                                                  const float* cf, const MxParams&, float* m);
//
// BSAMG_PLUGIN(PL) at the end of the file registers it.
#pragma once
#include <cuda_runtime.h>

#include "launch.h"

namespace bsamg {

// One cell of a patch in the FP64 pool, as the relaxation sees it: q, f and
// qold of variable 1 (variable v at + v*sq / + v*sf), the cell's offset in
// the ghosted arrays (c) and in the interior ones (fc), and the strides.
struct Cell64 {
  double* q;
  const double* f;
  const double* qold;
  long long c, fc, sy, sz, sq, sf;
};

// qold at the cell an operator or source is evaluated at: p points at
// variable 1 of that cell, variable v is at p[v*sq] and the neighbours at
// p[+-1], p[+-sy], p[+-sz] (the strides of qold's own array, which for the
// coarse operator of CoarseLoadingFunction is the parent's: the reference
// passes parent%qold(mb-1:mb+1), afasroutines.f90:700-704).
struct QoldView {
  const double* p;
  long long sy, sz, sq;
};

// One cell of the mixed path's FP32 correction: e (ghosted, like q), its
// right-hand side g and the frozen base planes (interior, like f).
struct Cell32 {
  float* e;
  const float* g;
  const float* base;
  long long c, fc, sy, sz, sq, sf;
};

// The plugin's parameters the FP32 correction kernels take, as floats.
struct MxParams {
  float p[4];
};

// Launchers of the plain FP64 path's plugin-dependent kernels.
struct PluginFp64 {
  int (*relax)(const LaunchCtx&, const Blk*, int nblk, int ipass);
  int (*coarse_load)(const LaunchCtx&, const Blk*, int nblk);
  int (*norm_partial)(const LaunchCtx&, const Blk*, int nblk, double* partial, int store_rf);
  int (*get_source)(const LaunchCtx&, const Blk*, int nblk);
  int (*update_source)(const LaunchCtx&, const Blk*, int nblk);
  int (*tail)(const LaunchCtx&, const TailPhase*, int nph);
  int (*tail_smem)(const LaunchCtx&, const PatchDev* shadow, const TailPhase*, int nph, const StageSeg*, int nsegs,
                   int smem_bytes);
  int (*tail_smem_attributes)();
};

// Launchers of the mixed path's plugin-dependent kernels (the correction
// form).  All take the hierarchy's stream, dimension and tables.
struct MxLaunch {
  cudaStream_t s;
  int ndims;
  const PatchDev* P;
  double* pool;
  float* fpool;
  ProbParams pp;
};
struct PluginMixed {
  int nbase, nupdate;
  int (*prep)(const MxLaunch&, const Blk*, int nblk, int mode);
  int (*relax)(const MxLaunch&, const Blk*, int nblk, int ipass);
  int (*coarse_load)(const MxLaunch&, const Blk*, int nblk);
  int (*track)(const MxLaunch&, const Blk*, int nblk, double* partial);
  // FP64 residual of the finest level, padded interior list of nb*kNormCells
  // blocks; nb partial sums of nrvars values
  int (*norm)(const MxLaunch&, const Blk* padded, int nb, double* partial);
  int (*tail)(const MxLaunch&, const PatchDev* table, const TailPhase*, int nph, const StageSeg*, int nsegs,
              int smem_bytes);
  int (*tail_smem_attributes)(int ndims);
  // the whole solve of a hierarchy with refinement levels in one cluster
  // launch; solve_setup returns how many clusters of that shape fit at once
  // (0: the shape cannot run)
  int (*solve)(const MxLaunch&, const void* image, SolveImage, SolveCtl*, double* res, double* partial, SolveShape);
  int (*solve_setup)(int ndims, SolveShape);
};

struct Plugin {
  int kind = 0;
  const char* name = nullptr;
  int nvars = 0, nparams = 0;
  bool coeffs_only = false, box = false;
  void (*set_params)(ProbParams&, const double*, int) = nullptr;
  void (*coefficients)(const ProbParams&, int, double, double*) = nullptr;
  int (*bc_mask)(int) = nullptr;
  int (*stats)(int) = nullptr;
  const PluginFp64* fp64 = nullptr;
  const PluginMixed* mixed = nullptr;
};

constexpr int kMaxPlugins = 64;
// interior blocks per partial sum of the mixed path's FP64 norm: one, so that
// a one-launch solve spreads the finest level's residual over the whole
// cluster (every group of 256 threads a few blocks)
constexpr int kNormCells = 1;

// registry (plugin.cu); a plugin file registers its FP64 part and, when it
// has one, its mixed part from static initialisers
int register_plugin_fp64(const Plugin& p);
int register_plugin_mixed(int kind, const PluginMixed* m);
const Plugin* find_plugin(int kind);
const Plugin* find_plugin_by_name(const char* name);

}  // namespace bsamg
