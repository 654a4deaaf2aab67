// Launchers of the device kernels (one function per kernel family).  Every
// launcher enqueues on the given stream and returns the number of kernel
// launches it issued; the caller checks cudaGetLastError().
#pragma once
#include <cuda_runtime.h>

#include "internal.h"

namespace bsamg {

constexpr int kNormOutLen = 8 + 3 * 128;

struct LaunchCtx {
  const PatchDev* P;  // device patch table
  double* pool;       // device FP64 pool
  float* fpool;       // device FP32 pool (mixed path), may be null
  cudaStream_t s;
  ProbParams pp;
  int ndims;
};

// work-list kinds: what one unit of a level's block list is
enum Kind : int {
  kKindColor = 0,     // one slot of a colour row: ceil(mx1/2) * mx2 * mx3
  kKindInterior = 1,  // one interior cell: mx1*mx2*mx3
  kKindCoarse = 2,    // one coarse cell under a child: cmx1*cmx2*cmx3
  kKindCGhost = 3,    // one ghosted coarse cell: (cmx+2)^d
  kKindFGhost = 4,    // one ghosted fine cell: (mx+2)^d
  kKindProl = 5,      // one coarse index -gs..cmx+gs per dimension under a child: (cmx+1+2gs)^d
  kNKind = 6
};

// One phase of a V-cycle's coarse tail run inside one thread block (the
// operations the separate launches of those levels would run, recorded on
// the host).  kTRing: the coarse ring (arg 0) or CorrectFine's first step
// (arg 1); kTRelax: arg = ipass; kTFill: FillDownLevel, arg = field.
enum TailOp : int { kTRelax = 0, kTRestrict = 1, kTRing = 2, kTLoad = 3, kTProlong = 4, kTGhost = 5, kTFill = 6 };
// Flag of a relaxation's ipass on the correction's coarsest level: the
// smoother computes in FP64 (FP32 storage), the coarse solve of the
// V-cycle at the reference's precision.
constexpr int kRelax64 = 4;
struct TailPhase {
  int op, arg, nblk, nstages;
  const Blk* blk;
  const GhostOp* ops;
  const int* stage_off;
};

// Marks, while a solve program is recorded, the start of the coarse end of
// a V-cycle that one CTA runs alone (nblk = number of phases that follow).
constexpr int kTSolo = 7;

// The whole mixed-precision solve of a hierarchy with refinement levels as
// one program executed by a single thread-block cluster (kern_solve.cuh):
// the FP32 correction V-cycle's operations (ops 0-5, as TailOp), the FP64
// operations of the defect-correction loop around it, and the exit test.
enum SolveOp : int {
  kSClear = 8,     // fpool[a .. a+len) = 0
  kSPrep = 9,      // base planes and g of a level (arg = mode of mx_prep)
  kSUpdate = 10,   // qbar += e over the ghosted cells, e = 0, base refresh (arg = variables refreshed)
  kSFill64 = 11,   // FillDown of q in FP64 (FillDownLevel, field 2)
  kSGhost64 = 12,  // an FP64 ghost program
  kSNorm = 13,     // FP64 residual of the finest level: rf and n partial sums (padded interior list)
  kSFinish = 14,   // one CTA: the deterministic final sum, the residual record and the exit decision
  kSSolo = 15      // the next n phases run in CTA 0 alone (barriers of that CTA between them)
};
// FP32 operations (0-5, kSClear, kSPrep, kSUpdate) take their work by
// owner: each CTA the blocks (ghost operations) of the patches it owns,
// part[rank] .. part[rank+1] of the phase's list (of each stage), CTA 0
// all of them inside a solo block.  FP64 operations spread their list over
// all threads of the cluster.
struct SolvePhase {
  int op, arg, n, nstages;
  int bar;    // a cluster barrier follows the phase
  int blk;    // the phase's work list: first entry in the program image's block pool
  int stage;  // ghost programs: first entry of their stage offsets in the image's stage pool
              // (FP64: nstages+1 offsets; FP32: for stage s and CTA r, the pair at 2*(s*ctas + r))
  int part;   // owner partition: first of ctas+1 entries in the image's part pool (-1: none)
  const GhostOp* ops;  // a ghost program's operations (global memory)
  long long a, len;    // kSClear: the range of the FP32 pool
};
// The program image every CTA of a solve copies into its shared memory at
// the start, after a data area of `data` bytes that holds the FP32 arrays
// of the patches it owns in distributed shared memory: the phases at
// offset 0, then the patch table, the block, stage and part pools (byte
// offsets from the image's start, 16-byte aligned).  Read-only data read
// from shared memory is not lost at a cluster barrier, whose acquire
// discards what the L1 cache holds.
struct SolveImage {
  int bytes, data, off_patches, off_blk, off_stage, off_part;
  // the FP32 ghost operations are ordered by CTA: CTA r's are [seg[r],
  // seg[r+1]) of the program's operation array (seg: ctas+1 entries of the
  // part pool at off_seg); when ops_smem, each CTA stages its own after its
  // data area (ops bytes reserved per CTA)
  int seg, ops_smem, ops;
  int tile_log2;  // FP32 work lists are split into tiles of 2^tile_log2 units (at most 256)
};
constexpr int kSolveSmemMax = 192 * 1024;  // largest image a solve stages
// Control block of a solve launch (device memory); the residual of V-cycle
// it (1-based) follows it at res[it-1].
struct SolveCtl {
  int body, nph;      // first phase of the loop body, phases in the program
  int maxv, errortype;
  double tol, count;  // exit tolerance, ErrorAFAS denominator of the finest level
  int nb, nrvars;     // partial sums of the norm, variables
  // results
  int ncycles, converged, nonfinite, stop;
  double norm[2];     // the last norm and its raw sum
  const GhostOp* ops;  // the program's FP32 ghost operations, CTA after CTA
  // when set: CTA 0's clock at the end of every phase of the prologue and
  // the first outer iteration (trace[x], cycles of the SM it runs on), and
  // at the start (trace[nph])
  long long* trace;
};
// launch shape of the solve kernel: CTAs in the cluster, threads per CTA
struct SolveShape {
  int ctas, threads;
  int tile;  // units per tile of the FP32 work lists (32, 64, 128 or 256)
};

// A contiguous run of pool elements staged in shared memory by a tail
// kernel: pool[g .. g+n) <-> smem[s .. s+n); written back when out != 0.
struct StageSeg {
  long long g;
  int s, n, out, pad;
};
constexpr int kTailSmemMax = 160 * 1024;  // shared-memory budget of a staged tail

// ---- plain FP64 path (fp64.cu, built with --fmad=false) ----
int launch_relax(const LaunchCtx& c, const Blk* blk, int nblk, int ipass);
int launch_restrict_q(const LaunchCtx& c, const Blk* blk, int nblk);
int launch_coarse_ghost(const LaunchCtx& c, const Blk* blk, int nblk);
int launch_coarse_load(const LaunchCtx& c, const Blk* blk, int nblk);
int launch_correct_a(const LaunchCtx& c, const Blk* blk, int nblk);
// qc of every patch in blk = its parent's q under it, ghost rings included
int launch_qc_from_parent(const LaunchCtx& c, const Blk* blk, int nblk);
int launch_correct_b(const LaunchCtx& c, const Blk* blk, int nblk);
int launch_fill_down(const LaunchCtx& c, const Blk* blk, int nblk, int field);
int launch_get_source(const LaunchCtx& c, const Blk* blk, int nblk);
int launch_update_source(const LaunchCtx& c, const Blk* blk, int nblk);
// partial sums of rf^2 (nrvars per CTA) -> partial[norm_partials(nblk)*nrvars]:
// one CTA per kNormGroup consecutive blocks of the work list, so the FP64
// shuffle reduction is paid once per kNormGroup * 256 cells
constexpr int kNormGroup = 4;
inline int norm_partials(int nblk) { return (nblk + kNormGroup - 1) / kNormGroup; }
int launch_norm_partial(const LaunchCtx& c, const Blk* blk, int nblk,
                        double* partial, int store_rf);
// deterministic final sum; writes out[0] = norm, out[1] = raw sum,
// and nonfinite[0] = 0 when the norm is finite, 1 otherwise (nothing when
// nonfinite is null).  out must hold
// kNormOutLen doubles (out[8 ..] is scratch of the two-stage sum); the
// partials hold nrvars values per block.
int launch_norm_finish(cudaStream_t s, const double* partial, int nblk,
                       int nrvars, double count, int errortype, double* out,
                       int* nonfinite);
int launch_ghost_stage(const LaunchCtx& c, const GhostOp* ops, int n);

// ---- after-step statistics and uniform-mesh output (io.cu, --fmad=false) ----
// partial[2*(pofs + b)] = (mass, energy) of block b of a level's interior
// list (coarse = false) or, negated, of the parent cells of its coarse list
int launch_stats(const LaunchCtx& c, const Blk* blk, int nblk, bool coarse, int mass, int energy, double* partial,
                 int pofs);
int launch_stats_finish(cudaStream_t s, const double* partial, int n, double* out);
// F = mass-corrected prolongation of the uniform (n+2)^d block A (one variable)
int launch_uniform_prolong(cudaStream_t s, int ndims, const double* A, double* F, const int n[3]);
// the seeded spinodal start of one CH patch (q: its ghosted q, two planes of sq)
int launch_seed_spinodal(cudaStream_t s, int ndims, int mbc, double* q, long long sq, const int mx[3], unsigned long long seed,
                         double mean, double amp, double eps2, double h);
// a patch's q(0:mx+1) (nv variables; oq the offset of its cell (0,0,0))
// into the uniform block U (extents un)
int launch_uniform_scatter(cudaStream_t s, int ndims, const double* pool, long long oq, long long sq, const int qn[3],
                           const int mx[3], const int g[3], double* U, const int un[3], int nv);
int launch_ghost_program_1cta(const LaunchCtx& c, const GhostOp* ops,
                              const int* stage_off, int nstages);
// the recorded coarse tail of an FP64 V-cycle, one block
int launch_tail(const LaunchCtx& c, const TailPhase* ph, int nph);
// the same on arrays staged in shared memory (shadow: the patch table that
// addresses them); tail_smem_attributes raises the dynamic shared-memory
// limit of a plugin's kernels to kTailSmemMax (0 on success)
int launch_tail_smem(const LaunchCtx& c, const PatchDev* shadow, const TailPhase* ph, int nph, const StageSeg* segs,
                     int nsegs, int smem_bytes);
int tail_smem_attributes(int problem);

}  // namespace bsamg
