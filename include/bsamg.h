/*
 * bsamg -- GB300 (sm_103a) FAS multigrid V-cycle for BSAM 1.2 patch
 * hierarchies.  C ABI: plain ints, doubles, pointers and sizes; no C++ or
 * torch types.  Every function returns an int status: 0 = OK, negative =
 * error (see bsamg_strerror).  Nothing in the library aborts, traps or
 * prints; a device-side failure is reported through the status of the call
 * that observes it.
 *
 * The entry points replace the following reference routines (paths within
 * the BSAM 1.2 project):
 *
 *   bsamg_hier_create / bsamg_patch_add / bsamg_commit
 *       -> LIBRARY/bsamstorage.f90:54-144 (AllocFields) and the patch
 *          descriptor of LIBRARY/nodeinfodef.f90:118-220; the Fortran host
 *          calls bsamg_patch_add once per node it visits with ApplyOnLevel
 *          (LIBRARY/treeops.f90:515-552) after a regrid
 *          (LIBRARY/bsamroutines.f90:682-702).
 *   bsamg_build_uniform
 *       -> RootInit + InitSeed, LIBRARY/bsamroutines.f90:226-510.
 *   bsamg_put_field / bsamg_get_field
 *       -> direct access to info%q, info%qold, ... of a node (the Fortran
 *          arrays are passed whole, ghost layers included).
 *   bsamg_multigrid_iterations
 *       -> MultigridIterations, LIBRARY/afasroutines.f90:48-110.
 *   bsamg_time_step
 *       -> one pass of the TakeTimeSteps loop body on a fixed mesh,
 *          LIBRARY/bsamroutines.f90:657-797.
 *   bsamg_copy_q_to_qold -> CopyQToQold, LIBRARY/bsamroutines.f90:592-605.
 *   bsamg_fill_down      -> FillDown, LIBRARY/afasroutines.f90:236-254.
 *   bsamg_vcycle         -> AFASVcycle, LIBRARY/afasroutines.f90:495-529.
 *   bsamg_level_relax    -> LevelRelax, LIBRARY/afasroutines.f90:532-557.
 *   bsamg_relax_level_color -> ApplyOnLevel(level, RelaxPatch) for one
 *          colour, LIBRARY/afasroutines.f90:549-550 / :560-607.
 *   bsamg_set_ghost      -> SetGhost, LIBRARY/boundary.f90:67-97.
 *   bsamg_residual_norm  -> ErrorAFAS, LIBRARY/afasroutines.f90:113-160.
 *
 * Field layout of put/get: the reference's Fortran layout
 * (LIBRARY/bsamstorage.f90:81-90, :106-115), column-major, variable index
 * slowest: q(1-mbc:mx1+mbc, 1-mbc:mx2+mbc, [1-mbc:mx3+mbc | 1:1], 1:nrvars).
 */
#ifndef BSAMG_H
#define BSAMG_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct bsamg_ctx bsamg_ctx;
typedef struct bsamg_hier bsamg_hier;

/* status codes */
#define BSAMG_OK 0
#define BSAMG_ERR_ARG -1         /* bad argument or call order */
#define BSAMG_ERR_CUDA -2        /* a CUDA runtime call failed */
#define BSAMG_ERR_BUDGET -3      /* allocation above the context's HBM budget */
#define BSAMG_ERR_NOT_CONVERGED -4 /* maxvcycles reached above qerrortol (returned only when requested) */
#define BSAMG_ERR_NONFINITE -5   /* the residual norm is NaN or Inf */
#define BSAMG_ERR_UNSUPPORTED -6 /* configuration not implemented */
#define BSAMG_ERR_NOT_FOUND -7   /* unknown patch id */
#define BSAMG_ERR_IO -8          /* a frame file could not be opened, read, parsed or written */

/* problem kinds: the device form of a PROBLEM/<name> plugin */
#define BSAMG_PROBLEM_CH 1        /* PROBLEM/CH/problem.f90 */
#define BSAMG_PROBLEM_BIOGROWTH 2 /* PROBLEM/BioGrowth/problem.f90 */
/* Three-variable growth plugin (phi, nutrient n, pressure p; nrvars = 3);
 * no reference counterpart (the reference's 3D BioGrowth is a stub,
 * BioGrowth/problem.f90:445-478, and has no pressure).  phi and n follow
 * BioGrowth's equations with 2*ndims neighbours; p solves
 * -Lap(p)/h^2 - cpress*phi*n = 0.  params: dt, eps, gamma, lambda, czero,
 * cpress.  Physical faces: phi reflected, n = 1, p = 0. */
#define BSAMG_PROBLEM_GROWTH 3

/* Problem plugins linked into this library.  Replaces the compile-time
 * binding `USE Problem, ONLY: RelaxGrid2D, ...` (afasroutines.f90:333, :387,
 * :441, :563, :677; boundary.f90:644, :717): every PROBLEM/<name> plugin
 * has a device plugin file (bsam1.2_gb300/plugins/<name>.cu) that registers
 * a kind and a name when the library loads.  bsamg_problem_kind returns the
 * kind of the plugin called `name` (BSAMG_ERR_NOT_FOUND if none);
 * bsamg_problem_info its nrvars, its minimum parameter count and whether it
 * has a mixed-precision correction form (BSAMG_MODE_MIXED). */
int bsamg_problem_kind(const char* name, int* kind);
int bsamg_problem_info(int kind, int* nrvars, int* nparams, int* has_mixed);

/* fields of a patch (nodeinfodef.f90:184-214) */
#define BSAMG_FIELD_Q 0
#define BSAMG_FIELD_QOLD 1
#define BSAMG_FIELD_QC 2
#define BSAMG_FIELD_F 3
#define BSAMG_FIELD_RF 4
#define BSAMG_FIELD_FTMP 5

/* arithmetic modes of bsamg_multigrid_iterations */
#define BSAMG_MODE_FP64 0  /* plain FP64 path: the drop-in, same order as the reference */
#define BSAMG_MODE_MIXED 1 /* FP32 smoothing/prolongation in an FP64 defect-correction loop */

/* Context: one device, one HBM budget.  hbm_budget_bytes = 0 means no
 * limit beyond the device's own memory. */
int bsamg_init(int device, size_t hbm_budget_bytes, bsamg_ctx** out);
int bsamg_finalize(bsamg_ctx* ctx);
/* bytes currently allocated by hierarchies of this context */
int bsamg_ctx_usage(const bsamg_ctx* ctx, size_t* used, size_t* budget);
/* Host waits of the context's hierarchies (the per-V-cycle convergence
 * read-back, put/get) sleep on a blocking-sync event instead of spinning
 * (on != 0).  For many host threads sharing the GPU (serving); a single run
 * keeps the default spin, which wakes sooner. */
int bsamg_ctx_set_blocking_wait(bsamg_ctx* ctx, int on);

/* Hierarchy.  params: [0]=dt [1]=eps, then for BIOGROWTH [2]=gamma
 * [3]=lambda [4]=czero.  qpo: nrvars quasi-periodic offsets (nodeinfodef
 * qpo), may be NULL.  mbc = 1 or 2 ghost layers (RootInit's range). */
int bsamg_hier_create(bsamg_ctx* ctx, int ndims, int nrvars, int mbc,
                      int problem_kind, const double* params, int nparams,
                      const double* qpo, bsamg_hier** out);
int bsamg_hier_destroy(bsamg_hier* h);

/* ---- AMR regrid ------------------------------------------------------
 * The AMR(rootlevel) pass that TakeTimeSteps runs before every time step
 * (LIBRARY/bsamroutines.f90:657-689, AMR :966-991): level by level from the
 * root, SetGhost(l,0); tag (ErrFlag :1059-1131 with the plugin rule
 * SetErrFlagsUser2D/3D, PROBLEM/CH/problem.f90:248-308, or the gradient
 * rule); buffer the tags (BufferAndList :1206-1247, InflateEdgeTags
 * :1267-1308, periodic images included); cluster the tags of every patch
 * (NewSubGrids :1408-1605, modified Berger-Rigoutsos); make the children
 * (MakeNewGrid :1663-1784) and fill them (InitFields :1787-1856: the
 * initial condition through `qinit` when `initial`, else mass-corrected
 * bilinear/trilinear prolongation from the parent); copy the previous
 * level-(l+1) values over them (TransferValues :1859-1951).  The per-level
 * arrays are the griddata namelist entries (bsamroutines.f90:243-266).
 * The result is a new committed hierarchy on the same context: the levels
 * <= 0 of h (q and qold) and the new levels > 0; h is left unchanged and
 * stays valid.  New patch ids are first_id, first_id+1, ... in creation
 * order (parents in visiting order, children in NewSubGrids order).
 * maxside > 0 splits new patches to at most maxside cells per side (not a
 * reference feature). */
#define BSAMG_TAG_CH 0       /* |second differences of phi| > (2|3) qtolerance */
#define BSAMG_TAG_GRADIENT 1 /* |grad phi| h > qtolerance (central differences) */
typedef struct {
  int maxlevel;
  int tagging;
  int initial;
  int maxside;
  int first_id;
  int ibuffer[11];
  int minimumgridpoints[11];
  double qtolerance[11];
  double desiredfillratio[11];
} bsamg_regrid_params;
/* Fill q (ghosted Fortran layout q(1-mbc:mx+mbc, ...), nrvars variables;
 * zero on entry) of a new patch with the initial condition (the plugin's
 * QInit2D/3D). */
typedef void (*bsamg_qinit_fn)(void* user, int level, const int* mx, const double* dx, const double* xlower,
                               double* q);
int bsamg_regrid(bsamg_hier* h, const bsamg_regrid_params* prm, bsamg_qinit_fn qinit, void* user,
                 bsamg_hier** out);

/* One patch (node).  Patches of a level are visited in the order they are
 * added, which the caller makes the reference's ApplyOnLevel order
 * (youngest first).  mglobal/mbounds are (lo,hi) pairs per dimension;
 * parent_id = -1 for the coarsest level. */
int bsamg_patch_add(bsamg_hier* h, int level, int id, int parent_id,
                    const int mx[3], const int mglobal[6],
                    const int mbounds[6], const int mthbc[6],
                    const double dx[3], const double xlower[3]);
/* Root grid (id 0) plus one grid per level -1..minlevel (id = -level). */
int bsamg_build_uniform(bsamg_hier* h, const int mx[3], int minlevel,
                        const int mthbc[6], const double xlower[3],
                        const double xupper[3]);
/* Builds tables, allocates the device pool (zero-filled) and the launch
 * schedule.  No patch may be added afterwards. */
int bsamg_commit(bsamg_hier* h);
int bsamg_num_patches(const bsamg_hier* h, int* n);
/* The coarsest and finest levels of a committed hierarchy (the host's
 * minlevel and finestlevel, bsamdriver's tree bookkeeping: after a regrid
 * the finest level is the deepest one the clustering produced). */
int bsamg_level_range(const bsamg_hier* h, int* minlevel, int* maxlevel);
/* Geometry of the patch at `index` in visiting order: out[0..23] = level,
 * id, parent_id, mx[3], mglobal[6], mbounds[6], mthbc[6]; dxl[0..5] =
 * dx[3], xlower[3] -- the nodeinfo fields a host walks after a regrid
 * (LIBRARY/nodeinfodef.f90:118-220). */
int bsamg_patch_info(const bsamg_hier* h, int index, int* out, double* dxl);
size_t bsamg_field_size(const bsamg_hier* h, int id, int field);
/* synchronous host <-> device copies of a whole field array (n doubles) */
int bsamg_put_field(bsamg_hier* h, int id, int field, const double* a,
                    size_t n);
int bsamg_get_field(bsamg_hier* h, int id, int field, double* a, size_t n);
/* The same for a box section of a field: lo[0..3], hi[0..3] are Fortran
 * bounds in the field's own index space (q, qold: 1-mbc..mx+mbc; qc:
 * 1-mbc..cmx+mbc; f, rf, ftmp: 1..mx; the unused dimension of a 2D patch
 * 1..1; the variable 1..nrvars last), and `a` holds exactly the section in
 * Fortran order, as the reference passes array sections such as
 * info%q(1:mx(1),1:mx(2),1,1:nrvars). */
int bsamg_put_field_section(bsamg_hier* h, int id, int field, const double* a, const int lo[4], const int hi[4]);
int bsamg_get_field_section(bsamg_hier* h, int id, int field, double* a, const int lo[4], const int hi[4]);

/* single operations, FP64 */
int bsamg_relax_level_color(bsamg_hier* h, int level, int ipass);
int bsamg_set_ghost(bsamg_hier* h, int level, int ipass);
int bsamg_level_relax(bsamg_hier* h, int level, int nsmooth);
int bsamg_fill_down(bsamg_hier* h, int field /*1=f, 2=q*/, int finestlevel,
                    int minlevel);
int bsamg_copy_q_to_qold(bsamg_hier* h, int minlevel, int finestlevel);
int bsamg_vcycle(bsamg_hier* h, int level, int minlevel, int nsmooth);
int bsamg_residual_norm(bsamg_hier* h, int level, int errortype,
                        double* out);

/* MultigridIterations.  residuals (may be NULL) receives up to maxvcycles
 * norms; *ncycles the number of V-cycles run.  Reaching maxvcycles without
 * convergence returns BSAMG_OK, as the reference does, unless
 * strict != 0, in which case it returns BSAMG_ERR_NOT_CONVERGED. */
int bsamg_multigrid_iterations(bsamg_hier* h, int finestlevel, int minlevel,
                               int nsmooth, int maxvcycles, double qerrortol,
                               int updateauxfreq, int errortype, int mode,
                               int strict, int* ncycles, double* residuals);
/* SetGhost(l,0) for l = 0..finest, FillDown(q) if first, CopyQToQold,
 * MultigridIterations. */
int bsamg_time_step(bsamg_hier* h, int first, int finestlevel, int minlevel,
                    int nsmooth, int maxvcycles, double qerrortol,
                    int updateauxfreq, int errortype, int mode, int strict,
                    int* ncycles, double* residuals);

/* ---- frame files, restart and after-step statistics ----
 *
 * bsamg_after_step_stats -> the AfterStepStatistics + GetMeshSize pass of
 *     TakeTimeSteps (LIBRARY/bsamroutines.f90:763-775, :846-868, :918-963)
 *     with the plugin's AfterStep2D/3D (PROBLEM/CH/problem.f90:149-215 and
 *     Energy2D :518-547; PROBLEM/BioGrowth/problem.f90:107-152) as one
 *     device reduction over levels 0..finestlevel: integral[0] = the
 *     integral of phi (variable 1), integral[1] = the CH 2D energy (0 for
 *     the other plugins), *meshsize = the composite cell count.  A level > 0
 *     patch subtracts its parent's cells under it, as the reference does.
 *     BioGrowth 3D reports zeros (its AfterStep3D is empty); the growth
 *     plugin reports the integral of phi.  Sums are a fixed-order tree
 *     (deterministic; equal to the reference's sequential SUM to rounding).
 * bsamg_write_q -> WriteQ, LIBRARY/bsaminputoutput.f90:60-181: the text
 *     frame file (F25.12 reals, I3/I8 integers, one record per ghosted cell)
 *     of levels 0..finestlevel, patches in visiting order; the caller names
 *     the file (the reference uses ./OUT/mNNNNN.dat).
 * bsamg_write_uniform_q -> WriteUniformMeshQ, :446-572: the composite
 *     solution on one uniform grid at the finest spacing (root prolonged with
 *     the mass-corrected bilinear/trilinear operator, each level's patches
 *     copied over it), computed on the device and written as one patch.
 * bsamg_read_q -> ReadQ, :184-443: restart from a frame file.  `root` is a
 *     committed hierarchy holding the run's root grid and the levels below it
 *     (bsamg_build_uniform); the new hierarchy copies it, takes the root's
 *     q(0:mx+1) from the file (a second ghost layer, mbc = 2, keeps the
 *     root's values; the records are q(0:mx+1) whatever mbc is, as WriteQ
 *     writes them) and adds the file's refinement
 *     patches (ids first_id, first_id + 1, ...; each parented by the patch of
 *     the level below that contains it; qold = q).  The root block is checked
 *     as ReadQ checks it (ndims, ratio 2, nrvars, dx, xlower, xupper, mx,
 *     mglobal); a mismatch or a malformed file returns BSAMG_ERR_IO.  *time
 *     receives the frame's time.
 * bsamg_format_f25_12 -> one F25.12 field (25 characters + NUL into out).
 * bsamg_format_stats_line -> one OUT/stats.dat record,
 *     '(3(F25.12),1x,I8)' (bsamroutines.f90:771-775), newline included. */
int bsamg_after_step_stats(bsamg_hier* h, int finestlevel, double integral[2], long long* meshsize);
int bsamg_write_q(bsamg_hier* h, const char* path, double time, int finestlevel);
int bsamg_write_uniform_q(bsamg_hier* h, const char* path, double time, int finestlevel);
int bsamg_read_q(bsamg_hier* root, const char* path, int first_id, double* time, bsamg_hier** out);
int bsamg_format_f25_12(double x, char* out);
int bsamg_format_stats_line(double time, const double integral[2], long long meshsize, char* out, size_t n);

/* The seeded spinodal start of the benchmark configurations, generated on
 * the device for one CH patch (no reference counterpart: it stands in for
 * the plugin's QInit2D/3D, CH/problem.f90:45-146, with the project's seeded
 * inputs): phi = mean + amp*U(-1,1), U = splitmix64(seed ^ (g * 0x9E3779B9
 * 7F4A7C15)) mapped to (-1,1) with g the cell's index within the patch
 * (i fastest); mu = phi^3 - phi - eps^2 Lap_h(phi), the Laplacian wrapped
 * over the patch; ghost layers zero.  Enqueued on the hierarchy's stream;
 * bit-identical to the host generator of the same definition. */
int bsamg_seed_spinodal(bsamg_hier* h, int id, unsigned long long seed, double mean, double amp);

/* Wait for all work of the hierarchy; returns the first deferred error. */
int bsamg_sync(bsamg_hier* h);
/* CUDA stream the hierarchy launches on (cudaStream_t as void*), for
 * callers that time or order work around it. */
int bsamg_stream(bsamg_hier* h, void** stream);
/* Kernel launches issued by this hierarchy since creation. */
int bsamg_launch_count(const bsamg_hier* h, long long* n);
/* CUDA graphs this hierarchy instantiated, and graphs it took over from the
 * hierarchy it was regridded from and updated in place. */
int bsamg_graph_stats(const bsamg_hier* h, int* instantiated, int* updated);
/* Reuse of a committed hierarchy for another run on the same mesh (no
 * reference counterpart; a serving loop keeps hierarchies of recurring
 * shapes instead of building them again).  bsamg_set_params replaces the
 * plugin parameters (same meaning and count rules as bsamg_hier_create) and
 * recomputes the per-patch coefficients; bsamg_hier_reset returns every
 * field to the zero fill of bsamg_commit.  Both are stream-ordered: work
 * already enqueued runs with the old values.  After both, a run gives the
 * same results as on a newly built hierarchy. */
int bsamg_set_params(bsamg_hier* h, const double* params, int nparams);
int bsamg_hier_reset(bsamg_hier* h);
/* Tuning (no reference counterpart): the smoothing of 3D levels on the
 * periodic-box mixed path.  0: colour sweeps, each thread relaxing two
 * rows' cells; 1: four rows' cells, all loads issued before any store;
 * 2: rows staged in shared memory by bulk asynchronous copies, for rows of
 * 128 to 512 cells (measured slower than 1 on a GB300; kept as the staged
 * alternative; it sums the neighbours in another order); 3 (the default):
 * a level visit's V(2,2) smoothing (four colour half-sweeps) as one pass
 * over z-planes staged in shared memory, on levels with rows of 256 cells,
 * and the four-row sweeps elsewhere.  0, 1 and 3 give the same bits.
 * Drops the hierarchy's captured graphs. */
int bsamg_set_box_sweep(bsamg_hier* h, int kind);
/* Tuning (no reference counterpart): the mixed V-cycle runs its coarse
 * tail -- the levels from minlevel up to the highest one at which the
 * levels together hold at most `cells` interior cells -- inside one thread
 * block, one launch instead of ~20 per level; results are bit-identical.
 * Default 2048, where one block is still as fast as the launches it
 * replaces; a larger value trades a single run's latency for throughput
 * when many hierarchies share the GPU.  0 disables.  Drops the hierarchy's
 * captured graphs. */
int bsamg_set_tail_cells(bsamg_hier* h, long long cells);
/* Tuning (no reference counterpart; replaces the loop of
 * MultigridIterations, afasroutines.f90:78-104, and the ApplyOnLevel loops
 * of AFASVcycle, :495-529, on the mixed path of adaptive hierarchies).
 * mode 1 (the default): a mixed-mode solve whose finest level is above 0
 * runs as ONE launch of one thread-block cluster -- every operation of
 * every V-cycle, the FP64 residual and the exit test on the device -- with
 * `ctas` CTAs of `threads` threads (ctas 1..16, threads 256, 512 or 1024),
 * the FP32 work lists cut into tiles of `tile` units (32, 64, 128 or 256:
 * a tile is the work of one group of `tile` threads, so small patches keep
 * few threads idle); the levels from minlevel up to the highest one at
 * which they hold at most `solo_cells` interior cells together run in one
 * CTA of the cluster (0: none).  Defaults 16 x 512, tiles of 64, 8192
 * cells.  Same iterates, V-cycle counts and residuals, bit for bit, as
 * mode 0, which launches every operation on its own from captured graphs.
 * BSAMG_ERR_UNSUPPORTED when the device cannot run a cluster of that
 * shape.  The settings carry over to the hierarchies bsamg_regrid makes
 * from this one. */
int bsamg_set_solve(bsamg_hier* h, int mode, int ctas, int threads, int tile, long long solo_cells);
int bsamg_get_solve(const bsamg_hier* h, int* mode, int* ctas, int* threads, int* tile, long long* solo_cells);
/* Profiling of the one-launch solve (no reference counterpart).  With the
 * trace enabled, the next solves record CTA 0's clock (cycles of its SM)
 * at the end of every phase of the program's prologue and first outer
 * iteration; bsamg_solve_trace_read returns, for each of the `count` phases
 * of the last traced solve (up to cap), its operation code (0-5 the FP32
 * V-cycle's relax, restrict, ring, load, prolong, ghost; 8-15 clear, prep,
 * update, FP64 FillDown, FP64 ghost, norm, finish, solo block), its work
 * size (blocks, or ghost stages) and the cycles since the previous phase
 * ended (a solo block's time is given on its last phase, 0 on the others). */
int bsamg_solve_trace(bsamg_hier* h, int enable);
/* The last one-launch solve program of the hierarchy: info[0] phases,
 * [1] first phase of the loop body, [2] levels whose FP32 arrays it keeps in
 * the cluster's distributed shared memory, [3] bytes of that data area per
 * CTA, [4] bytes of the program image each CTA stages, [5] CTAs, [6]
 * threads per CTA, [7] 1 when the last program was too large to stage (the
 * per-launch path ran); the last solve's host clock in microseconds: [8]
 * building its program (0 when it was cached), [9] launch to finish, [10]
 * reading the results back.  Up to n of the 11 values. */
int bsamg_solve_info(const bsamg_hier* h, long long* info, int n);
/* Host clock (ms) of the regrid that made hierarchy h (no reference
 * counterpart: measurement): [0] download of q, [1] the host model
 * (tagging, clustering, the new patches' values), [2] creating and
 * committing the new hierarchy, [3] the upload; [4] and [5] the part of [2]
 * spent compiling ghost programs and the rest of the commit; [6] .. [11]
 * the parts of [1], summed over levels: ghost fill, tagging and buffer
 * lists, edge-tag inflation, clustering, the new patches and their values,
 * TransferValues.  n entries are written (at most 12). */
int bsamg_regrid_timing(const bsamg_hier* h, double* ms, int n);
/* Autotuner of the mixed solve of adaptive hierarchies (no reference
 * counterpart).  While on (the default), the first mixed solve of an
 * adaptive hierarchy whose size class (plugin, dimension, variables, levels
 * in the V-cycle, binary order of magnitude of the cells on levels >= 0)
 * the context has not seen times one V-cycle of each candidate -- the
 * per-launch path, and the one-launch solve with 16 CTAs of 256, 512 or
 * 1024 threads, tiles of 32, 64 or 128 units and 2048 or 8192 cells run by
 * one CTA -- each from the same q, which it restores: the solve's result is
 * unchanged.  The fastest is used and kept in the context for that class; a
 * hierarchy whose shape was set by bsamg_set_solve is not tuned.
 * bsamg_tune_save writes the context's choices as JSON (ctas 0: the
 * per-launch path), bsamg_tune_load adds those of a file written by it
 * (BSAMG_ERR_IO for anything else), bsamg_tune_count returns how many
 * classes the context holds. */
int bsamg_ctx_set_autotune(bsamg_ctx* ctx, int on);
int bsamg_tune_save(bsamg_ctx* ctx, const char* path);
int bsamg_tune_load(bsamg_ctx* ctx, const char* path);
int bsamg_tune_count(const bsamg_ctx* ctx, int* n);
int bsamg_solve_trace_read(const bsamg_hier* h, int cap, int* op, int* n, long long* cycles, int* count);

/* Timing support (no reference counterpart: measurement hooks).
 * bsamg_mark records CUDA event `slot` (0..63) on the hierarchy's stream;
 * bsamg_elapsed_ms waits for event b and returns the time from a to b. */
int bsamg_mark(bsamg_hier* h, int slot);
int bsamg_elapsed_ms(bsamg_hier* h, int a, int b, double* ms);
/* Launches the smoother of `level` reps times in the given mode on the
 * current state and returns the mean device time of one launch; the state
 * is modified.  A launch is one colour half-sweep (alternating red and
 * black), or, where the periodic-box mixed path smooths the level in one
 * pass (bsamg_set_box_sweep 3), one V(2,2) smoothing. */
int bsamg_time_smoother(bsamg_hier* h, int level, int mode, int reps,
                        double* ms_per_launch);
/* Colour half-sweeps one launch of that smoother performs (1, or 4 for the
 * one-pass smoothing). */
int bsamg_smoother_colours(bsamg_hier* h, int level, int mode, int* colours);

/* Allocation-free convergence norm of one CH patch.  No counterpart in the
 * reference: it exists for callers that cannot let a library call
 * cudaMalloc -- hosts whose device memory is owned by their own allocator
 * (a PyTorch caching allocator, a Fortran code with a fixed device-memory
 * plan) and serving loops that must not trigger the device-wide
 * synchronisation cudaMalloc/cudaFree imply while other streams run.
 * q (one ghost layer, q(0:mx+1, ..., 1:2), the slice the reference passes
 * to Operator2D/3D) and f (interior) are the caller's device arrays in the
 * Fortran layout above; the ErrorAFAS norm (errortype 1 or 2) is written
 * to the caller's device double *norm_out, on `stream` (a cudaStream_t, or
 * NULL for the default stream).  The call allocates nothing: its block
 * partial sums live in a fixed file-scope device array, so a patch may have
 * at most BSAMG_NOALLOC_MAX_CELLS interior cells (larger patches return
 * BSAMG_ERR_ARG).  Every call on a device shares that array, so calls whose
 * kernels overlap on the GPU race; order them on one stream.  The first call
 * on a device looks up the array's address and keeps it for the process:
 * make it before any stream capture, and do not call this entry point on a
 * device after cudaDeviceReset.  Same per-block partials and final
 * reduction as bsamg_residual_norm, so it agrees with it bit for bit on the
 * same data.  A NaN or Inf in the data gives a NaN or Inf norm (there is no
 * separate non-finite flag). */
#define BSAMG_NOALLOC_MAX_CELLS 16777216
int bsamg_ch_residual_norm_noalloc(const double* q, const double* f,
                                   int ndims, const int mx[3], double h,
                                   double dt, double eps, int errortype,
                                   double* norm_out, void* stream);

/* Page-locks (pins) an existing host buffer so put/get copies run at full
 * PCIe/NVLink-C2C speed; a Fortran host can pin its node arrays once. */
int bsamg_host_register(void* ptr, size_t bytes);
int bsamg_host_unregister(void* ptr);

const char* bsamg_strerror(int status);
/* Last CUDA error text seen by the library (thread-local), or "". */
const char* bsamg_last_error_detail(void);

#ifdef __cplusplus
}
#endif
#endif
