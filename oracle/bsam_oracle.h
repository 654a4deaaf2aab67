/*
 * CPU oracle for the BSAM 1.2 FAS V-cycle on block-structured patches.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * Fortran (LIBRARY/afasroutines.f90, LIBRARY/boundary.f90,
 * LIBRARY/gridutilities.f90, LIBRARY/bsamroutines.f90 RootInit/InitSeed/
 * CopyQToQold/TakeTimeSteps, PROBLEM/CH/problem.f90, PROBLEM/BioGrowth/
 * problem.f90).  Only the tests, the smoke check and the CPU-baseline leg of
 * the benchmark may load it; the product library never links it.
 *
 * Parity status: pinned to the reference itself.  The reference ships no
 * tests, golden vectors or fixtures, and no Fortran compiler exists on the
 * build or GPU machines; its unmodified source is run instead by a
 * Fortran-subset interpreter (oracle/fortran_exec.py), whose outputs on 2D
 * and 3D CH (periodic, Neumann, Dirichlet, two ghost layers), 2D BioGrowth
 * and 2D/3D CH on meshes regridded before every step are committed as
 * fixtures (tests/golden/ref_*.npz, tests/golden/make_reference_golden.py).
 * The oracle reproduces them bit for bit: every node's q after every time
 * step, the residual of every V-cycle, the mesh and the order in which
 * ApplyOnLevel visits it (tests/test_reference_golden_cpu.py).  Math-derived
 * known-answer tests (tests/test_oracle_kat.py) and a numpy transcription of
 * the reference's statements (tests/test_oracle_transcription_cpu.py) check
 * it as well.  The three-variable growth plugin has no reference counterpart
 * and is pinned by exact solutions only.
 *
 * Arithmetic follows the reference's evaluation order term by term and is
 * compiled with -ffp-contract=off (no FMA contraction), so the CUDA plain-FP64
 * path, which uses the same order with explicit round-to-nearest intrinsics,
 * is expected to agree bit for bit except in reductions.
 *
 * Field layout is the reference's Fortran layout (bsamstorage.f90:81-90,
 * :106-115): q(1-mbc:mx1+mbc, 1-mbc:mx2+mbc, [1-mbc:mx3+mbc | 1], 1:nrvars),
 * column-major, variable index slowest.  The same layout is used by the CUDA
 * library's put/get calls, so arrays move between the two unchanged.
 */
#ifndef BSAM_ORACLE_H
#define BSAM_ORACLE_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct bsamo_hier bsamo_hier;

/* problem kinds (same codes as include/bsamg.h) */
#define BSAMO_PROBLEM_CH 1
#define BSAMO_PROBLEM_BIOGROWTH 2
#define BSAMO_PROBLEM_GROWTH 3 /* three variables, no reference counterpart */

/* field codes (same codes as include/bsamg.h) */
#define BSAMO_FIELD_Q 0
#define BSAMO_FIELD_QOLD 1
#define BSAMO_FIELD_QC 2
#define BSAMO_FIELD_F 3
#define BSAMO_FIELD_RF 4
#define BSAMO_FIELD_FTMP 5

/* params: [0]=dt [1]=eps [2]=gamma [3]=lambda [4]=czero [5]=cpress; qpo[nrvars] */
int bsamo_create(int ndims, int nrvars, int mbc, int problem,
                 const double* params, int nparams, const double* qpo,
                 bsamo_hier** out);
int bsamo_destroy(bsamo_hier* h);
int bsamo_patch_add(bsamo_hier* h, int level, int id, int parent_id,
                    const int mx[3], const int mglobal[6],
                    const int mbounds[6], const int mthbc[6],
                    const double dx[3], const double xlower[3]);
/* RootInit (bsamroutines.f90:226-440) + InitSeed (:443-510) for one root
 * grid and levels -1..minlevel below it. */
int bsamo_build_uniform(bsamo_hier* h, const int mx[3], int minlevel,
                        const int mthbc[6], const double xlower[3],
                        const double xupper[3]);
int bsamo_commit(bsamo_hier* h);
int bsamo_num_patches(const bsamo_hier* h);
/* out[0..27]: level,id,parent_id,mx[3],mglobal[6],mbounds[6],mthbc[6],
 * then 4 unused */
int bsamo_patch_info(const bsamo_hier* h, int index, int* out, double* dxl);
size_t bsamo_field_size(const bsamo_hier* h, int id, int field);
int bsamo_put_field(bsamo_hier* h, int id, int field, const double* a,
                    size_t n);
int bsamo_get_field(const bsamo_hier* h, int id, int field, double* a,
                    size_t n);

/* single operations (tier-(i)/(ii) parity) */
int bsamo_relax_level_color(bsamo_hier* h, int level, int ipass);
int bsamo_set_ghost(bsamo_hier* h, int level, int ipass);
int bsamo_level_relax(bsamo_hier* h, int level, int nsmooth);
int bsamo_fill_down(bsamo_hier* h, int field, int finestlevel, int minlevel);
int bsamo_copy_q_to_qold(bsamo_hier* h, int minlevel, int finestlevel);
int bsamo_vcycle(bsamo_hier* h, int level, int minlevel, int nsmooth);
/* CorrectFine on every patch of a level (parent%q - qc, q += P1/P2 of it) */
int bsamo_correct_fine(bsamo_hier* h, int level);
/* a per-patch operation on every patch of a level: RestrictSolution (which
 * = 1), GetCoarseGhostPoints (2), CoarseLoadingFunction (3),
 * GetSourceFunction (4), UpdateSourceFunction (5), FillDownLevel of f (6)
 * or of q (7) */
int bsamo_level_op(bsamo_hier* h, int level, int which);
/* NewSubGrids alone on one patch's flags (x fastest): boxes as (lo, hi) per
 * dimension, at most cap of them into out; returns their number */
int bsamo_new_sub_grids(int nd, const int mx[3], const int* flags, double desfill, int mgp, int* out, int cap);
/* P1MC (mbc = 1) / P2MC (mbc = 2) of one variable: a has cmx+2 mbc cells per
 * used dimension, out 2 cmx + 2 mbc (Fortran order, ghost layers included) */
int bsamo_prolong_mc(int nd, int mbc, const double* a, const int cmx[3], double* out);
int bsamo_residual_norm(bsamo_hier* h, int level, int errortype,
                        double* out);

/* MultigridIterations (afasroutines.f90:48-110).  residuals[maxvcycles]
 * receives ErrorAFAS per V-cycle; *ncycles the number run. */
int bsamo_multigrid_iterations(bsamo_hier* h, int finestlevel, int minlevel,
                               int nsmooth, int maxvcycles, double qerrortol,
                               int updateauxfreq, int errortype,
                               int* ncycles, double* residuals);
/* One TakeTimeSteps step (bsamroutines.f90:657-797) on a fixed mesh:
 * SetGhost(l,0) for l=0..finest, FillDown(q) if first, CopyQToQold,
 * MultigridIterations. */
int bsamo_time_step(bsamo_hier* h, int first, int finestlevel, int minlevel,
                    int nsmooth, int maxvcycles, double qerrortol,
                    int updateauxfreq, int errortype, int* ncycles,
                    double* residuals);

/* AMR regrid: the AMR(rootlevel) pass that TakeTimeSteps runs before every
 * step (bsamroutines.f90:657-689, :966-1951).  Level by level from the root:
 * SetGhost(l,0), tag (CH SetErrFlagsUser2D/3D or the gradient rule), buffer
 * the tags (BufferAndList, InflateEdgeTags with periodic images), cluster
 * the tags of each patch with the modified Berger-Rigoutsos algorithm
 * (NewSubGrids), make the children (MakeNewGrid), fill them (InitFields:
 * the initial condition, or mass-corrected bilinear/trilinear prolongation
 * from the parent) and copy the previous level-(l+1) values over them
 * (TransferValues).  The result is a new committed hierarchy: the levels
 * <= 0 of `old` (all fields copied) and the new levels > 0. */
#define BSAMO_TAG_CH 0       /* CH/problem.f90:248-308: second differences of phi */
#define BSAMO_TAG_GRADIENT 1 /* |grad phi| h > qtolerance, central differences */
typedef struct {
  int maxlevel;
  int tagging;
  int initial;  /* new grids take the initial condition (InitFields :1804) */
  int maxside;  /* 0, or split new patches to at most maxside cells per side */
  int first_id; /* ids of the new patches: first_id, first_id + 1, ... */
  int ibuffer[11];
  int minimumgridpoints[11];
  double qtolerance[11];
  double desiredfillratio[11];
} bsamo_regrid_params;
/* fill the interior of q (ghosted Fortran layout) of a new patch */
typedef void (*bsamo_qinit_fn)(void* user, int level, const int* mx,
                               const double* dx, const double* xlower,
                               double* q);
int bsamo_regrid(const bsamo_hier* old, const bsamo_regrid_params* prm,
                 bsamo_qinit_fn qinit, void* user, bsamo_hier** out);

/* AfterStepStatistics + GetMeshSize over levels finest..0
 * (bsamroutines.f90:763-775, :846-868, :918-963; CH/problem.f90:149-215,
 * :518-547; BioGrowth/problem.f90:107-152): integral[0] = integral of phi,
 * integral[1] = the CH 2D energy (0 elsewhere), *meshsize = composite cells */
int bsamo_after_step_stats(const bsamo_hier* h, int finestlevel, double integral[2], long long* meshsize);
/* WriteQ (bsaminputoutput.f90:60-181): the frame file of levels 0..finest */
int bsamo_write_q(const bsamo_hier* h, const char* path, double time, int finestlevel);
/* WriteUniformMeshQ (bsaminputoutput.f90:446-572) */
int bsamo_write_uniform_q(const bsamo_hier* h, const char* path, double time, int finestlevel);
/* ReadQ (bsaminputoutput.f90:184-443): restart from a frame file; `root`
 * holds the root grid and the levels below it */
int bsamo_read_q(const bsamo_hier* root, const char* path, int first_id, double* time, bsamo_hier** out);
/* one F25.12 field (25 characters and a terminating zero) */
void bsamo_format_f25_12(double x, char out[26]);
/* one record of OUT/stats.dat (bsamroutines.f90:771-775), newline included */
int bsamo_format_stats_line(double time, const double integral[2], long long meshsize, char* out, size_t n);

/* seeded inputs: U(-1,1) from splitmix64 on a global cell index */
double bsamo_uniform_pm1(unsigned long long seed, unsigned long long gidx);

#ifdef __cplusplus
}
#endif
#endif
