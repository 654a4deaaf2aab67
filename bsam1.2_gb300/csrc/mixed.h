// Mixed-precision path: FP32 smoothing and prolongation inside an FP64
// defect-correction loop (see mixed.cu).
#pragma once
#include <cstddef>

#include "hier.h"

namespace bsamg {

size_t mixed_pool_bytes(const Hier& H);
int mixed_alloc(Hier& H);
void mixed_free(Hier& H);
// work lists of the mixed path, after the level tables exist
int mixed_tables(Hier& H);
// MultigridIterations in the mixed mode (after the common prologue:
// FillDown(q), sources, FillDown(f)); same contract as the FP64 loop
int mixed_iterations(Hier& H, int finest, int minlevel, int nsmooth, int maxvcycles, double tol, int errortype,
                     int strict, int* ncycles, double* residuals);
// choose the coarse tail of the mixed V-cycle: levels from minlevel up to
// the highest one at which the cumulative interior cell count is at most
// `cells` run inside one CTA (0 disables)
void set_tail(Hier& H, long long cells);
// one outer iteration of the one-launch solve in the current shape, timed
// with CUDA events on the hierarchy's stream (ms); changes q
int solve_time_one_cycle(Hier& H, int finest, int minlevel, int nsmooth, int errortype, double* ms);
bool solve_applies(const Hier& H, int finest);
// the autotuner (tune.cu): the shape of the one-launch solve for this
// hierarchy's size class, from the context's cache or measured now
int solve_autotune(Hier& H, int finest, int minlevel, int nsmooth, int errortype);
// drop the one-launch solve's program image (rebuilt on its next use)
void solve_invalidate(Hier& H);
// whether the device runs the one-launch solve's cluster in this shape
bool solve_shape_runs(const Hier& H, SolveShape sh);
// one FP32 colour sweep of the correction smoother on `level`
int mixed_enq_relax(Hier& H, int level, int ipass);

}  // namespace bsamg
