// Mixed-precision MultigridIterations on periodic boxes (box.cu).
#pragma once
#include <cstddef>

#include "hier.h"

namespace bsamg {

// every level one fully periodic patch (periodic_single), qpo = 0, even
// extents, each level covering its parent, problem CH
bool box_eligible(const Hier& H, bool periodic_single);
// fills H.blev / H.b_* offsets; returns the float-pool size in elements
size_t box_layout(Hier& H);
// the plugin coefficients of every box level (from the current parameters)
void box_coefficients(Hier& H);
// same contract as the FP64 loop; runs instead of the common prologue
// (it forms f from qold itself); finest must be the hierarchy's finest level
int box_iterations(Hier& H, int finest, int minlevel, int nsmooth, int maxvcycles, double tol, int errortype,
                   int strict, int* ncycles, double* residuals);
// one colour sweep of the FP32 correction smoother on `level`
int box_enq_relax(Hier& H, int level, int ipass);
// colour half-sweeps of one launch of the smoother the V-cycle runs on
// `level` (4 where it smooths in one pass, else 1), and one such launch
// (the one-pass smoothing writes the level's second e array)
int box_smoother_colours(const Hier& H, int level);
int box_enq_smoother(Hier& H, int level, int ipass);

}  // namespace bsamg
