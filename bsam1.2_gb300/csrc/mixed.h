// Mixed-precision path: FP32 smoothing and prolongation inside an FP64
// defect-correction loop (see mixed.cu).
#pragma once
#include <cstddef>

#include "hier.h"

namespace bsamg {

size_t mixed_pool_bytes(const Hier& H);
int mixed_alloc(Hier& H);
void mixed_free(Hier& H);
// once per MultigridIterations call, after the FP64 sources are in place
int mixed_prepare(Hier& H, int finest, int minlevel);
// one outer defect-correction iteration, ending with the FP64 norm copied
// to H.h_norm (captured into a CUDA graph by the caller)
int mixed_enq_iteration(Hier& H, int finest, int minlevel, int nsmooth, int errortype);
// one FP32 colour sweep of the correction smoother on `level`
int mixed_enq_relax(Hier& H, int level, int ipass);

}  // namespace bsamg
