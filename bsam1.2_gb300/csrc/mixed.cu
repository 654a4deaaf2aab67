// Mixed-precision path (placeholder until the FP32 kernels land).
#include "mixed.h"

namespace bsamg {

size_t mixed_pool_bytes(const Hier&) { return 0; }
int mixed_alloc(Hier&) { return BSAMG_OK; }
void mixed_free(Hier&) {}
int mixed_prepare(Hier&, int, int) { return BSAMG_ERR_UNSUPPORTED; }
int mixed_enq_iteration(Hier&, int, int, int, int) { return BSAMG_ERR_UNSUPPORTED; }

}  // namespace bsamg
