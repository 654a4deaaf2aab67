// Included by a problem plugin file (plugins/<name>.cu) after nothing else:
// brings in the contract (plugin.h), the cell helpers and the kernel
// templates of the part being compiled, and defines BSAMG_PLUGIN(PL), which
// registers the plugin struct PL when the library loads.
//
// A plugin file is compiled twice: with -DBSAMG_PART_FP64 and --fmad=false
// (the plain FP64 path, evaluated in the reference's order) and with
// -DBSAMG_PART_MIXED and the default --fmad=true (the mixed path's
// correction form, if the plugin has one).
#pragma once
#include "../../include/bsamg.h"
#include "cellops.cuh"
#include "plugin.h"
#if defined(BSAMG_PART_FP64)
#include "kern_fp64.cuh"
#elif defined(BSAMG_PART_MIXED)
#include "kern_mixed.cuh"
#else
#error "compile a plugin file with -DBSAMG_PART_FP64 (and --fmad=false) or -DBSAMG_PART_MIXED"
#endif

namespace bsamg {

#if defined(BSAMG_PART_FP64)
template <class PL>
int register_part() {
  Plugin p;
  p.kind = PL::kKind;
  p.name = PL::kName;
  p.nvars = PL::kNV;
  p.nparams = PL::kNParams;
  p.coeffs_only = PL::kCoeffsOnly;
  p.box = PL::kBox;
  p.set_params = &PL::set_params;
  p.coefficients = &PL::coefficients;
  p.bc_mask = &PL::bc_mask;
  p.stats = &PL::stats;
  p.fp64 = fp64_ops<PL>();
  return register_plugin_fp64(p);
}
#else
template <class PL>
int register_part() {
  if constexpr (PL::kMixed) return register_plugin_mixed(PL::kKind, mx::mixed_ops<PL>());
  return 0;
}
#endif

}  // namespace bsamg

// invoked inside namespace bsamg, after the plugin struct
#define BSAMG_PLUGIN(PL) static const int bsamg_plugin_registered_##PL = register_part<PL>();
