// Registry of the problem plugins linked into the library (see plugin.h).
// Plugins register from static initialisers while the library loads, before
// any entry point can run; lookups afterwards only read.
#include <cstring>
#include <mutex>

#include "../../include/bsamg.h"
#include "plugin.h"

namespace bsamg {

namespace {

struct Registry {
  std::mutex mu;
  Plugin slot[kMaxPlugins];
  const PluginMixed* mixed[kMaxPlugins] = {};
};

Registry& registry() {
  static Registry r;
  return r;
}

}  // namespace

int register_plugin_fp64(const Plugin& p) {
  if (p.kind <= 0 || p.kind >= kMaxPlugins || !p.name || !p.fp64) return -1;
  Registry& r = registry();
  std::lock_guard<std::mutex> lk(r.mu);
  if (r.slot[p.kind].fp64) return -1;  // the kind is taken
  r.slot[p.kind] = p;
  r.slot[p.kind].mixed = r.mixed[p.kind];  // the mixed part may have registered first
  return 0;
}

int register_plugin_mixed(int kind, const PluginMixed* m) {
  if (kind <= 0 || kind >= kMaxPlugins) return -1;
  Registry& r = registry();
  std::lock_guard<std::mutex> lk(r.mu);
  r.mixed[kind] = m;
  r.slot[kind].mixed = m;
  return 0;
}

const Plugin* find_plugin(int kind) {
  if (kind <= 0 || kind >= kMaxPlugins) return nullptr;
  const Plugin& p = registry().slot[kind];
  return p.fp64 ? &p : nullptr;
}

const Plugin* find_plugin_by_name(const char* name) {
  if (!name) return nullptr;
  for (int k = 1; k < kMaxPlugins; k++) {
    const Plugin* p = find_plugin(k);
    if (p && std::strcmp(p->name, name) == 0) return p;
  }
  return nullptr;
}

}  // namespace bsamg

extern "C" int bsamg_problem_kind(const char* name, int* kind) {
  const bsamg::Plugin* p = bsamg::find_plugin_by_name(name);
  if (!p || !kind) return BSAMG_ERR_NOT_FOUND;
  *kind = p->kind;
  return BSAMG_OK;
}

extern "C" int bsamg_problem_info(int kind, int* nrvars, int* nparams, int* has_mixed) {
  const bsamg::Plugin* p = bsamg::find_plugin(kind);
  if (!p) return BSAMG_ERR_NOT_FOUND;
  if (nrvars) *nrvars = p->nvars;
  if (nparams) *nparams = p->nparams;
  if (has_mixed) *has_mixed = p->mixed ? 1 : 0;
  return BSAMG_OK;
}
