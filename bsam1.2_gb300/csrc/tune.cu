// Autotuner of the mixed solve of adaptive hierarchies (no reference
// counterpart).
//
// The one-launch solve (kern_solve.cuh) has launch parameters whose best
// values depend on the mesh -- threads per CTA, units per tile of the FP32
// work lists (patches of 8-64 cells per side leave most threads of a large
// tile idle; small tiles cost more iterations on large patches) and the
// cells of the coarse end that one CTA runs alone (its phases are cheaper,
// its work serial) -- and on meshes whose levels hold many cells (3D, more
// variables) the FP64 work it does on one cluster's SMs makes the
// per-launch path, which spreads every operation over the whole GPU, the
// faster one.  The first mixed solve of a hierarchy whose size class the
// context has not seen times one outer iteration of every candidate (the
// per-launch path included) on the host clock, each from the same copy of
// q, and restores q afterwards, so the solve itself is unchanged: every
// candidate computes the same iterates.  The winner is kept in the context
// for the size class -- plugin, dimension, variables, levels in the V-cycle
// and the binary order of magnitude of the cells on the levels >= 0 -- so
// the hierarchies a regrid makes every step reuse it; bsamg_tune_save /
// bsamg_tune_load keep it across runs as JSON.  Clusters are 16 CTAs: the
// widest cluster was the fastest on every mesh measured.
#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "hier.h"
#include "mixed.h"

namespace bsamg {

namespace {

int log2_floor(long long x) {
  int k = 0;
  while (x > 1) {
    x >>= 1;
    k++;
  }
  return k;
}

std::vector<int> size_class(const Hier& H, int finest, int minlevel) {
  long long cells = 0;
  int npatch = 0;
  for (int l = 0; l <= finest; l++)
    for (int p : H.L(l).patches) {
      const HostPatch& P = H.patches[p];
      cells += (long long)P.mx[0] * P.mx[1] * P.mx[2];
      npatch++;
    }
  (void)npatch;
  return {H.problem, H.ndims, H.nrvars, finest - minlevel + 1, log2_floor(cells)};
}

// a shape of the one-launch solve, or (ctas = 0) the per-launch path
struct Candidate {
  SolveShape shape;
  long long solo;
};

std::vector<Candidate> candidates() {
  std::vector<Candidate> v;
  v.push_back(Candidate{SolveShape{0, 0, 0}, 0});
  for (int threads : {256, 512, 1024})
    for (int tile : {32, 64, 128})
      for (long long solo : {2048LL, 8192LL}) v.push_back(Candidate{SolveShape{16, threads, tile}, solo});
  return v;
}

// one outer iteration of the per-launch path (ms, host clock)
int time_launches(Hier& H, int finest, int minlevel, int nsmooth, int errortype, double* ms) {
  const int mode = H.solve_mode;
  H.solve_mode = 0;
  auto t0 = std::chrono::steady_clock::now();
  int n = 0;
  int r = mixed_iterations(H, finest, minlevel, nsmooth, 1, 0.0, errortype, 0, &n, nullptr);
  if (r == BSAMG_OK) r = stream_wait(H);
  *ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  H.solve_mode = mode;
  return r;
}

}  // namespace

int solve_autotune(Hier& H, int finest, int minlevel, int nsmooth, int errortype) {
  if (!solve_applies(H, finest)) return BSAMG_OK;
  std::vector<int> key = size_class(H, finest, minlevel);
  {
    std::lock_guard<std::mutex> g(H.ctx->mu);
    auto it = H.ctx->tuned.find(key);
    if (it != H.ctx->tuned.end()) {
      const bsamg_ctx::Tuned& t = it->second;
      if (t.ctas == 0) {
        H.solve_launches = true;
        return BSAMG_OK;
      }
      SolveShape sh{t.ctas, t.threads, t.tile};
      if (solve_shape_runs(H, sh)) {
        H.solve_launches = false;
        H.solve_shape = sh;
        H.solve_solo_cells = t.solo_cells;
        return BSAMG_OK;
      }
    }
  }
  // every candidate starts from the same q; the original comes back at the end
  double* snap = nullptr;
  size_t qbytes = sizeof(double) * (size_t)H.q_len;
  cudaError_t e = dev_alloc(H, (void**)&snap, qbytes);
  if (e == cudaSuccess) e = cudaMemcpyAsync(snap, H.pool + H.q_region, qbytes, cudaMemcpyDeviceToDevice, H.s);
  if (e != cudaSuccess) return cuda_fail(e, "autotune snapshot");
  const SolveShape keep = H.solve_shape;
  const long long keep_solo = H.solve_solo_cells;
  double best = 1e30;
  Candidate win{keep, keep_solo};
  int rc = BSAMG_OK;
  for (const Candidate& c : candidates()) {
    const bool launches = c.shape.ctas == 0;
    if (!launches && !solve_shape_runs(H, c.shape)) continue;
    if (!launches) {
      H.solve_shape = c.shape;
      H.solve_solo_cells = c.solo;
    }
    double t = 1e30;
    for (int rep = 0; rep < 2 && rc == BSAMG_OK; rep++) {
      e = cudaMemcpyAsync(H.pool + H.q_region, snap, qbytes, cudaMemcpyDeviceToDevice, H.s);
      if (e != cudaSuccess) {
        rc = cuda_fail(e, "autotune restore");
        break;
      }
      double ms = 0.0;
      int r = launches ? time_launches(H, finest, minlevel, nsmooth, errortype, &ms)
                       : solve_time_one_cycle(H, finest, minlevel, nsmooth, errortype, &ms);
      if (r == BSAMG_ERR_UNSUPPORTED) break;  // the program does not fit this shape's staging
      if (r) {
        rc = r;
        break;
      }
      t = std::min(t, ms);
    }
    if (rc) break;
    if (t < best) {
      best = t;
      win = c;
    }
  }
  e = cudaMemcpyAsync(H.pool + H.q_region, snap, qbytes, cudaMemcpyDeviceToDevice, H.s);
  cudaFreeAsync(snap, H.s);
  if (rc) {
    H.solve_shape = keep;
    H.solve_solo_cells = keep_solo;
    return rc;
  }
  if (e != cudaSuccess) return cuda_fail(e, "autotune restore");
  H.solve_launches = win.shape.ctas == 0;
  if (H.solve_launches) {
    H.solve_shape = keep;
    H.solve_solo_cells = keep_solo;
  } else {
    H.solve_shape = win.shape;
    H.solve_solo_cells = win.solo;
  }
  if (best < 1e30) {
    std::lock_guard<std::mutex> g(H.ctx->mu);
    H.ctx->tuned[key] = bsamg_ctx::Tuned{win.shape.ctas, win.shape.threads, win.shape.tile, win.solo, 1e3 * best};
  }
  return BSAMG_OK;
}

}  // namespace bsamg

using namespace bsamg;

namespace {
// one entry per line, written and read with the same format
const char* kEntry =
    "{\"problem\": %d, \"ndims\": %d, \"nrvars\": %d, \"levels\": %d, \"log2_cells\": %d, "
    "\"ctas\": %d, \"threads\": %d, \"tile\": %d, \"solo_cells\": %lld, \"us_per_cycle\": %lf}";
}  // namespace

int bsamg_ctx_set_autotune(bsamg_ctx* ctx, int on) {
  if (!ctx) return BSAMG_ERR_ARG;
  ctx->autotune = on != 0;
  return BSAMG_OK;
}

int bsamg_tune_save(bsamg_ctx* ctx, const char* path) {
  if (!ctx || !path) return BSAMG_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  FILE* f = std::fopen(path, "w");
  if (!f) return BSAMG_ERR_IO;
  std::fprintf(f, "{\"bsamg_solve_tuning\": 1, \"entries\": [\n");
  size_t k = 0;
  for (const auto& kv : ctx->tuned) {
    const std::vector<int>& c = kv.first;
    const bsamg_ctx::Tuned& t = kv.second;
    std::fprintf(f, k++ ? ",\n  " : "  ");
    std::fprintf(f, kEntry, c[0], c[1], c[2], c[3], c[4], t.ctas, t.threads, t.tile, t.solo_cells, t.us_per_cycle);
  }
  std::fprintf(f, "\n]}\n");
  return std::fclose(f) == 0 ? BSAMG_OK : BSAMG_ERR_IO;
}

int bsamg_tune_load(bsamg_ctx* ctx, const char* path) {
  if (!ctx || !path) return BSAMG_ERR_ARG;
  FILE* f = std::fopen(path, "r");
  if (!f) return BSAMG_ERR_IO;
  std::string text;
  char buf[4096];
  size_t n;
  while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, n);
  std::fclose(f);
  if (text.find("\"bsamg_solve_tuning\": 1") == std::string::npos) return BSAMG_ERR_IO;
  std::lock_guard<std::mutex> g(ctx->mu);
  for (size_t at = text.find("{\"problem\""); at != std::string::npos; at = text.find("{\"problem\"", at + 1)) {
    int c[5], ctas, threads, tile;
    long long solo;
    double us;
    if (std::sscanf(text.c_str() + at, kEntry, &c[0], &c[1], &c[2], &c[3], &c[4], &ctas, &threads, &tile, &solo,
                    &us) != 10)
      return BSAMG_ERR_IO;
    bool launches = ctas == 0;  // the per-launch path
    if (!launches && (ctas < 1 || ctas > 16 || (threads != 256 && threads != 512 && threads != 1024) ||
                      (tile != 32 && tile != 64 && tile != 128 && tile != 256) || solo < 0))
      return BSAMG_ERR_IO;
    ctx->tuned[std::vector<int>(c, c + 5)] = bsamg_ctx::Tuned{ctas, threads, tile, solo, us};
  }
  return BSAMG_OK;
}

int bsamg_tune_count(const bsamg_ctx* ctx, int* n) {
  if (!ctx || !n) return BSAMG_ERR_ARG;
  *n = (int)ctx->tuned.size();
  return BSAMG_OK;
}
