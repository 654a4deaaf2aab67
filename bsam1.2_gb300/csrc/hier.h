// Host-side hierarchy state of libbsamg (not part of the C ABI).
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <functional>
#include <map>
#include <mutex>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "../../include/bsamg.h"
#include "internal.h"
#include "launch.h"
#include "plugin.h"

namespace bsamg {

struct HostPatch {
  int level, id, parent_id, parent;
  int mx[3], mglobal[3][2], mbounds[3][2], mthbc[6];
  double dx[3], xlower[3];
  int cmx[3], qn[3], cn[3];
  long long oq, oqold, oqc, of, orf, oftmp;
  long long sq, sc, sf;
  // mixed-path FP32 offsets (into the float pool)
  long long e_oq, e_oqc, e_of, e_orf, e_ophi;
};

// A compiled SetGhost(level, ipass): operations sorted by stage.
struct GhostProg {
  std::vector<GhostOp> ops;
  std::vector<int> stage_off;  // size nstages+1
  GhostOp* d_ops = nullptr;
  int* d_stage_off = nullptr;
};

struct LevelT {
  std::vector<int> patches;  // visiting order
  Blk* d_blk[kNKind] = {};
  int nblk[kNKind] = {};
  std::vector<Blk> h_blk[kNKind];  // host copies (program images of the one-launch solve)
  GhostProg gp[3];           // ipass 0, 1, 2
  double count = 0.0;        // nrvars * cells (ErrorAFAS denominator)
};

struct Hier;
// f(0) .. f(n-1) on the library's host thread pool and the calling thread
// (pool.cpp); returns when all are done
void parallel_for(int n, const std::function<void(int)>& f);
// Inputs of the ghost compiler.
std::vector<GhostOp> compile_set_ghost(const Hier& H, int level, int ipass, std::vector<int>& stage_off);
// the programs of several (level, ipass) jobs at once, every emission item
// of every job on the thread pool
void compile_set_ghost_all(const Hier& H, const std::vector<std::pair<int, int>>& jobs,
                           std::vector<std::vector<GhostOp>*> out, std::vector<std::vector<int>*> stage_off);
// the same writes unprocessed, in the reference's order (for sequential
// execution on the host)
std::vector<GhostOp> set_ghost_sequence(const Hier& H, int level, int ipass);

struct Hier {
  bsamg_ctx* ctx = nullptr;
  int ndims = 2, nrvars = 2, mbc = 1, problem = 1;
  ProbParams pp{};
  std::vector<double> params;  // as given to bsamg_hier_create
  bool has_root_xupper = false;  // built by bsamg_build_uniform: the root's xupper
  double root_xupper[3] = {};
  std::vector<HostPatch> patches;
  std::unordered_map<int, int> id2idx;
  bool committed = false;
  int minlevel = 0, maxlevel = 0;
  int periodic = 0, nperoff = 0, peroffidx[13] = {};
  int mxmax[kMaxDepth + 1][3] = {};

  PatchDev* dP = nullptr;
  std::vector<PatchDev> hP;  // host copy of the patch table
  double* pool = nullptr;
  size_t pool_elems = 0;
  long long q_region = 0, q_len = 0, qold_region = 0;
  float* fpool = nullptr;
  size_t fpool_elems = 0;
  size_t e_len = 0;  // leading FP32 elements holding every patch's correction e
  size_t e_coarse_off = 0, e_coarse_len = 0;  // the part of it on levels < 0
  Blk* mx_norm_blk[kNLev] = {};               // padded interior lists (mixed norm)
  Blk* mx_prep_coarse = nullptr;              // interior lists of all levels < 0
  int mx_prep_coarse_n = 0;
  std::vector<Blk> h_mx_norm_blk[kNLev], h_mx_prep_coarse;  // host copies of the two
  // coarse tail of the V-cycle (levels <= tail_level run in one CTA); the
  // recorded programs per (minlevel, nsmooth): device phases and their count
  int tail_level = -kMaxDepth - 2;
  long long tail_cells = 2048;  // latency-friendly; a serving loop may raise it
  // keys: (start level, minlevel, nsmooth) for V-cycles, (start level,
  // minlevel, -field) for FillDown
  using TailKey = std::tuple<int, int, int>;
  struct TailProg {
    void* phases = nullptr;  // TailPhase[nph]
    int nph = 0;
    // when the tail levels' arrays fit, they are staged in the block's
    // shared memory: a patch table whose tail patches address it, and the
    // copy segments (StageSeg[nsegs]); smem_bytes = 0 otherwise
    void* shadow = nullptr;
    std::vector<PatchDev> hshadow;  // host copy (coefficients follow bsamg_set_params)
    void* segs = nullptr;
    int nsegs = 0;
    int smem_bytes = 0;
  };
  std::map<TailKey, TailProg> mx_tail_progs, fp_tail_progs;
  void* rec = nullptr;  // std::vector<TailPhase> being recorded
  // while a solve program is recorded: the V-cycle level from which CTA 0
  // runs the coarse end alone (a kTSolo marker precedes those phases)
  int rec_solo = -kMaxDepth - 2;
  // the mixed solve of a hierarchy with refinement levels as one cluster
  // launch (kern_solve.cuh): mode 1 uses it where it applies, 0 keeps the
  // per-launch graphs; its launch shape and the cells of the coarse end run
  // by one CTA; the recorded program of (finest, minlevel, nsmooth, solo
  // level) and the device control block (SolveCtl + residuals)
  int solve_mode = 1;
  SolveShape solve_shape{16, 512, 64};
  long long solve_solo_cells = 8192;
  bool solve_tuned = false;     // the caller set the shape (bsamg_set_solve): not tuned
  bool solve_launches = false;  // the autotuner chose the per-launch path for this hierarchy
  void* solve_img = nullptr;  // program image (SolveImage layout)
  SolveImage solve_im{};
  bool solve_nofit = false;   // the program of solve_key is too large to stage
  double solve_ms[3] = {};    // last solve, host clock: program build, launch to finish, read-back
  int solve_nph = 0, solve_body = 0, solve_nb = 0;
  std::tuple<int, int, int, int, int> solve_key{kMaxDepth + 1, 0, 0, 0, 0};
  GhostOp* solve_ops = nullptr;  // the program's FP32 ghost operations, each stage in owner order
  int solve_dsm_levels = 0;      // levels whose FP32 arrays the program keeps in distributed shared memory
  void* solve_ctl = nullptr;
  int solve_ctl_cap = 0;  // residual slots of solve_ctl
  // host clock of the regrid that made this hierarchy (ms): download of q,
  // the host model (tagging, clustering, new patches' values), creating and
  // committing the new hierarchy, the upload; and of commit: the ghost
  // programs' compilation, everything else
  double regrid_ms[12] = {};
  bool solve_trace_on = false;
  long long* solve_trace = nullptr;  // device, solve_trace_cap + 1 clocks
  int solve_trace_cap = 0;
  std::vector<long long> solve_trace_h;  // the last traced solve's clocks
  std::vector<int> solve_trace_ops, solve_trace_n;  // op and n of each phase
  // periodic-box mixed path (box.cu): every level one periodic box with even
  // extents covering its parent; FP64 iterate held as float pairs
  bool box = false;
  // 3D box smoothing (box.cu): colour sweeps of two (0) or four (1) rows a
  // thread or rows staged by bulk copies (2); 3: a level's V(2,2) smoothing in
  // one pass where it applies, four-row sweeps elsewhere
  int box_sweep = 3;
  // the box path's g holds the true residual of the finest level at the
  // current q for the f in fhi/flo (set when box_iterations returns; any
  // entry point that changes fields or coefficients clears it)
  bool box_g_valid = false;
  int box_sms = 152;      // multiprocessors of the device (persistent grids)
  BoxLev blev[kNLev] = {};
  long long b_oqlo = 0, b_ofhi = 0, b_oflo = 0;  // float offsets (qhi is blev[finest].opb)
  size_t b_partials = 0;                         // partial-sum slots the box kernels need
  // the box path's solve as one graph launch: a device-side loop of
  // V-cycles with the exit test on the device (box.cu box_loop_graph)
  cudaGraphExec_t box_loop = nullptr;
  std::tuple<int, int, int, int> box_loop_key{};
  long long box_loop_n1 = 0, box_loop_n2 = 0;  // launches per cycle, per confirming residual
  bool box_loop_off = false;                   // the loop graph could not be built: host loop
  void* box_ctl = nullptr;                     // device control block of the loop
  size_t bytes = 0;
  size_t reserved = 0;  // bytes counted against the context budget

  LevelT lev[kNLev];
  cudaStream_t s = nullptr;
  double* d_partial = nullptr;
  int partial_cap = 0;
  double* d_norm = nullptr;      // [0] norm, [1] raw sum, plus scratch
  int* d_nonfinite = nullptr;
  int pinned_slot = -1;
  double* h_norm = nullptr;      // pinned (a slot of the context's pool)
  int* h_nonfinite = nullptr;    // pinned
  long long launches = 0;
  bool capturing = false;
  long long capture_launches = 0;

  struct GraphRec {
    cudaGraphExec_t exec = nullptr;
    long long nlaunch = 0;
  };
  std::map<std::tuple<int, int, int, int, int>, GraphRec> graphs;
  // executable graphs of the hierarchy this one was regridded from, updated
  // in place by capture_graph when the launch sequence keeps its shape
  std::map<std::tuple<int, int, int, int, int>, GraphRec> graph_donors;
  int graphs_instantiated = 0, graphs_updated = 0;
  cudaEvent_t marks[64] = {};
  cudaEvent_t done_ev = nullptr;  // blocking-sync event of stream_wait

  LevelT& L(int level) { return lev[level + kMaxDepth]; }
  const LevelT& L(int level) const { return lev[level + kMaxDepth]; }
  LaunchCtx lc() const {
    LaunchCtx c;
    c.P = dP;
    c.pool = pool;
    c.fpool = fpool;
    c.s = s;
    c.pp = pp;
    c.ndims = ndims;
    return c;
  }
};

// schedule helpers shared by the FP64 and mixed paths (hier.cu)
int cuda_fail(cudaError_t e, const char* what);
int after_launch(Hier& H, int n);
int set_device(const Hier& H);
int enq_set_ghost(Hier& H, int level, int ipass);
int enq_fill_down(Hier& H, int field, int finest, int minlevel);
int enq_update_source(Hier& H, int finest);
int enq_norm(Hier& H, int level, int errortype);
int enq_relax(Hier& H, int level, int ipass);
// plugin coefficients for a spacing h (PatchDev::c)
void coefficients(const Hier& H, double h, double* c);
// host tables of an uncommitted hierarchy (parent links, extents, level
// lists, periodic offsets); commit() starts with it
int build_tables(Hier& H);
// xupper of a patch as the reference's frame files carry it (frames.cpp)
double xupper_of(const Hier& H, const HostPatch& P, int d);
// Offset of Fortran cell (0,0,0) from the start of a ghosted q-like (n =
// qn) or qc-like (n = cn) plane: 0 for mbc = 1, one cell of each used
// dimension's stride for mbc = 2 (the arrays start at index 1 - mbc).
// Per-device one-time setup (a kernel attribute): true when device dev has
// not been marked in `done` yet; the caller marks it after the setup
// succeeded.  Repeating the setup from two threads is harmless, the flag
// itself is atomic.
inline bool needs_setup(const std::atomic<unsigned long long>& done, int dev) {
  return !(done.load(std::memory_order_acquire) & (1ull << (dev & 63)));
}
inline void mark_setup(std::atomic<unsigned long long>& done, int dev) {
  done.fetch_or(1ull << (dev & 63), std::memory_order_release);
}
inline long long origin_of(const Hier& H, const int* n) {
  long long s = H.mbc - 1;
  return H.ndims == 2 ? s * (1 + n[0]) : s * (1 + n[0] + (long long)n[0] * n[1]);
}
// units of a level work list of this kind for patch P (blocks of kBlock units)
long long kind_units(const Hier& H, const HostPatch& P, int kind);
// AMR regrid of a committed hierarchy into a new one (regrid.cpp)
int regrid(Hier& H, const bsamg_regrid_params& prm, bsamg_qinit_fn qinit, void* user, bsamg_hier** out);
using GraphKey = std::tuple<int, int, int, int, int>;
// capture what `body` enqueues as a CUDA graph (once per key) and replay it
int capture_graph(Hier& H, const GraphKey& key, const std::function<int()>& body, Hier::GraphRec** out);
int replay(Hier& H, Hier::GraphRec* g);
void drop_graphs(Hier& H);
// wait for the hierarchy's stream (spinning, or sleeping with blocking waits)
int stream_wait(Hier& H);
// release the device arrays of a tail program (stream-ordered)
void free_tail(Hier& H, Hier::TailProg& T);

}  // namespace bsamg

struct bsamg_ctx {
  int device = 0;
  size_t budget = 0;
  size_t used = 0;
  // every device allocation of the context's hierarchies comes from this
  // stream-ordered pool; it keeps freed memory (release threshold = max), so
  // creating and destroying hierarchies neither maps nor unmaps memory
  cudaMemPool_t mempool = nullptr;
  bool blocking_wait = false;  // host waits sleep on an event instead of spinning
  std::mutex mu;
  double* pinned = nullptr;     // pinned read-back words, one slot per hierarchy
  std::vector<int> free_slots;
  // the one-launch solve's autotuner (tune.cu): on, and the launch shape it
  // chose per size class of adaptive hierarchy (kept until the context
  // ends; bsamg_tune_save / bsamg_tune_load persist it as JSON)
  bool autotune = true;
  struct Tuned {
    int ctas, threads, tile;
    long long solo_cells;
    double us_per_cycle;
  };
  std::map<std::vector<int>, Tuned> tuned;
};

struct bsamg_hier : bsamg::Hier {};

namespace bsamg {
// stream-ordered allocation from the context's pool on the hierarchy's stream
inline cudaError_t dev_alloc(const Hier& H, void** p, size_t bytes) {
  return cudaMallocFromPoolAsync(p, bytes, H.ctx->mempool, H.s);
}
}  // namespace bsamg
