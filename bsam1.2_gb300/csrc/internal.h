// Internal types shared by the host side and the kernels of libbsamg.
//
// Device data model (replaces the pointer-linked nodeinfo records of
// LIBRARY/nodeinfodef.f90:118-220 and the per-node ALLOCATEs of
// LIBRARY/bsamstorage.f90:54-144): every field of every patch lives in one
// pooled allocation, addressed by element offsets held in a flat PatchDev
// table.  Each field keeps the reference's Fortran layout, so a whole node
// array moves between host and device with one copy.  All q arrays of a
// hierarchy are contiguous and followed by all qold arrays in the same order,
// so CopyQToQold is a single device-to-device copy.
#pragma once
#include <cstdint>

namespace bsamg {

constexpr int kMaxDepth = 10;            // nodeinfodef.f90:62
constexpr int kNLev = 2 * kMaxDepth + 1; // levels -10..10
constexpr int kInternalBC = 999;         // nodeinfodef.f90:59
constexpr int kMaxVars = 10;             // nodeinfodef.f90:64
constexpr int kBlock = 256;              // threads per block of the cell kernels

struct PatchDev {
  int mx[3];   // interior extents (1 for the unused dimension in 2D)
  int qn[3];   // ghosted extents of q/qold (1 for the unused dimension)
  int cmx[3];  // coarse extents (mx/2, or 1)
  int cn[3];   // ghosted extents of qc
  int mb[3];   // lower mbounds in the parent (1-based)
  int parent;  // index into the patch table, -1 if none
  int level;
  int gs;      // mbc - 1: the ghosted arrays start at Fortran index -gs
  // Read only by the one-launch solve, in the copy of the table in its
  // program image: the CTA of the cluster that works on this patch's FP32
  // arrays, and whether those arrays live in that CTA's shared memory (then
  // eq, ecq, eg and ephi count from the start of its shared-memory data).
  int owner, dsm;
  // element offsets into the pool; for the ghosted arrays (q, qold, qc) the
  // offset of Fortran cell (0,0,0) of variable 1, so that a cell's offset
  // is the same expression whatever mbc is (negative indices reach the
  // second ghost layer when mbc = 2)
  long long oq, oqold, oqc, of, orf, oftmp;
  long long sq, sc, sf;                      // elements per variable plane
  // mixed path, offsets into the FP32 pool: correction e (ghosted, like q;
  // the offset of cell (0,0,0) as above), its coarse image ec (like qc),
  // correction right-hand side g (interior, like f) and the frozen base
  // phase field phib (interior, one plane)
  long long eq, ecq, eg, ephi;
  // Plugin coefficients for this patch's spacing, computed on the host by
  // the plugin's coefficients() with the reference's expressions, e.g.
  //   CH : c0 = dt/h^2, c1 = eps^2/h^2, c2 = (4|6)*eps^2/h^2, c3 = (4|6)*c0
  //        (CH/problem.f90:339-346, :575-582)
  //   Bio: c0 = dt*eps^2/h^2, c1 = 1/h^2, c2 = 4*c0 + 1, c3 = 4*c1
  //        (BioGrowth/problem.f90:276-288)
  double c[4];
  float cf[4];  // the same coefficients rounded to FP32 on the host (mixed path)
  double h;
};

// One level of the periodic-box mixed path (box.cu): the level is a single
// fully periodic n0 x n1 x n2 box with even extents.  Its FP32 arrays are
// stored colour-split: for variable v and colour c (c = parity of the
// 1-based i+j(+k), so ipass 1 is c = 0) the cells of that colour follow row
// by row (row = (z, y)), hh = n0/2 of them per row; element
// (v*2 + c)*half + row*hh + x/2.  pb (the base phase field) has one variable.
struct BoxLev {
  int n[3];        // cells per dimension (n[2] = 1 in 2D)
  int hh;          // n[0] / 2
  int pad;
  long long half;  // cells of one colour
  long long oe, og, opb, oec;   // float offsets: e, g, pb, ec (ec: levels below the finest)
  long long oe2;                // a second e (the one-pass smoothing's output), -1: none
  float c0, c1, tmp3, a12;      // dt/h^2, eps^2/h^2, (4|6) eps^2/h^2, (4|6) dt/h^2
  float c0h, c0l, c1h, c1l;     // dt/h^2 and eps^2/h^2 as float pairs (hi + lo)
  double cd[4];                 // c0, c1, tmp3, a12 in FP64 (the coarsest level's FP64 smoother)
};

// One block of a level's work list: block covers units [start, start+kBlock)
// of patch `patch`.
struct Blk {
  int patch;
  int start;
};

// Ghost program operations (compiled by ghostc.cpp).
enum GhostType : int {
  kGCopy = 0,     // dst = src
  kGCopyAdd = 1,  // dst = src + qpo[v]
  kGCopySub = 2,  // dst = src - qpo[v]
  kGBC = 3,       // dst = (mask bit v) ? 2 - src : (mask bit 8+v) ? -src : src
  kGCfA = 4,      // a1*s0 + a2*s1 + a3*c0
  kGCfAB = 5,     // a1*s0 + a2*s1 + a3*(b1*c0 + b2*c1 + b3*c2)
  kGCfAC = 6,     // a1*s0 + a2*s1 + a3*(c1*c0 + c2*c1 + c3*c2 + c4*c3)
};

struct GhostOp {
  int type;
  int dp;     // destination patch index
  int dcell;  // destination cell offset within a q plane of dp
  int sp;     // source patch for copies, parent patch for CF ops
  int s0, s1; // source cells (copies: in sp; CF: fine cells in dp)
  int c0, c1, c2, c3;  // coarse cells in sp (CF ops)
  int mask;   // BC: bits 0-7 variables with value 1 on the face (2 - q), bits 8-15 value 0 (-q)
};

// The problem's parameters as the plugin's kernels see them (a kernel
// argument): dt and the reference plugins' problemdata (eps^2, gamma,
// lambda, c0), the growth plugin's pressure coefficient, and eight slots a
// new plugin may fill in its set_params; the quasi-periodic offsets qpo of
// SelfPeriodicBC; nrvars; the plugin's kind.
struct ProbParams {
  double dt, eps2, gamma, lambda, czero;
  double cpress;
  double user[8];
  double qpo[kMaxVars];
  int nrvars;
  int problem;
};

}  // namespace bsamg
