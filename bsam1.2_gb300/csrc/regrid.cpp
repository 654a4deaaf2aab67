// AMR regrid: the AMR(rootlevel) pass that TakeTimeSteps runs before every
// time step (LIBRARY/bsamroutines.f90:657-689, AMR :966-991).
//
// The clustering is inherently sequential and branchy host work on small
// integer arrays, so it runs on the host, as in the reference; the library
// downloads the solution once, builds the new mesh level by level, and
// uploads the new hierarchy once.  Level by level from the root:
//   SetGhost(l, 0)                       ghost programs executed on host arrays
//   tag (ErrFlag :1059-1131)             CH SetErrFlagsUser2D/3D or |grad phi|
//   buffer (BufferAndList :1206-1247, InflateEdgeTags :1267-1308)
//   cluster (NewSubGrids :1408-1605)     modified Berger-Rigoutsos per patch
//   MakeNewGrid (:1663-1784) + InitFields (:1787-1856)
//   TransferValues (:1859-1951)          previous level-(l+1) values
// Floating-point work (ghost interpolation, mass-corrected prolongation) is
// evaluated in the reference's order and built with -ffp-contract=off, so
// the new mesh and its values equal a sequential restatement bit for bit.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "hier.h"

namespace bsamg {

namespace {

constexpr int kMaxSubgrids = 1024;  // nodeinfodef.f90:62

struct Model {
  const Hier& src;                     // the hierarchy being regridded
  std::vector<HostPatch> g;            // geometry, in visiting order
  std::vector<std::vector<double>> q;  // ghosted q of levels >= 0 (empty below)
  std::vector<std::vector<double>> qold;
  std::vector<int> src_idx;            // index in src, or -1 for new patches
  explicit Model(const Hier& h) : src(h) {}
  int nd() const { return src.ndims; }
  size_t nq(const HostPatch& P) const { return (size_t)P.qn[0] * P.qn[1] * P.qn[2]; }
  // q(i,j,k,v) with Fortran indices i, j (and k in 3D; 0 in 2D)
  double& Q(int p, int i, int j, int k, int v) {
    const HostPatch& P = g[p];
    int s = src.mbc - 1, sk = src.ndims == 3 ? s : 0;
    return q[p][(((size_t)v * P.qn[2] + k + sk) * P.qn[1] + j + s) * P.qn[0] + i + s];
  }
};

// a host-only hierarchy with the model's geometry (tables, no device memory)
int host_tables(const Model& M, Hier& T) {
  T.ctx = M.src.ctx;
  T.ndims = M.src.ndims;
  T.nrvars = M.src.nrvars;
  T.mbc = M.src.mbc;
  T.problem = M.src.problem;
  T.pp = M.src.pp;
  for (const HostPatch& P : M.g) {
    HostPatch c = P;
    c.parent = -1;
    T.id2idx[c.id] = (int)T.patches.size();
    T.patches.push_back(c);
  }
  return build_tables(T);
}

// SetGhost(level, 0) on the model's host arrays: the level's writer
// sequence executed in order
int host_set_ghost(Model& M, int level) {
  Hier T;
  int r = host_tables(M, T);
  if (r) return r;
  std::vector<GhostOp> ops = set_ghost_sequence(T, level, 0);
  const double a1 = -01.0 / 05.0, a2 = 02.0 / 03.0, a3 = 08.0 / 15.0;   // boundary.f90:54-63
  const double b1 = 05.0 / 32.0, b2 = 15.0 / 16.0, b3 = -03.0 / 32.0;
  const double c1 = 09.0 / 16.0, c2 = 03.0 / 16.0, c3 = 03.0 / 16.0, c4 = 01.0 / 16.0;
  // cells are counted from cell (0,0,0) of each patch's q plane
  std::vector<double*> base(M.g.size(), nullptr);
  std::vector<size_t> plane(M.g.size());
  for (size_t p = 0; p < M.g.size(); p++) {
    plane[p] = M.nq(M.g[p]);
    if (!M.q[p].empty()) base[p] = M.q[p].data() + origin_of(M.src, M.g[p].qn);
  }
  for (const GhostOp& o : ops) {
    if (!base[o.dp] || !base[o.sp]) return BSAMG_ERR_ARG;  // below-root data is not on the host
    for (int v = 0; v < M.src.nrvars; v++) {
      double* dq = base[o.dp] + v * plane[o.dp];
      const double* sq = base[o.sp] + v * plane[o.sp];
      double val;
      switch (o.type) {
        case kGCopy: val = sq[o.s0]; break;
        case kGCopyAdd: val = sq[o.s0] + M.src.pp.qpo[v]; break;
        case kGCopySub: val = sq[o.s0] - M.src.pp.qpo[v]; break;
        case kGBC: val = ((o.mask >> v) & 1) ? 2.0 - sq[o.s0] : (((o.mask >> (8 + v)) & 1) ? -sq[o.s0] : sq[o.s0]); break;
        case kGCfA: val = a1 * dq[o.s0] + a2 * dq[o.s1] + a3 * sq[o.c0]; break;
        case kGCfAB: val = a1 * dq[o.s0] + a2 * dq[o.s1] + a3 * (b1 * sq[o.c0] + b2 * sq[o.c1] + b3 * sq[o.c2]); break;
        default:
          val = a1 * dq[o.s0] + a2 * dq[o.s1] + a3 * (c1 * sq[o.c0] + c2 * sq[o.c1] + c3 * sq[o.c2] + c4 * sq[o.c3]);
          break;
      }
      dq[o.dcell] = val;
    }
  }
  return BSAMG_OK;
}

// error flags of one patch, interior cells, x fastest
struct Flags {
  int mx[3];
  std::vector<int> f;
  int& at(int i, int j, int k) { return f[((size_t)(k - 1) * mx[1] + (j - 1)) * mx[0] + (i - 1)]; }
};

// SetErrFlagsUser2D/3D (CH/problem.f90:248-308): second differences of phi
// above (2|3) qtolerance; or the gradient rule |grad phi| h > qtolerance
void tag_patch(Model& M, int p, const bsamg_regrid_params& prm, Flags& F) {
  const HostPatch& P = M.g[p];
  int nd = M.nd();
  double tol = prm.qtolerance[P.level];
  for (int d = 0; d < 3; d++) F.mx[d] = P.mx[d];
  F.f.assign((size_t)P.mx[0] * P.mx[1] * P.mx[2], 0);
  // phi(i,j,k) from cell (0,0,0) of the ghosted plane (k unused in 2D)
  const double* q0 = M.q[p].data() + origin_of(M.src, P.qn);
  const long long sy = P.qn[0], sz = nd == 3 ? (long long)P.qn[0] * P.qn[1] : 0;
  auto q = [&](int i, int j, int k) { return q0[i + j * sy + k * sz]; };
  for (int k = 1; k <= P.mx[2]; k++)
    for (int j = 1; j <= P.mx[1]; j++)
      for (int i = 1; i <= P.mx[0]; i++) {
        bool t;
        if (prm.tagging == BSAMG_TAG_CH) {
          double s = std::fabs(q(i + 1, j, k) - 2.0 * q(i, j, k) + q(i - 1, j, k)) +
                     std::fabs(q(i, j + 1, k) - 2.0 * q(i, j, k) + q(i, j - 1, k));
          if (nd == 3) s = s + std::fabs(q(i, j, k + 1) - 2.0 * q(i, j, k) + q(i, j, k - 1));
          t = s > (nd == 3 ? 3.0 : 2.0) * tol;
        } else {
          double gx = (q(i + 1, j, k) - q(i - 1, j, k)) * 0.5;
          double gy = (q(i, j + 1, k) - q(i, j - 1, k)) * 0.5;
          double gs = gx * gx + gy * gy;
          if (nd == 3) {
            double gz = (q(i, j, k + 1) - q(i, j, k - 1)) * 0.5;
            gs = gs + gz * gz;
          }
          t = gs > tol * tol;
        }
        F.at(i, j, k) = t ? 1 : 0;
      }
}

struct Tag {
  int c[3];
};

// BufferAndList (:1206-1247): buffer inside the patch, list the tags whose
// buffer crosses its edge (global coordinates)
void buffer_and_list(const Model& M, const HostPatch& P, int ib, Flags& F, std::vector<Tag>& list) {
  std::vector<int> tmp = F.f;
  int nd = M.nd();
  for (int k = 1; k <= P.mx[2]; k++)
    for (int j = 1; j <= P.mx[1]; j++)
      for (int i = 1; i <= P.mx[0]; i++) {
        if (tmp[((size_t)(k - 1) * P.mx[1] + (j - 1)) * P.mx[0] + (i - 1)] != 1) continue;
        int idx[3] = {i, j, k}, lo[3] = {1, 1, 1}, hi[3] = {1, 1, 1};
        bool out = false;
        for (int d = 0; d < nd; d++) lo[d] = idx[d] - ib, hi[d] = idx[d] + ib;
        for (int d = 0; d < 3; d++) out = out || lo[d] < 1 || hi[d] > P.mx[d];
        if (out) {
          Tag t;
          for (int d = 0; d < 3; d++) t.c[d] = d < nd ? idx[d] + P.mglobal[d][0] - 1 : 1;
          list.push_back(t);
        } else {
          for (int c = lo[2]; c <= hi[2]; c++)
            for (int b = lo[1]; b <= hi[1]; b++)
              for (int a = lo[0]; a <= hi[0]; a++) F.at(a, b, c) = 1;
        }
      }
}

// BufferTaggedCells (:1311-1349)
void buffer_tagged(int nd, const HostPatch& P, const int* tag, int ib, Flags& F) {
  int lo[3] = {1, 1, 1}, hi[3] = {1, 1, 1};
  for (int d = 0; d < nd; d++) {
    lo[d] = std::max(tag[d] - ib, P.mglobal[d][0]);
    hi[d] = std::min(tag[d] + ib, P.mglobal[d][1]);
    if (hi[d] < lo[d]) return;
    lo[d] -= P.mglobal[d][0] - 1;
    hi[d] -= P.mglobal[d][0] - 1;
  }
  for (int c = lo[2]; c <= hi[2]; c++)
    for (int b = lo[1]; b <= hi[1]; b++)
      for (int a = lo[0]; a <= hi[0]; a++) F.at(a, b, c) = 1;
}

using Box = int[3][2];

// GetSignatures (:1608-1632) along dimension n over box b
void signature(Flags& F, const Box& b, int n, std::vector<int>& sig) {
  for (int i = b[n][0]; i <= b[n][1]; i++) {
    int lo[3], hi[3], s = 0;
    for (int d = 0; d < 3; d++) lo[d] = b[d][0], hi[d] = b[d][1];
    lo[n] = hi[n] = i;
    for (int c = lo[2]; c <= hi[2]; c++)
      for (int y = lo[1]; y <= hi[1]; y++)
        for (int x = lo[0]; x <= hi[0]; x++) s += F.at(x, y, c);
    sig[i] = s;
  }
}

// GridFlagRatio (:1635-1660)
double flag_ratio(Flags& F, Box& b, int nd) {
  double total = 1.0;
  for (int d = 0; d < nd; d++) total = total * (double)(b[d][1] - b[d][0] + 1);
  for (int d = nd; d < 3; d++) b[d][0] = b[d][1] = 1;
  long long s = 0;
  for (int c = b[2][0]; c <= b[2][1]; c++)
    for (int y = b[1][0]; y <= b[1][1]; y++)
      for (int x = b[0][0]; x <= b[0][1]; x++) s += F.at(x, y, c);
  return (double)s / total;
}

struct Sub {
  Box b;
};

// NewSubGrids (:1408-1605), the modified Berger-Rigoutsos algorithm; false
// on the reference's error stops
bool new_sub_grids(int nd, const HostPatch& P, Flags& F, const bsamg_regrid_params& prm, std::vector<Sub>& out) {
  out.clear();
  int level = P.level;
  double desfill = prm.desiredfillratio[level];
  int mgp = prm.minimumgridpoints[level];
  if (mgp < 4 || mgp % 2) return false;
  Sub whole;
  for (int d = 0; d < 3; d++) whole.b[d][0] = 1, whole.b[d][1] = d < nd ? P.mx[d] : 1;
  if (flag_ratio(F, whole.b, nd) < 1.0e-10) return true;
  int maxm = 0;
  for (int d = 0; d < nd; d++) maxm = std::max(maxm, P.mx[d]);
  std::vector<std::vector<int>> sig(3, std::vector<int>(maxm + 2, 0)), dds(3, std::vector<int>(maxm + 2, 0));
  std::vector<char> cansplit(kMaxSubgrids + 1, 1);
  out.push_back(whole);
  int igrid = 1;
  auto imod2 = [](int a) { return ((a % 2) + 2) % 2; };
  while ((int)out.size() < kMaxSubgrids && igrid <= (int)out.size()) {
    int npass = 0;
    while (cansplit[igrid] && npass < 15) {
      npass++;
      Box& b = out[igrid - 1].b;
      for (int n = 0; n < nd; n++) signature(F, b, n, sig[n]);
      for (int n = 0; n < nd; n++) {  // trim unflagged edges
        int i1 = b[n][0], i2 = b[n][1];
        while (sig[n][i1] == 0 && i1 < b[n][1] && i2 - i1 + 1 > mgp) i1++;
        while (sig[n][i2] == 0 && i2 > b[n][0] && i2 - i1 + 1 > mgp) i2--;
        b[n][0] = i1 - imod2(i1 + 1);
        b[n][1] = i2 + imod2(i2);
      }
      if (flag_ratio(F, b, nd) >= desfill) {
        cansplit[igrid] = 0;
        continue;
      }
      for (int n = 0; n < nd; n++) signature(F, b, n, sig[n]);
      int isplit[3] = {0, 0, 0};
      bool have = false;
      for (int n = 0; n < nd && !have; n++) {  // holes
        int i1 = b[n][0], i2 = b[n][1];
        for (int i = i1 + mgp - 1; i <= i2 - mgp; i += 2)
          if (sig[n][i] == 0 && std::min(i - i1 + 1, i2 - i) >= mgp) {
            isplit[n] = i;
            have = true;
            break;
          }
      }
      if (!have) {  // inflection points
        for (int n = 0; n < nd; n++)
          for (int i = b[n][0] + 1; i <= b[n][1] - 1; i++) dds[n][i] = sig[n][i - 1] - 2 * sig[n][i] + sig[n][i + 1];
        int inflect = 0, dist0 = 0;
        for (int n = 0; n < nd; n++) {
          int i1 = b[n][0], i2 = b[n][1];
          for (int i = i1 + mgp; i <= i2 - mgp + 1; i += 2) {
            int del = std::abs(dds[n][i] - dds[n][i - 1]);
            if (del > inflect) {
              inflect = del;
              isplit[0] = isplit[1] = isplit[2] = 0;
              isplit[n] = i - 1;
              have = true;
              dist0 = std::min(i - i1, i2 - i + 1);
            } else if (del == inflect && inflect > 0) {
              int dist1 = std::min(i - i1, i2 - i + 1);
              if (dist1 > dist0) {
                isplit[0] = isplit[1] = isplit[2] = 0;
                isplit[n] = i - 1;
                have = true;
                dist0 = dist1;
              }
            }
          }
        }
      }
      if (!have) {
        cansplit[igrid] = 0;
        continue;
      }
      for (int n = 0; n < nd; n++)
        if (isplit[n] > 0 && std::min(b[n][1] - isplit[n], isplit[n] - b[n][0] + 1) >= mgp) {
          Sub s = out[igrid - 1];
          s.b[n][0] = isplit[n] + 1;
          out[igrid - 1].b[n][1] = isplit[n];
          out.push_back(s);
          cansplit[out.size()] = 1;
          break;
        }
    }
    igrid++;
  }
  for (const Sub& s : out)  // the reference's checks, :1565-1595
    for (int n = 0; n < nd; n++) {
      int len = s.b[n][1] - s.b[n][0] + 1;
      if (len < mgp || len % 2 || s.b[n][0] % 2 == 0 || s.b[n][1] % 2 == 1) return false;
    }
  return true;
}

// Patches longer than maxside child cells are cut into nearly equal even
// pieces (not a reference feature: it bounds patch sizes for the batched
// kernels)
void split_long(int nd, int maxside, std::vector<Sub>& subs) {
  if (maxside <= 0) return;
  int P = maxside / 2;
  for (size_t g = 0; g < subs.size(); g++)
    for (int n = 0; n < nd; n++) {
      int len = subs[g].b[n][1] - subs[g].b[n][0] + 1;
      if (len <= P) continue;
      int pieces = (len + P - 1) / P, half = len / 2, base = half / pieces, extra = half % pieces;
      int lo = subs[g].b[n][0];
      Sub tmpl = subs[g];
      for (int k = 0; k < pieces; k++) {
        int plen = 2 * (base + (k < extra ? 1 : 0));
        Sub piece = tmpl;
        piece.b[n][0] = lo;
        piece.b[n][1] = lo + plen - 1;
        if (k == 0) subs[g] = piece;
        else subs.push_back(piece);
        lo += plen;
      }
    }
}

// BiLin/TriLinProlongationP1MC and P2MC (gridutilities.f90:242-369,
// :628-829): a is the coarse block with mbc ghost layers (cmx+2 mbc per
// dimension, index 1-mbc first), out the fine block with mbc ghost layers.
// Fine cell 2c takes 3 a(c) + a(c+1) and fine cell 2c+1 takes a(c) +
// 3 a(c+1) in each direction (x, then y, then z; the last divided by 16 or
// 64; P2 writes the odd cells' sum as 3 a(c+1) + a(c), the same IEEE sum),
// then each interior coarse cell's mass correction goes to its 2^d cells.
void prolong_mc(int nd, int mbc, const double* a, const int cmx[3], double* out) {
  const int L = 1 - mbc, kL = nd == 3 ? L : 0, g = mbc - 1;
  const int cn0 = cmx[0] + 2 * mbc, cn1 = cmx[1] + 2 * mbc, cn2 = nd == 3 ? cmx[2] + 2 * mbc : 1;
  const int fn0 = 2 * cmx[0] + 2 * mbc, fn1 = 2 * cmx[1] + 2 * mbc, fn2 = nd == 3 ? 2 * cmx[2] + 2 * mbc : 1;
  auto A = [&](int i, int j, int k) { return a[((size_t)(k - kL) * cn1 + (j - L)) * cn0 + (i - L)]; };
  auto O = [&](int i, int j, int k) -> double& { return out[((size_t)(k - kL) * fn1 + (j - L)) * fn0 + (i - L)]; };
  std::vector<double> b((size_t)fn0 * cn1 * cn2);
  auto Bx = [&](int i, int j, int k) -> double& { return b[((size_t)(k - kL) * cn1 + (j - L)) * fn0 + (i - L)]; };
  // fine cells 2I and 2I+1 of coarse pair (I, I+1), I = -g..cmx+g, kept
  // where they lie in L..2 cmx + mbc
  const int hi0 = 2 * cmx[0] + mbc, hi1 = 2 * cmx[1] + mbc, hi2 = nd == 3 ? 2 * cmx[2] + mbc : 0;
  for (int k = kL; k < kL + cn2; k++)
    for (int j = L; j < L + cn1; j++)
      for (int I = -g; I <= cmx[0] + g; I++) {
        double lo = A(I, j, k), up = A(I + 1, j, k);
        if (2 * I >= L) Bx(2 * I, j, k) = 3.0 * lo + up;
        if (2 * I + 1 <= hi0) Bx(2 * I + 1, j, k) = lo + 3.0 * up;
      }
  if (nd == 2) {
    for (int J = -g; J <= cmx[1] + g; J++)
      for (int i = L; i < L + fn0; i++) {
        double lo = Bx(i, J, 0), up = Bx(i, J + 1, 0);
        if (2 * J >= L) O(i, 2 * J, 0) = (3.0 * lo + up) / 16.0;
        if (2 * J + 1 <= hi1) O(i, 2 * J + 1, 0) = (lo + 3.0 * up) / 16.0;
      }
    for (int J = 1; J <= cmx[1]; J++)
      for (int I = 1; I <= cmx[0]; I++) {
        double cor = A(I, J, 0) - 0.25 * (O(2 * I, 2 * J, 0) + O(2 * I - 1, 2 * J, 0) + O(2 * I, 2 * J - 1, 0) +
                                          O(2 * I - 1, 2 * J - 1, 0));
        O(2 * I, 2 * J, 0) = O(2 * I, 2 * J, 0) + cor;
        O(2 * I - 1, 2 * J, 0) = O(2 * I - 1, 2 * J, 0) + cor;
        O(2 * I, 2 * J - 1, 0) = O(2 * I, 2 * J - 1, 0) + cor;
        O(2 * I - 1, 2 * J - 1, 0) = O(2 * I - 1, 2 * J - 1, 0) + cor;
      }
    return;
  }
  std::vector<double> c((size_t)fn0 * fn1 * cn2);
  auto Cy = [&](int i, int j, int k) -> double& { return c[((size_t)(k - kL) * fn1 + (j - L)) * fn0 + (i - L)]; };
  for (int k = kL; k < kL + cn2; k++)
    for (int J = -g; J <= cmx[1] + g; J++)
      for (int i = L; i < L + fn0; i++) {
        double lo = Bx(i, J, k), up = Bx(i, J + 1, k);
        if (2 * J >= L) Cy(i, 2 * J, k) = 3.0 * lo + up;
        if (2 * J + 1 <= hi1) Cy(i, 2 * J + 1, k) = lo + 3.0 * up;
      }
  for (int K = -g; K <= cmx[2] + g; K++)
    for (int j = L; j < L + fn1; j++)
      for (int i = L; i < L + fn0; i++) {
        double lo = Cy(i, j, K), up = Cy(i, j, K + 1);
        if (2 * K >= L) O(i, j, 2 * K) = (3.0 * lo + up) / 64.0;
        if (2 * K + 1 <= hi2) O(i, j, 2 * K + 1) = (lo + 3.0 * up) / 64.0;
      }
  (void)fn2;
  for (int K = 1; K <= cmx[2]; K++)
    for (int J = 1; J <= cmx[1]; J++)
      for (int I = 1; I <= cmx[0]; I++) {
        double cor = A(I, J, K) - 0.125 * (O(2 * I, 2 * J, 2 * K) + O(2 * I - 1, 2 * J, 2 * K) +
                                           O(2 * I, 2 * J - 1, 2 * K) + O(2 * I - 1, 2 * J - 1, 2 * K) +
                                           O(2 * I, 2 * J, 2 * K - 1) + O(2 * I - 1, 2 * J, 2 * K - 1) +
                                           O(2 * I, 2 * J - 1, 2 * K - 1) + O(2 * I - 1, 2 * J - 1, 2 * K - 1));
        for (int dk = 0; dk < 2; dk++)
          for (int dj = 0; dj < 2; dj++)
            for (int di = 0; di < 2; di++)
              O(2 * I - di, 2 * J - dj, 2 * K - dk) = O(2 * I - di, 2 * J - dj, 2 * K - dk) + cor;
      }
}

// InitFields' prolongation for child c of patch p over box b (:1815-1818,
// :1834-1837): child%qc(1-mbc:cmx+mbc) = parent%q(mb-mbc:mb+mbc), then
// child%q(1-mbc:mx+mbc) = P1MC / P2MC(child%qc); child%qold = child%q (:1782)
void init_from_parent(Model& M, int c, int p, const Box& b) {
  const HostPatch& C = M.g[c];
  int nd = M.nd();
  const int mbc = M.src.mbc;
  size_t nq = (size_t)C.qn[0] * C.qn[1] * C.qn[2], nc = (size_t)C.cn[0] * C.cn[1] * C.cn[2];
  std::vector<double> qc(nc * M.src.nrvars, 0.0);
  std::vector<double>& q = M.q[c];
  int cmx[3] = {C.cmx[0], C.cmx[1], nd == 3 ? C.cmx[2] : 0};
  int k0 = nd == 3 ? b[2][0] - mbc : 0, k1 = nd == 3 ? b[2][1] + mbc : 0;
  for (int v = 0; v < M.src.nrvars; v++) {
    size_t t = v * nc;
    for (int k = k0; k <= k1; k++)
      for (int j = b[1][0] - mbc; j <= b[1][1] + mbc; j++)
        for (int i = b[0][0] - mbc; i <= b[0][1] + mbc; i++) qc[t++] = M.Q(p, i, j, k, v);
    prolong_mc(nd, mbc, qc.data() + v * nc, cmx, q.data() + v * nq);
  }
  M.qold[c] = q;
}

// MakeNewGrid (:1663-1784) and InitFields (:1787-1856) for box b of patch p;
// without QInit the values come later from init_from_parent (the caller
// runs it for every new child of the level, in parallel)
void make_new_grid(Model& M, int p, const Box& b, int id, const bsamg_regrid_params& prm, bsamg_qinit_fn qinit,
                   void* user) {
  int nd = M.nd();
  HostPatch C{};
  const HostPatch& P = M.g[p];
  C.level = P.level + 1;
  C.id = id;
  C.parent_id = P.id;
  C.parent = p;
  for (int d = 0; d < 3; d++) {
    C.mx[d] = 1;
    C.mglobal[d][0] = C.mglobal[d][1] = C.mbounds[d][0] = C.mbounds[d][1] = 1;
    C.dx[d] = C.xlower[d] = 0.0;
    if (d >= nd) continue;
    C.mx[d] = (b[d][1] - b[d][0] + 1) * 2;
    C.mbounds[d][0] = b[d][0];
    C.mbounds[d][1] = b[d][1];
    int g0 = P.mglobal[d][0] + b[d][0] - 1, g1 = g0 + b[d][1] - b[d][0];
    C.mglobal[d][0] = (g0 - 1) * 2 + 1;
    C.mglobal[d][1] = g1 * 2;
    C.xlower[d] = (double)(b[d][0] - 1) * P.dx[d] + P.xlower[d];
    C.dx[d] = P.dx[d] / 2.0;
  }
  for (int f = 0; f < 6; f++) C.mthbc[f] = f < 2 * nd ? kInternalBC : 10;
  for (int n = 0; n < nd; n++) {
    if (P.mthbc[2 * n] < kInternalBC && C.mbounds[n][0] == 1) C.mthbc[2 * n] = P.mthbc[2 * n];
    if (P.mthbc[2 * n + 1] < kInternalBC && C.mbounds[n][1] == P.mx[n]) C.mthbc[2 * n + 1] = P.mthbc[2 * n + 1];
  }
  const int mbc = M.src.mbc;
  for (int d = 0; d < 3; d++) {
    C.cmx[d] = d < nd ? C.mx[d] / 2 : 1;
    C.qn[d] = d < nd ? C.mx[d] + 2 * mbc : 1;
    C.cn[d] = d < nd ? C.cmx[d] + 2 * mbc : 1;
  }
  size_t nq = (size_t)C.qn[0] * C.qn[1] * C.qn[2];
  std::vector<double> q(nq * M.src.nrvars, 0.0);  // AllocFields' zero fill
  if (prm.initial) qinit(user, C.level, C.mx, C.dx, C.xlower, q.data());
  M.g.push_back(C);
  M.src_idx.push_back(-1);
  M.qold.push_back(prm.initial ? q : std::vector<double>());  // child%qold = child%q (:1782)
  M.q.push_back(std::move(q));
}

// TransferOverlap (:1919-1951): interior q of src onto dst
void transfer_overlap(int nrvars, const HostPatch& S, const std::vector<double>& sq, const HostPatch& D,
                      std::vector<double>& dq, int nd) {
  int lo[3], hi[3];
  for (int d = 0; d < 3; d++) {
    lo[d] = std::max(S.mglobal[d][0], D.mglobal[d][0]);
    hi[d] = std::min(S.mglobal[d][1], D.mglobal[d][1]);
    if (hi[d] < lo[d]) return;
  }
  size_t ns = (size_t)S.qn[0] * S.qn[1] * S.qn[2], ndd = (size_t)D.qn[0] * D.qn[1] * D.qn[2];
  // local Fortran index = global - mglobal + 1; the arrays start at 1 - mbc
  int g = (int)((D.qn[0] - D.mx[0]) / 2), ko = nd == 3 ? g : 0;
  auto at = [&](const HostPatch& P, int i, int j, int k) {
    return ((size_t)(k - P.mglobal[2][0] + ko) * P.qn[1] + (j - P.mglobal[1][0] + g)) * P.qn[0] +
           (i - P.mglobal[0][0] + g);
  };
  for (int v = 0; v < nrvars; v++)
    for (int k = lo[2]; k <= hi[2]; k++)
      for (int j = lo[1]; j <= hi[1]; j++)
        for (int i = lo[0]; i <= hi[0]; i++) dq[v * ndd + at(D, i, j, k)] = sq[v * ns + at(S, i, j, k)];
}


}  // namespace

int regrid(Hier& H, const bsamg_regrid_params& prm, bsamg_qinit_fn qinit, void* user, bsamg_hier** out) {
  if (!H.committed || prm.maxlevel < 0 || prm.maxlevel > kMaxDepth || (prm.initial && !qinit)) return BSAMG_ERR_ARG;
  if (prm.tagging != BSAMG_TAG_CH && prm.tagging != BSAMG_TAG_GRADIENT) return BSAMG_ERR_ARG;
  int r = set_device(H);
  if (r) return r;
  int nd = H.ndims, nv = H.nrvars;
  Model M(H);
  using clk = std::chrono::steady_clock;
  auto ms = [](clk::time_point a, clk::time_point b) { return std::chrono::duration<double, std::milli>(b - a).count(); };
  const clk::time_point t0 = clk::now();
  // one copy of the whole q region (every patch, ghosts included)
  std::vector<double> qreg((size_t)H.q_len);
  cudaError_t ce = cudaMemcpyAsync(qreg.data(), H.pool + H.q_region, qreg.size() * sizeof(double),
                                   cudaMemcpyDeviceToHost, H.s);
  if (ce != cudaSuccess) return cuda_fail(ce, "cudaMemcpyAsync(regrid download)");
  ce = cudaStreamSynchronize(H.s);
  if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamSynchronize(regrid)");
  const clk::time_point t1 = clk::now();
  auto slice = [&](int n) {
    const HostPatch& P = H.patches[n];
    const double* b = qreg.data() + (P.oq - H.q_region);
    return std::vector<double>(b, b + (size_t)P.sq * nv);
  };
  // the root and the levels below persist; q of level 0 is regridded on the host
  for (size_t n = 0; n < H.patches.size(); n++) {
    const HostPatch& P = H.patches[n];
    if (P.level > 0) continue;
    M.g.push_back(P);
    M.src_idx.push_back((int)n);
    M.q.push_back(P.level == 0 ? slice((int)n) : std::vector<double>());
    M.qold.emplace_back();
  }
  // previous refinement levels, for TransferValues
  std::vector<std::vector<double>> oldq(H.patches.size());
  for (size_t n = 0; n < H.patches.size(); n++)
    if (H.patches[n].level > 0) oldq[n] = slice((int)n);

  int next_id = prm.first_id;
  int level;
  double part[6] = {};  // host ms of the model's parts, summed over levels
  clk::time_point tp = clk::now();
  auto lap = [&](int x) {
    const clk::time_point t = clk::now();
    part[x] += ms(tp, t);
    tp = t;
  };
  // a level's patches in visiting order (youngest first: the reverse of
  // creation order, as ApplyOnLevel walks them), so that RefineGrid runs
  // over the parents, and creates their children, in the reference's order
  auto level_patches = [&](int l) {
    std::vector<int> v;
    for (size_t p = M.g.size(); p-- > 0;)
      if (M.g[p].level == l) v.push_back((int)p);
    return v;
  };
  for (level = 0; level < prm.maxlevel; level++) {  // AMR(level), :966-991
    std::vector<int> lp = level_patches(level);
    if (lp.empty()) break;
    tp = clk::now();
    if ((r = host_set_ghost(M, level))) return r;
    lap(0);
    std::vector<Flags> fl(lp.size());
    std::vector<Tag> list;
    int ib = prm.ibuffer[level];
    {  // ErrFlag, per patch on the thread pool; the edge lists joined in patch order
      std::vector<std::vector<Tag>> lists(lp.size());
      parallel_for((int)lp.size(), [&](int a) {
        tag_patch(M, lp[a], prm, fl[a]);
        if (ib > 0) buffer_and_list(M, M.g[lp[a]], ib, fl[a], lists[a]);
      });
      for (auto& v : lists) list.insert(list.end(), v.begin(), v.end());
    }
    lap(1);
    if (!list.empty()) {  // InflateEdgeTags
      Hier T;
      if ((r = host_tables(M, T))) return r;
      int poff[13][3] = {};
      for (int o = 0; o < T.nperoff; o++) {
        const int* mm = T.mxmax[level];
        int a = 0, b = 0, c = 0;
        switch (T.peroffidx[o]) {  // GetPeriodicOffsets, boundary.f90:875-954
          case 1: a = mm[0]; break;
          case 2: b = mm[1]; break;
          case 3: c = mm[2]; break;
          case 4: a = mm[0]; b = mm[1]; break;
          case 5: a = -mm[0]; b = mm[1]; break;
          case 6: b = mm[1]; c = mm[2]; break;
          case 7: b = mm[1]; c = -mm[2]; break;
          case 8: a = mm[0]; c = mm[2]; break;
          case 9: a = -mm[0]; c = mm[2]; break;
          case 10: a = mm[0]; b = mm[1]; c = mm[2]; break;
          case 11: a = mm[0]; b = mm[1]; c = -mm[2]; break;
          case 12: a = -mm[0]; b = mm[1]; c = mm[2]; break;
          case 13: a = mm[0]; b = -mm[1]; c = mm[2]; break;
        }
        poff[o][0] = a, poff[o][1] = b, poff[o][2] = c;
      }
      // every patch's flags see the tags in the reference's order; the
      // patches are independent, so each is done on the thread pool
      parallel_for((int)lp.size(), [&](int a) {
        for (int t = (int)list.size() - 1; t >= 0; t--) {
          buffer_tagged(nd, M.g[lp[a]], list[t].c, ib, fl[a]);
          if (T.periodic)
            for (int pol = -1; pol <= 1; pol += 2)
              for (int o = 0; o < T.nperoff; o++) {
                int c[3];
                for (int d = 0; d < 3; d++) c[d] = list[t].c[d] + pol * poff[o][d];
                buffer_tagged(nd, M.g[lp[a]], c, ib, fl[a]);
              }
        }
      });
    }
    lap(2);
    size_t first_new = M.g.size();
    {  // GridAdapt -> RefineGrid: each parent's clustering on the thread pool,
       // the children made in the parents' order (their ids and visiting
       // order), then their values, in parallel again
      std::vector<std::vector<Sub>> subs_of(lp.size());
      std::vector<char> ok(lp.size(), 1);
      parallel_for((int)lp.size(), [&](int a) {
        ok[a] = new_sub_grids(nd, M.g[lp[a]], fl[a], prm, subs_of[a]) ? 1 : 0;
        if (ok[a]) split_long(nd, prm.maxside, subs_of[a]);
      });
      lap(3);
      std::vector<std::pair<int, const Sub*>> made;  // (parent, box) of each new child
      for (size_t a = 0; a < lp.size(); a++) {
        if (!ok[a]) return BSAMG_ERR_ARG;
        for (const Sub& sb : subs_of[a]) {
          make_new_grid(M, lp[a], sb.b, next_id++, prm, qinit, user);
          made.emplace_back(lp[a], &sb);
        }
      }
      if (!prm.initial)
        parallel_for((int)made.size(), [&](int x) {
          init_from_parent(M, (int)(first_new + x), made[x].first, made[x].second->b);
        });
    }
    lap(4);
    std::vector<int> olds;  // TransferValues from the previous level-(l+1) patches
    for (size_t n = 0; n < H.patches.size(); n++)
      if (H.patches[n].level == level + 1) olds.push_back((int)n);
    parallel_for((int)(M.g.size() - first_new), [&](int x) {
      size_t c = first_new + x;
      for (int n : olds) transfer_overlap(nv, H.patches[n], oldq[n], M.g[c], M.q[c], nd);
    });
    lap(5);
  }
  // AMR(finest) ends with SetGhost(finest, 0); nothing on the host reads its
  // result, so it runs on the device after the upload (the compiled program
  // gives the sequential sequence's values)
  int final_ghost = level_patches(level).empty() ? -kMaxDepth - 1 : level;

  const clk::time_point t2 = clk::now();
  // the new hierarchy, on the same context
  bsamg_hier* nh = nullptr;
  r = bsamg_hier_create(H.ctx, nd, nv, H.mbc, H.problem, H.params.data(), (int)H.params.size(), H.pp.qpo, &nh);
  if (r) return r;
  nh->has_root_xupper = H.has_root_xupper;
  std::memcpy(nh->root_xupper, H.root_xupper, sizeof(H.root_xupper));
  nh->tail_cells = H.tail_cells;  // tuning carries over
  nh->box_sweep = H.box_sweep;
  nh->solve_mode = H.solve_mode;
  nh->solve_shape = H.solve_shape;
  nh->solve_solo_cells = H.solve_solo_cells;
  nh->solve_tuned = H.solve_tuned;
  auto fail = [&](int rc) {
    bsamg_hier_destroy(nh);
    return rc;
  };
  for (const HostPatch& P : M.g) {
    int mg[6], mb[6];
    for (int d = 0; d < 3; d++) {
      mg[2 * d] = P.mglobal[d][0], mg[2 * d + 1] = P.mglobal[d][1];
      mb[2 * d] = P.mbounds[d][0], mb[2 * d + 1] = P.mbounds[d][1];
    }
    if ((r = bsamg_patch_add(nh, P.level, P.id, P.parent_id, P.mx, mg, mb, P.mthbc, P.dx, P.xlower))) return fail(r);
  }
  if ((r = bsamg_commit(nh))) return fail(r);
  const clk::time_point t3 = clk::now();
  Hier& N = *nh;
  // q: one image of the new q region; qold: one image (new patches) and a
  // device-to-device copy for the persisting levels <= 0
  std::vector<double> qimg((size_t)N.q_len, 0.0), oimg((size_t)N.q_len, 0.0);
  for (size_t p = 0; p < M.g.size(); p++) {
    const HostPatch& D = N.patches[p];
    double* dq = qimg.data() + (D.oq - N.q_region);
    size_t n = (size_t)D.sq * nv;
    if (M.src_idx[p] >= 0 && M.g[p].level < 0) {
      const HostPatch& S = H.patches[M.src_idx[p]];
      std::memcpy(dq, qreg.data() + (S.oq - H.q_region), n * sizeof(double));
    } else {
      std::memcpy(dq, M.q[p].data(), n * sizeof(double));
    }
    if (M.src_idx[p] < 0) std::memcpy(oimg.data() + (D.oq - N.q_region), M.qold[p].data(), n * sizeof(double));
  }
  ce = cudaMemcpyAsync(N.pool + N.q_region, qimg.data(), qimg.size() * sizeof(double), cudaMemcpyHostToDevice, N.s);
  if (ce == cudaSuccess)
    ce = cudaMemcpyAsync(N.pool + N.qold_region, oimg.data(), oimg.size() * sizeof(double), cudaMemcpyHostToDevice,
                         N.s);

  for (size_t p = 0; p < M.g.size() && ce == cudaSuccess; p++)
    if (M.src_idx[p] >= 0) {
      const HostPatch& D = N.patches[p];
      const HostPatch& S = H.patches[M.src_idx[p]];
      ce = cudaMemcpyAsync(N.pool + D.oqold, H.pool + S.oqold, (size_t)D.sq * nv * sizeof(double),
                           cudaMemcpyDeviceToDevice, N.s);
      // the persisting patches keep their qc (with mbc = 2 its second ring
      // carries the last correction)
      if (ce == cudaSuccess)
        ce = cudaMemcpyAsync(N.pool + D.oqc, H.pool + S.oqc, (size_t)D.sc * nv * sizeof(double),
                             cudaMemcpyDeviceToDevice, N.s);
    }
  if (ce != cudaSuccess) return fail(cuda_fail(ce, "cudaMemcpyAsync(regrid upload)"));
  // InitFields' child qc = parent q on the new patches (their parents' q is
  // final in the uploaded image); QInit'd patches keep the zero fill
  if (!prm.initial)
    for (int l = 1; l <= N.maxlevel; l++) {
      LevelT& L = N.L(l);
      if ((r = after_launch(N, launch_qc_from_parent(N.lc(), L.d_blk[kKindCGhost], L.nblk[kKindCGhost]))))
        return fail(r);
    }
  if (final_ghost >= 0 && (r = enq_set_ghost(N, final_ghost, 0))) return fail(r);
  ce = cudaStreamSynchronize(N.s);  // the host arrays are freed on return
  if (ce != cudaSuccess) return fail(cuda_fail(ce, "cudaStreamSynchronize(regrid upload)"));
  // the old hierarchy's executable graphs go to the new one, which updates
  // them in place on its first capture; the old one captures again if used
  N.graph_donors = std::move(H.graphs);
  H.graphs.clear();
  const clk::time_point t4 = clk::now();
  N.regrid_ms[0] = ms(t0, t1);
  N.regrid_ms[1] = ms(t1, t2);
  N.regrid_ms[2] = ms(t2, t3);
  N.regrid_ms[3] = ms(t3, t4);
  for (int x = 0; x < 6; x++) N.regrid_ms[6 + x] = part[x];
  *out = nh;
  return BSAMG_OK;
}

}  // namespace bsamg
