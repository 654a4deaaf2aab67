// Frame files, restart and after-step statistics (host side).
//
// WriteQ / ReadQ / WriteUniformMeshQ (LIBRARY/bsaminputoutput.f90:60-572)
// keep the reference's MATLAB-readable text format: every real is an F25.12
// field, the header records are I3 / I8 fields as the reference's FORMAT
// statements give them, and the data of a patch are one record per ghosted
// cell (column-major, ghost layers included) holding its nrvars values.
// The statistics of AfterStepStatistics (LIBRARY/bsamroutines.f90:918-963)
// are reduced on the device (io.cu); only two doubles come back.
//
// The text is produced in parallel: a patch's field arrays come down in one
// copy of the whole q region, every record has the same length, and the
// records of a window are formatted by all host threads into disjoint parts
// of one buffer before it is written.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "hier.h"

namespace bsamg {

int io_fail(const char* what);

namespace {

constexpr int kField = 25;                    // F25.12
constexpr size_t kWindowRecords = 1 << 20;  // records formatted per write

int host_threads() {
  unsigned n = std::thread::hardware_concurrency();
  return (int)std::max(1u, std::min(n, 32u));
}

// run fn(t, nt) on nt threads
template <class F>
void parallel(int nt, F fn) {
  if (nt <= 1) {
    fn(0, 1);
    return;
  }
  std::vector<std::thread> th;
  for (int t = 1; t < nt; t++) th.emplace_back(fn, t, nt);
  fn(0, nt);
  for (auto& x : th) x.join();
}

void right_justify(const char* s, char* out) {
  size_t n = std::strlen(s);
  std::memset(out, ' ', kField - n);
  std::memcpy(out + kField - n, s, n);
}

// One F25.12 field into out[0..24].  |x| * 10^12 is rounded to the nearest
// integer (ties to even) exactly: x = M * 2^e with a 53-bit M, so
// x * 10^12 = M * 5^12 * 2^(e+12) and M * 5^12 < 2^81 fits in 128 bits; the
// rounding is then a shift with an exact remainder.  This is the value the
// C library's "%25.12f" prints.  A number that needs more than 25
// characters gives 25 asterisks, as Fortran output does.
void f25(double x, char* out) {
  if (std::isnan(x)) return right_justify("NaN", out);
  if (std::isinf(x)) return right_justify(x < 0 ? "-Infinity" : "Infinity", out);
  bool neg = std::signbit(x);
  double a = std::fabs(x);
  unsigned __int128 N = 0;
  if (a != 0.0) {
    int e;
    double m = std::frexp(a, &e);
    if (e > 60) {  // at least 19 integer digits
      std::memset(out, '*', kField);
      return;
    }
    uint64_t M = (uint64_t)std::ldexp(m, 53);
    unsigned __int128 P = (unsigned __int128)M * 244140625u;  // 5^12
    int s = e - 53 + 12;
    if (s >= 0) {
      N = P << s;
    } else if (-s <= 81) {
      int r = -s;
      N = P >> r;
      unsigned __int128 rem = P & ((((unsigned __int128)1) << r) - 1);
      unsigned __int128 half = ((unsigned __int128)1) << (r - 1);
      if (rem > half || (rem == half && (N & 1))) N++;
    }  // else P < 2^81 <= half: rounds to 0
  }
  const uint64_t kTen12 = 1000000000000ull;
  uint64_t ip = (uint64_t)(N / kTen12), fp = (uint64_t)(N % kTen12);
  char buf[48];
  int p = 47;
  buf[p] = 0;
  for (int d = 0; d < 12; d++) {
    buf[--p] = (char)('0' + fp % 10);
    fp /= 10;
  }
  buf[--p] = '.';
  do {
    buf[--p] = (char)('0' + ip % 10);
    ip /= 10;
  } while (ip);
  if (neg) buf[--p] = '-';
  int len = 47 - p;
  if (len > kField) {
    std::memset(out, '*', kField);
    return;
  }
  std::memset(out, ' ', kField - len);
  std::memcpy(out + kField - len, buf + p, len);
}

std::string f25s(double x) {
  char b[kField];
  f25(x, b);
  return std::string(b, kField);
}

// Iw output ("%wd", asterisks when it does not fit)
std::string iw(long long v, int w) {
  char b[32];
  int n = std::snprintf(b, sizeof b, "%*lld", w, v);
  if (n > w) return std::string(w, '*');
  return std::string(b, n);
}

// the header records of one patch block (OutputQ, bsaminputoutput.f90:85-124)
std::string block_header(int nd, int nv, int level, const double* dx, const double* xl, const double* xu,
                         const int* mx, const int (*mg)[2]) {
  std::string s = "  \n";  // WRITE(54,*) ' ': list-directed, a leading blank then ' '
  s += iw(level, 3) + " " + iw(nd, 3) + " " + iw(2, 3) + " " + iw(nv, 3) + "\n";
  const double* rows[3] = {dx, xl, xu};
  for (auto r : rows) {
    for (int d = 0; d < nd; d++) s += (d ? " " : "") + f25s(r[d]);
    s += "\n";
  }
  for (int d = 0; d < nd; d++) s += (d ? " " : "") + iw(mx[d], 8);
  s += "\n";
  for (int d = 0; d < nd; d++) s += (d ? " " : "") + iw(mg[d][0], 8) + " " + iw(mg[d][1], 8);
  s += "\n";
  return s;
}

// WriteQ2D/3D (:132-181): one record per ghosted cell, nv F25.12 fields
// separated by 2X (the 2X after the last field writes nothing)
bool write_records(FILE* f, const double* q, size_t plane, int nv) {
  size_t rec = (size_t)nv * kField + 2 * (size_t)(nv - 1) + 1;
  std::vector<char> buf;
  int nt = host_threads();
  for (size_t c0 = 0; c0 < plane; c0 += kWindowRecords) {
    size_t nrec = std::min(kWindowRecords, plane - c0);
    buf.resize(nrec * rec);
    parallel(nt, [&](int t, int n) {
      size_t a = nrec * t / n, b = nrec * (t + 1) / n;
      for (size_t r = a; r < b; r++) {
        char* o = buf.data() + r * rec;
        for (int v = 0; v < nv; v++) {
          if (v) {
            o[0] = o[1] = ' ';
            o += 2;
          }
          f25(q[(size_t)v * plane + c0 + r], o);
          o += kField;
        }
        *o = '\n';
      }
    });
    if (std::fwrite(buf.data(), 1, buf.size(), f) != buf.size()) return false;
  }
  return true;
}

bool write_block(FILE* f, int nd, int nv, int level, const double* dx, const double* xl, const double* xu,
                 const int* mx, const int (*mg)[2], const double* q) {
  std::string h = block_header(nd, nv, level, dx, xl, xu, mx, mg);
  if (std::fwrite(h.data(), 1, h.size(), f) != h.size()) return false;
  size_t plane = (size_t)(mx[0] + 2) * (mx[1] + 2) * (nd == 3 ? mx[2] + 2 : 1);
  return write_records(f, q, plane, nv);
}

bool write_head(FILE* f, double time, int finest) {
  std::string s = f25s(time) + "\n" + iw(finest, 3) + "\n";
  return std::fwrite(s.data(), 1, s.size(), f) == s.size();
}

int download_q(Hier& H, std::vector<double>& q) {
  q.resize((size_t)H.q_len);
  cudaError_t e = cudaMemcpyAsync(q.data(), H.pool + H.q_region, q.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                  H.s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(H.s);
  return e == cudaSuccess ? BSAMG_OK : cuda_fail(e, "cudaMemcpyAsync(frame download)");
}

// ---- reading (ReadQ, :184-443) ----

struct Text {
  std::vector<char> buf;
  std::vector<size_t> off, len;  // records
};

bool read_text(const char* path, Text& T) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return false;
  std::fseek(f, 0, SEEK_END);
  long sz = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  T.buf.resize((size_t)std::max(0L, sz) + 1);
  bool ok = sz >= 0 && std::fread(T.buf.data(), 1, (size_t)sz, f) == (size_t)sz;
  std::fclose(f);
  if (!ok) return false;
  T.buf[sz] = 0;
  for (size_t i = 0; i < (size_t)sz;) {
    size_t e = i;
    while (e < (size_t)sz && T.buf[e] != '\n') e++;
    size_t n = e - i;
    if (n && T.buf[i + n - 1] == '\r') n--;
    T.off.push_back(i);
    T.len.push_back(n);
    i = e + 1;
  }
  return true;
}

// the characters [col, col+w) of record ln, blank-padded (PAD='YES')
void field(const Text& T, size_t ln, int col, int w, char* out) {
  for (int c = 0; c < w; c++) out[c] = (size_t)(col + c) < T.len[ln] ? T.buf[T.off[ln] + col + c] : ' ';
  out[w] = 0;
}

bool get_int(const Text& T, size_t ln, int col, int w, int* v) {
  char b[32], *e;
  field(T, ln, col, w, b);
  long x = std::strtol(b, &e, 10);
  while (*e == ' ') e++;
  if (*e) return false;
  *v = (int)x;
  return true;
}

// an F25.12 field as F25.12 output writes it (decimal point required; a
// blank field reads as 0)
bool get_real(const Text& T, size_t ln, int col, double* v) {
  char b[32], *e;
  field(T, ln, col, kField, b);
  bool blank = true, point = false;
  for (int c = 0; c < kField; c++) {
    if (b[c] != ' ') blank = false;
    if (b[c] == '.') point = true;
  }
  if (blank) {
    *v = 0.0;
    return true;
  }
  if (!point) return false;
  *v = std::strtod(b, &e);
  while (*e == ' ') e++;
  return *e == 0;
}

struct Block {
  int level, mx[3], mg[3][2];
  double dx[3], xl[3], xu[3];
  size_t data;  // first data record
};

}  // namespace

double xupper_of(const Hier& H, const HostPatch& P, int d) {
  // the root's xupper as given to RootInit (bsamroutines.f90:267-413);
  // MakeNewGrid's mbounds(2)*parent%dx + parent%xlower (:1752); otherwise
  // xlower + mx*dx
  if (P.level <= 0 && H.has_root_xupper) return H.root_xupper[d];
  if (P.level > 0 && P.parent >= 0) {
    const HostPatch& Q = H.patches[P.parent];
    return (double)P.mbounds[d][1] * Q.dx[d] + Q.xlower[d];
  }
  return P.xlower[d] + (double)P.mx[d] * P.dx[d];
}

int after_step_stats(Hier& H, int finest, double* integral, long long* meshsize) {
  if (!H.committed || finest < 0 || finest > kMaxDepth || !integral) return BSAMG_ERR_ARG;
  int r = set_device(H);
  if (r) return r;
  int nd = H.ndims;
  // which of AfterStep2D/3D's sums the plugin has (bit 0: the integral of
  // phi, bit 1: CH's energy)
  int which = find_plugin(H.problem)->stats(nd);
  int mass = which & 1;
  int energy = (which >> 1) & 1;
  long long ms = 0;
  int total = 0;
  for (int l = 0; l <= finest; l++) {
    const LevelT& L = H.L(l);
    total += L.nblk[kKindInterior] + (l > 0 ? L.nblk[kKindCoarse] : 0);
    for (int p : L.patches) {
      const HostPatch& P = H.patches[p];
      long long pm = 1, pc = 1;
      for (int d = 0; d < nd; d++) {
        pm *= P.mx[d];
        pc *= P.mx[d] / 2;
      }
      ms += l == 0 ? pm : pm - pc;  // GetMeshSize, bsamroutines.f90:846-868
    }
  }
  if (meshsize) *meshsize = ms;
  integral[0] = integral[1] = 0.0;
  if (total == 0) return BSAMG_OK;
  double* partial = nullptr;
  cudaError_t e = dev_alloc(H, (void**)&partial, sizeof(double) * 2 * (size_t)total);
  if (e != cudaSuccess) return cuda_fail(e, "device allocation (stats)");
  LaunchCtx c = H.lc();
  int pofs = 0, n = 0;
  for (int l = finest; l >= 0; l--) {
    const LevelT& L = H.L(l);
    n += launch_stats(c, L.d_blk[kKindInterior], L.nblk[kKindInterior], false, mass, energy, partial, pofs);
    pofs += L.nblk[kKindInterior];
    if (l > 0) {
      n += launch_stats(c, L.d_blk[kKindCoarse], L.nblk[kKindCoarse], true, mass, energy, partial, pofs);
      pofs += L.nblk[kKindCoarse];
    }
  }
  n += launch_stats_finish(H.s, partial, total, H.d_norm);
  if ((r = after_launch(H, n))) return r;
  e = cudaMemcpyAsync(H.h_norm, H.d_norm, 2 * sizeof(double), cudaMemcpyDeviceToHost, H.s);
  cudaFreeAsync(partial, H.s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(H.s);
  if (e != cudaSuccess) return cuda_fail(e, "after-step statistics");
  integral[0] = H.h_norm[0];
  integral[1] = H.h_norm[1];
  return BSAMG_OK;
}

// q(0:mx+1) of a patch's ghosted array a (all variables, any mbc): into
// out (gather, when b is null) or from b back into a (scatter)
void inner_cells(const Hier& H, const HostPatch& P, const double* a, const double* b, std::vector<double>& out,
                 double* a_out = nullptr) {
  int nd = H.ndims, s = H.mbc - 1;
  int e[3] = {P.mx[0] + 2, P.mx[1] + 2, nd == 3 ? P.mx[2] + 2 : 1};
  size_t cells = (size_t)e[0] * e[1] * e[2];
  if (!b) out.resize(cells * H.nrvars);
  size_t t = 0;
  for (int v = 0; v < H.nrvars; v++)
    for (int k = 0; k < e[2]; k++)
      for (int j = 0; j < e[1]; j++)
        for (int i = 0; i < e[0]; i++, t++) {
          size_t c = (size_t)v * P.sq + ((size_t)(nd == 3 ? k + s : 0) * P.qn[1] + (j + s)) * P.qn[0] + (i + s);
          if (b) a_out[c] = b[t];
          else out[t] = a[c];
        }
}

int write_q(Hier& H, const char* path, double time, int finest) {
  if (!H.committed || !path || finest < 0 || finest > kMaxDepth) return BSAMG_ERR_ARG;
  int r = set_device(H);
  if (r) return r;
  std::vector<double> q;
  if ((r = download_q(H, q))) return r;
  FILE* f = std::fopen(path, "wb");
  if (!f) return io_fail("cannot open the frame file for writing");
  bool ok = write_head(f, time, finest);
  std::vector<double> inner;
  for (int l = 0; l <= finest && ok; l++)
    for (int p : H.L(l).patches) {
      const HostPatch& P = H.patches[p];
      double xu[3];
      for (int d = 0; d < 3; d++) xu[d] = xupper_of(H, P, d);
      const double* src = q.data() + (P.oq - H.q_region);
      if (H.mbc > 1) {  // the records are q(0:mx+1) (OutputQ, :114-126)
        inner_cells(H, P, src, nullptr, inner);
        src = inner.data();
      }
      ok = ok && write_block(f, H.ndims, H.nrvars, P.level, P.dx, P.xlower, xu, P.mx, P.mglobal, src);
    }
  if (std::fclose(f) != 0) ok = false;
  return ok ? BSAMG_OK : io_fail("writing the frame file failed");
}

int write_uniform_q(Hier& H, const char* path, double time, int finest) {
  if (!H.committed || !path || finest < 0 || finest > kMaxDepth || H.L(0).patches.empty()) return BSAMG_ERR_ARG;
  int r = set_device(H);
  if (r) return r;
  int nd = H.ndims, nv = H.nrvars;
  const HostPatch& R = H.patches[H.L(0).patches[0]];
  int n[3] = {R.mx[0], R.mx[1], nd == 3 ? R.mx[2] : 1};
  auto ghosted = [&](const int* m) { return (size_t)(m[0] + 2) * (m[1] + 2) * (nd == 3 ? m[2] + 2 : 1); };
  int nf[3] = {n[0] << finest, n[1] << finest, nd == 3 ? n[2] << finest : 1};
  size_t fine_elems = ghosted(nf) * nv;
  size_t need = 2 * fine_elems * sizeof(double);
  {
    std::lock_guard<std::mutex> lk(H.ctx->mu);
    if (H.ctx->budget && H.ctx->used + need > H.ctx->budget) return BSAMG_ERR_BUDGET;
    H.ctx->used += need;
  }
  auto release = [&]() {
    std::lock_guard<std::mutex> lk(H.ctx->mu);
    H.ctx->used -= std::min(H.ctx->used, need);
  };
  double* buf[2] = {nullptr, nullptr};
  cudaError_t e = dev_alloc(H, (void**)&buf[0], fine_elems * sizeof(double));
  if (e == cudaSuccess) e = dev_alloc(H, (void**)&buf[1], fine_elems * sizeof(double));
  // uniform level 0 = the root's q(0:mx+1) (bsaminputoutput.f90:476-480)
  int launches = 0;
  if (e == cudaSuccess) {
    int g[3] = {1, 1, 1}, un[3] = {n[0] + 2, n[1] + 2, nd == 3 ? n[2] + 2 : 1};
    launches += launch_uniform_scatter(H.s, nd, H.pool, R.oq + origin_of(H, R.qn), R.sq, R.qn, R.mx, g, buf[0], un, nv);
  }
  double dx[3] = {R.dx[0], R.dx[1], R.dx[2]};
  int cur = 0;
  for (int l = 1; l <= finest && e == cudaSuccess; l++) {
    int m[3] = {2 * n[0], 2 * n[1], nd == 3 ? 2 * n[2] : 1};
    size_t cs = ghosted(n), fs = ghosted(m);
    for (int v = 0; v < nv; v++)
      launches += launch_uniform_prolong(H.s, nd, buf[cur] + v * cs, buf[1 - cur] + v * fs, n);
    for (int d = 0; d < nd; d++) dx[d] = dx[d] / 2.0;
    int un[3] = {m[0] + 2, m[1] + 2, nd == 3 ? m[2] + 2 : 1};
    for (int p : H.L(l).patches) {  // CopyPatchToUniformGrid, in visiting order
      const HostPatch& P = H.patches[p];
      int g[3] = {P.mglobal[0][0], P.mglobal[1][0], P.mglobal[2][0]};
      launches += launch_uniform_scatter(H.s, nd, H.pool, P.oq + origin_of(H, P.qn), P.sq, P.qn, P.mx, g, buf[1 - cur],
                                         un, nv);
    }
    cur = 1 - cur;
    std::memcpy(n, m, sizeof(n));
    e = cudaGetLastError();
  }
  if ((r = after_launch(H, launches))) {
    cudaFreeAsync(buf[0], H.s);
    cudaFreeAsync(buf[1], H.s);
    release();
    return r;
  }
  std::vector<double> u;
  if (e == cudaSuccess) {
    u.resize(ghosted(n) * nv);
    e = cudaMemcpyAsync(u.data(), buf[cur], u.size() * sizeof(double), cudaMemcpyDeviceToHost, H.s);
  }
  if (buf[0]) cudaFreeAsync(buf[0], H.s);
  if (buf[1]) cudaFreeAsync(buf[1], H.s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(H.s);
  release();
  if (e != cudaSuccess) return cuda_fail(e, "uniform mesh");
  FILE* f = std::fopen(path, "wb");
  if (!f) return io_fail("cannot open the uniform-mesh file for writing");
  double xu[3];
  int mg[3][2];
  for (int d = 0; d < 3; d++) {
    xu[d] = xupper_of(H, R, d);
    mg[d][0] = 1;
    mg[d][1] = n[d];
  }
  bool ok = write_head(f, time, 0) && write_block(f, nd, nv, 0, dx, R.xlower, xu, n, mg, u.data());
  if (std::fclose(f) != 0) ok = false;
  return ok ? BSAMG_OK : io_fail("writing the uniform-mesh file failed");
}

// Restart from a frame file.  The result copies `root`'s levels <= 0,
// replaces the root's q (ghost layers included) by the file's and adds the
// file's refinement patches with ids first_id, first_id + 1, ...  The
// checks of the root block are ReadQ's (:296-336, including its one-sided
// dx test).  Unlike ReadQ, whose restart patches all hang off the youngest
// patch of the level below (:246), each patch gets the patch of the level
// below that contains it as parent, with mbounds and mthbc as MakeNewGrid
// sets them, and qold = q.  Restart patches only feed TransferValues of the
// first regrid, so a regrid result does not depend on that choice.
int read_q(Hier& root, const char* path, int first_id, double* time, bsamg_hier** out) {
  if (!root.committed || !path || !out) return BSAMG_ERR_ARG;
  int r = set_device(root);
  if (r) return r;
  Text T;
  if (!read_text(path, T)) return io_fail("cannot read the frame file");
  int nd = root.ndims, nv = root.nrvars;
  const HostPatch* R = nullptr;
  for (const HostPatch& P : root.patches)
    if (P.level == 0) {
      R = &P;
      break;
    }
  if (!R) return BSAMG_ERR_ARG;
  double t;
  int finest;
  if (T.off.size() < 2 || !get_real(T, 0, 0, &t) || !get_int(T, 1, 0, 3, &finest))
    return io_fail("frame file: bad time or level record");
  if (finest < 0 || finest > kMaxDepth) return io_fail("frame file: finest level out of range");
  std::vector<Block> blocks;
  size_t ln = 2;
  for (int lvl = 0; lvl <= finest; lvl++) {
    for (;;) {
      if (ln >= T.off.size()) goto parsed;  // end of file
      int level, rnd, ratio, rnv;
      if (ln + 1 >= T.off.size() || !get_int(T, ln + 1, 0, 3, &level) || !get_int(T, ln + 1, 4, 3, &rnd) ||
          !get_int(T, ln + 1, 8, 3, &ratio) || !get_int(T, ln + 1, 12, 3, &rnv))
        return io_fail("frame file: bad patch header");
      if (level != lvl) break;  // read again for the next level
      ln += 2;
      if (rnd != nd) return io_fail("frame file: ndims differs from the hierarchy's");
      if (ratio != 2) return io_fail("frame file: refinement ratio is not 2");
      if (rnv != nv) return io_fail("frame file: nrvars differs from the hierarchy's");
      if (ln + 5 > T.off.size()) return io_fail("frame file: truncated patch header");
      Block B{};
      B.level = level;
      for (int d = 0; d < 3; d++) {
        B.mx[d] = 1;
        B.mg[d][0] = B.mg[d][1] = 1;
      }
      for (int d = 0; d < nd; d++)
        if (!get_real(T, ln, 26 * d, &B.dx[d]) || !get_real(T, ln + 1, 26 * d, &B.xl[d]) ||
            !get_real(T, ln + 2, 26 * d, &B.xu[d]) || !get_int(T, ln + 3, 9 * d, 8, &B.mx[d]) ||
            !get_int(T, ln + 4, 18 * d, 8, &B.mg[d][0]) || !get_int(T, ln + 4, 18 * d + 9, 8, &B.mg[d][1]))
          return io_fail("frame file: bad patch geometry");
      ln += 5;
      for (int d = 0; d < nd; d++)
        if (B.mx[d] < 2 || B.mx[d] > (1 << 24)) return io_fail("frame file: bad patch extents");
      if (level == 0) {
        const double small = 1.0e-08;
        for (int d = 0; d < nd; d++) {
          if (B.dx[d] - R->dx[d] > small) return io_fail("frame file: root dx differs");
          if (std::fabs(B.xl[d] - R->xlower[d]) > small) return io_fail("frame file: root xlower differs");
          if (std::fabs(B.xu[d] - xupper_of(root, *R, d)) > small) return io_fail("frame file: root xupper differs");
          if (B.mx[d] != R->mx[d]) return io_fail("frame file: root mx differs");
          if (B.mg[d][0] != 1 || B.mg[d][1] != R->mx[d]) return io_fail("frame file: root mglobal differs");
        }
      } else {
        for (int d = 0; d < nd; d++)
          if (B.mg[d][0] % 2 != 1 || B.mg[d][1] % 2 != 0 || B.mg[d][1] - B.mg[d][0] + 1 != B.mx[d])
            return io_fail("frame file: refinement patch not aligned with its parent level");
      }
      B.data = ln;
      size_t plane = (size_t)(B.mx[0] + 2) * (B.mx[1] + 2) * (nd == 3 ? B.mx[2] + 2 : 1);
      if (ln + plane > T.off.size()) return io_fail("frame file: truncated patch data");
      ln += plane;
      blocks.push_back(B);
    }
  }
parsed:
  // the new hierarchy: root's levels <= 0, then the file's patches
  bsamg_hier* nh = nullptr;
  r = bsamg_hier_create(root.ctx, nd, nv, root.mbc, root.problem, root.params.data(), (int)root.params.size(),
                        root.pp.qpo, &nh);
  if (r) return r;
  nh->has_root_xupper = root.has_root_xupper;
  std::memcpy(nh->root_xupper, root.root_xupper, sizeof(root.root_xupper));
  auto fail = [&](int rc) {
    bsamg_hier_destroy(nh);
    return rc;
  };
  struct Geo {
    int level, id, parent_id, mx[3], mg[6], mb[6], thbc[6];
    double dx[3], xl[3];
  };
  std::vector<Geo> geo;
  for (const HostPatch& P : root.patches) {
    if (P.level > 0) continue;
    Geo G{};
    G.level = P.level, G.id = P.id, G.parent_id = P.parent_id;
    for (int d = 0; d < 3; d++) {
      G.mx[d] = P.mx[d];
      G.mg[2 * d] = P.mglobal[d][0], G.mg[2 * d + 1] = P.mglobal[d][1];
      G.mb[2 * d] = P.mbounds[d][0], G.mb[2 * d + 1] = P.mbounds[d][1];
      G.dx[d] = P.dx[d], G.xl[d] = P.xlower[d];
    }
    for (int f = 0; f < 6; f++) G.thbc[f] = P.mthbc[f];
    geo.push_back(G);
  }
  std::vector<int> block_of(geo.size(), -1);  // the block whose data a patch takes
  int next_id = first_id;
  for (size_t b = 0; b < blocks.size(); b++) {
    const Block& B = blocks[b];
    if (B.level == 0) {
      for (size_t g = 0; g < geo.size(); g++)
        if (geo[g].level == 0) block_of[g] = (int)b;
      continue;
    }
    int par = -1;
    for (size_t g = 0; g < geo.size() && par < 0; g++) {
      if (geo[g].level != B.level - 1) continue;
      bool in = true;
      for (int d = 0; d < nd; d++)
        if ((B.mg[d][0] + 1) / 2 < geo[g].mg[2 * d] || B.mg[d][1] / 2 > geo[g].mg[2 * d + 1]) in = false;
      if (in) par = (int)g;
    }
    if (par < 0) return fail(io_fail("frame file: refinement patch outside the level below"));
    const Geo& Q = geo[par];
    Geo G{};
    G.level = B.level, G.id = next_id++, G.parent_id = Q.id;
    for (int d = 0; d < 3; d++) {
      G.mx[d] = B.mx[d];
      G.mg[2 * d] = B.mg[d][0], G.mg[2 * d + 1] = B.mg[d][1];
      G.mb[2 * d] = G.mb[2 * d + 1] = 1;
      G.dx[d] = B.dx[d], G.xl[d] = B.xl[d];
      if (d < nd) {
        G.mb[2 * d] = (B.mg[d][0] + 1) / 2 - Q.mg[2 * d] + 1;
        G.mb[2 * d + 1] = B.mg[d][1] / 2 - Q.mg[2 * d] + 1;
      }
    }
    for (int f = 0; f < 6; f++) G.thbc[f] = f < 2 * nd ? kInternalBC : 10;
    for (int e = 0; e < nd; e++) {  // MakeNewGrid, bsamroutines.f90:1726-1741
      if (Q.thbc[2 * e] < kInternalBC && G.mb[2 * e] == 1) G.thbc[2 * e] = Q.thbc[2 * e];
      if (Q.thbc[2 * e + 1] < kInternalBC && G.mb[2 * e + 1] == Q.mx[e]) G.thbc[2 * e + 1] = Q.thbc[2 * e + 1];
    }
    geo.push_back(G);
    block_of.push_back((int)b);
  }
  for (const Geo& G : geo)
    if ((r = bsamg_patch_add(nh, G.level, G.id, G.parent_id, G.mx, G.mg, G.mb, G.thbc, G.dx, G.xl))) return fail(r);
  if ((r = bsamg_commit(nh))) return fail(r);
  Hier& N = *nh;
  // q image: the file's data where a block exists, else root's q; qold
  // likewise (qold = q for the file's patches)
  std::vector<double> qimg((size_t)N.q_len, 0.0);
  std::vector<double> rq;
  if ((r = download_q(root, rq))) return fail(r);
  bool bad = false;
  for (size_t p = 0; p < geo.size(); p++) {
    const HostPatch& D = N.patches[p];
    double* dq = qimg.data() + (D.oq - N.q_region);
    size_t plane = (size_t)D.sq;
    if (block_of[p] < 0) {
      const HostPatch& S = root.patches[root.id2idx.at(D.id)];
      std::memcpy(dq, rq.data() + (S.oq - root.q_region), plane * nv * sizeof(double));
      continue;
    }
    size_t d0 = blocks[block_of[p]].data;
    // the records are q(0:mx+1) (ReadQ2D/3D, :392-440): with mbc = 1 the
    // whole ghosted array, else its inner part; the second layer keeps the
    // persisting patch's values (a new patch's are zero)
    std::vector<double> inner, none;
    if (N.mbc > 1 && D.level <= 0 && root.id2idx.count(D.id)) {
      const HostPatch& S = root.patches[root.id2idx.at(D.id)];
      std::memcpy(dq, rq.data() + (S.oq - root.q_region), plane * nv * sizeof(double));
    }
    size_t recs = (size_t)(D.mx[0] + 2) * (D.mx[1] + 2) * (N.ndims == 3 ? D.mx[2] + 2 : 1);
    double* tgt = dq;
    if (N.mbc > 1) {
      inner.resize(recs * nv);
      tgt = inner.data();
    }
    int nt = host_threads();
    std::vector<char> okt(nt, 1);
    parallel(nt, [&](int t, int n) {
      size_t a = recs * t / n, b = recs * (t + 1) / n;
      for (size_t c = a; c < b; c++)
        for (int v = 0; v < nv; v++)
          if (!get_real(T, d0 + c, 27 * v, &tgt[(size_t)v * recs + c])) okt[t] = 0;
    });
    for (char o : okt) bad = bad || !o;
    if (N.mbc > 1) inner_cells(N, D, nullptr, inner.data(), none, dq);
  }
  if (bad) return fail(io_fail("frame file: bad data record"));
  cudaError_t e =
      cudaMemcpyAsync(N.pool + N.q_region, qimg.data(), qimg.size() * sizeof(double), cudaMemcpyHostToDevice, N.s);
  // qold: root's for the persisting levels, q for the file's patches
  for (size_t p = 0; p < geo.size() && e == cudaSuccess; p++) {
    const HostPatch& D = N.patches[p];
    size_t bytes = (size_t)D.sq * nv * sizeof(double);
    if (D.level <= 0) {  // the persisting levels keep qold and qc
      const HostPatch& S = root.patches[root.id2idx.at(D.id)];
      e = cudaMemcpyAsync(N.pool + D.oqold, root.pool + S.oqold, bytes, cudaMemcpyDeviceToDevice, N.s);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(N.pool + D.oqc, root.pool + S.oqc, (size_t)D.sc * nv * sizeof(double),
                            cudaMemcpyDeviceToDevice, N.s);
    } else {
      e = cudaMemcpyAsync(N.pool + D.oqold, N.pool + D.oq, bytes, cudaMemcpyDeviceToDevice, N.s);
    }
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(N.s);  // qimg is freed on return
  if (e != cudaSuccess) return fail(cuda_fail(e, "cudaMemcpyAsync(restart upload)"));
  if (time) *time = t;
  *out = nh;
  return BSAMG_OK;
}

}  // namespace bsamg

using namespace bsamg;

extern "C" {

int bsamg_after_step_stats(bsamg_hier* h, int finestlevel, double integral[2], long long* meshsize) {
  if (!h) return BSAMG_ERR_ARG;
  return after_step_stats(*h, finestlevel, integral, meshsize);
}

int bsamg_write_q(bsamg_hier* h, const char* path, double time, int finestlevel) {
  if (!h) return BSAMG_ERR_ARG;
  return write_q(*h, path, time, finestlevel);
}

int bsamg_write_uniform_q(bsamg_hier* h, const char* path, double time, int finestlevel) {
  if (!h) return BSAMG_ERR_ARG;
  return write_uniform_q(*h, path, time, finestlevel);
}

int bsamg_read_q(bsamg_hier* root, const char* path, int first_id, double* time, bsamg_hier** out) {
  if (!root) return BSAMG_ERR_ARG;
  return read_q(*root, path, first_id, time, out);
}

int bsamg_seed_spinodal(bsamg_hier* h, int id, unsigned long long seed, double mean, double amp) {
  if (!h || !h->committed || h->problem != BSAMG_PROBLEM_CH || h->nrvars != 2) return BSAMG_ERR_ARG;
  h->box_g_valid = false;
  auto it = h->id2idx.find(id);
  if (it == h->id2idx.end()) return BSAMG_ERR_NOT_FOUND;
  const HostPatch& P = h->patches[it->second];
  int r = set_device(*h);
  if (r) return r;
  int n = launch_seed_spinodal(h->s, h->ndims, h->mbc, h->pool + P.oq, P.sq, P.mx, seed, mean, amp, h->pp.eps2, P.dx[0]);
  return after_launch(*h, n);
}

int bsamg_format_f25_12(double x, char* out) {
  if (!out) return BSAMG_ERR_ARG;
  f25(x, out);
  out[kField] = 0;
  return BSAMG_OK;
}

int bsamg_format_stats_line(double time, const double integral[2], long long meshsize, char* out, size_t n) {
  if (!integral || !out) return BSAMG_ERR_ARG;
  std::string s = f25s(time) + f25s(integral[0]) + f25s(integral[1]) + " " + iw(meshsize, 8) + "\n";
  if (s.size() + 1 > n) return BSAMG_ERR_ARG;
  std::memcpy(out, s.c_str(), s.size() + 1);
  return BSAMG_OK;
}

}  // extern "C"
