// Device plugin of the three-variable growth problem (no reference
// counterpart: the reference's 3D BioGrowth is a stub without pressure).
// phi and the nutrient n follow BioGrowth's equations with 2*ndims
// neighbours (growth gamma (phi_old + 1)/2, uptake lambda (phi_old + 1)/2,
// source (1 + dt) phi_old for phi), and the pressure p solves
// -ULap(p)/h^2 - cpress phi n = 0.  On physical faces phi is reflected,
// n = 2 - n (value 1) and p = -p (value 0).  The pointwise relaxation
// updates phi, then n, then p from the new phi and n.
#include "plugin_def.cuh"

namespace bsamg {

struct Growth {
  static constexpr int kKind = BSAMG_PROBLEM_GROWTH;
  static constexpr const char* kName = "growth";
  static constexpr int kNV = 3;
  static constexpr int kNParams = 6;  // dt, eps, gamma, lambda, c0, cpress
  static constexpr bool kCoeffsOnly = false;
  static constexpr bool kBox = false;
  static constexpr bool kMixed = true;
  static constexpr int kMxBase = 4;    // phib, nb, G, U
  static constexpr int kMxUpdate = 2;  // phib and nb follow qbar

  static void set_params(ProbParams& pp, const double* prm, int) {
    pp.dt = prm[0];
    pp.eps2 = prm[1] * prm[1];
    pp.gamma = prm[2];
    pp.lambda = prm[3];
    pp.czero = prm[4];
    pp.cpress = prm[5];
  }
  // BioGrowth's RelaxGrid2D constants (BioGrowth/problem.f90:276-288) with
  // 2*ndims neighbours
  static void coefficients(const ProbParams& pp, int ndims, double h, double* c) {
    double h2 = h * h;
    double k = 2.0 * ndims;
    c[0] = pp.dt * pp.eps2 / h2;
    c[1] = 1.0 / h2;
    c[2] = k * c[0] + 1.0;
    c[3] = k * c[1];
  }
  static int bc_mask(int) { return 2 | (4 << 8); }
  static int stats(int) { return 1; }

  template <int DIM>
  __device__ __forceinline__ static void relax(const Cell64& x, const double* cf, const ProbParams& pp) {
    double* q0 = x.q;
    double* q1 = q0 + x.sq;
    double* q2 = q1 + x.sq;
    const double* f0 = x.f;
    const double* f1 = f0 + x.sf;
    const double* f2 = f1 + x.sf;
    const long long c = x.c, fc = x.fc, sy = x.sy, sz = x.sz;
    double dt = pp.dt;
    double phi = q0[c];
    double ol = x.qold[c];
    double tmp2 = cf[2] + dt * sqr(phi);
    double s0 = q0[c - 1] + q0[c + 1] + q0[c - sy] + q0[c + sy];
    double s1 = q1[c + 1] + q1[c - 1] + q1[c + sy] + q1[c - sy];
    double s2 = q2[c + 1] + q2[c - 1] + q2[c + sy] + q2[c - sy];
    if (DIM == 3) {
      s0 = s0 + q0[c - sz] + q0[c + sz];
      s1 = s1 + q1[c + sz] + q1[c - sz];
      s2 = s2 + q2[c + sz] + q2[c - sz];
    }
    double np = (f0[fc] + dt * (pp.gamma * 0.5 * (ol + 1.0)) * (q1[c] - pp.czero) + cf[0] * s0) / tmp2;
    double tmp4 = cf[3] + (pp.lambda * 0.5 * (ol + 1.0));
    double nn = (f1[fc] + cf[1] * s1) / tmp4;
    q0[c] = np;
    q1[c] = nn;
    q2[c] = (f2[fc] + cf[1] * s2 + pp.cpress * np * nn) / cf[3];
  }

  template <int DIM>
  __device__ __forceinline__ static void op(const double* a, long long c, long long sy, long long sz, long long ps,
                                            const QoldView& qo, const double* cf, const ProbParams& pp, double* r) {
    const double o0 = qo.p[0];
    const double* a0 = a;
    const double* a1 = a + ps;
    const double* a2 = a + 2 * ps;
    double dt = pp.dt;
    r[0] = a0[c] - cf[0] * ulap<DIM>(a0, c, sy, sz) + dt * cube(a0[c]) -
           dt * (pp.gamma * 0.5 * (o0 + 1.0)) * (a1[c] - pp.czero);
    r[1] = -cf[1] * ulap<DIM>(a1, c, sy, sz) + (pp.lambda * 0.5 * (o0 + 1.0)) * a1[c];
    r[2] = -cf[1] * ulap<DIM>(a2, c, sy, sz) - pp.cpress * a0[c] * a1[c];
  }
  template <int DIM>
  __device__ __forceinline__ static void source(const double*, long long, long long, long long, long long,
                                                const QoldView& qo, const double*, const ProbParams& pp, double* s) {
    const double o0 = qo.p[0];
    s[0] = (1.0 + pp.dt) * o0;
    s[1] = 0.0;
    s[2] = 0.0;
  }
  template <int DIM>
  __device__ __forceinline__ static void source_update(const double*, long long, long long, long long, long long,
                                                       const QoldView&, const double*, const ProbParams&,
                                                       double* su) {
    su[0] = 0.0;
    su[1] = 0.0;
    su[2] = 0.0;
  }

  // ---- correction form (mixed path), FP32 ----
  // Base planes: phib, nb (the frozen phi and n), G = gamma (phi_old + 1)/2
  // and U = lambda (phi_old + 1)/2.  With w = phib + e_phi:
  //   M0 = e_phi - c0 ULap(e_phi) + dt e_phi (3 phib w + e_phi^2) - dt G e_n
  //   M1 = -c1 ULap(e_n) + U e_n
  //   M2 = -c1 ULap(e_p) - cp (phib e_n + e_phi nb + e_phi e_n)
  // and the smoother is the FP64 one rewritten for e so that no term
  // cancels: e_phi = (g0 + dt G e_n + c0 sum(e_phi) - dt phib e_phi
  // (2 phib + e_phi)) / (c2 + dt w^2), e_n = (g1 + c1 sum(e_n)) / (c3 + U),
  // e_p = (g2 + c1 sum(e_p) + cp (phib e_n + e_phi nb + e_phi e_n)) / c3.
  static MxParams mx_params(const ProbParams& pp) { return MxParams{{(float)pp.dt, (float)pp.cpress, 0.f, 0.f}}; }

  template <int DIM>
  __device__ __forceinline__ static void mx_prep(const Cell64& x, const double* rf, float* base, float* g, int mode,
                                                 const double* cf, const ProbParams& pp) {
    const double* q0 = x.q;
    const double* q1 = q0 + x.sq;
    const double* q2 = q1 + x.sq;
    const long long c = x.c, fc = x.fc, sf = x.sf;
    double ol = x.qold[c];
    double G = pp.gamma * 0.5 * (ol + 1.0), U = pp.lambda * 0.5 * (ol + 1.0);
    base[fc] = (float)q0[c];
    base[sf + fc] = (float)q1[c];
    base[2 * sf + fc] = (float)G;
    base[3 * sf + fc] = (float)U;
    if (mode == 0) return;
    double r[3];
    if (mode == 1) {
      for (int v = 0; v < 3; v++) r[v] = rf[v * sf + fc];
    } else {
      double phi = q0[c];
      double o0 = phi - cf[0] * ulap<DIM>(q0, c, x.sy, x.sz) + pp.dt * phi * phi * phi - pp.dt * G * (q1[c] - pp.czero);
      double o1 = -cf[1] * ulap<DIM>(q1, c, x.sy, x.sz) + U * q1[c];
      double o2 = -cf[1] * ulap<DIM>(q2, c, x.sy, x.sz) - pp.cpress * phi * q1[c];
      r[0] = x.f[fc] - o0;
      r[1] = x.f[sf + fc] - o1;
      r[2] = x.f[2 * sf + fc] - o2;
    }
    for (int v = 0; v < 3; v++) g[v * sf + fc] = (float)r[v];
  }

  // the correction smoother in arithmetic T (float on every level, double
  // on the coarsest; e, g and the base planes stay FP32, cf is in T)
  template <int DIM, typename T>
  __device__ __forceinline__ static void mx_relax(const Cell32& x, const T* cf, const MxParams& mp) {
    float* e0 = x.e;
    float* e1 = e0 + x.sq;
    float* e2 = e1 + x.sq;
    const long long c = x.c, fc = x.fc, sy = x.sy, sz = x.sz, sf = x.sf;
    const float* base = x.base;
    const float* g = x.g;
    T dt = mp.p[0], cp = mp.p[1];
    T pb = base[fc], nb = base[sf + fc], G = base[2 * sf + fc], U = base[3 * sf + fc];
    T c0 = cf[0], c1 = cf[1], c2 = cf[2], c3 = cf[3];
    T s0 = T(e0[c - 1]) + T(e0[c + 1]) + T(e0[c - sy]) + T(e0[c + sy]);
    T s1 = T(e1[c - 1]) + T(e1[c + 1]) + T(e1[c - sy]) + T(e1[c + sy]);
    T s2 = T(e2[c - 1]) + T(e2[c + 1]) + T(e2[c - sy]) + T(e2[c + sy]);
    if (DIM == 3) {
      s0 += T(e0[c - sz]) + T(e0[c + sz]);
      s1 += T(e1[c - sz]) + T(e1[c + sz]);
      s2 += T(e2[c - sz]) + T(e2[c + sz]);
    }
    T xx = e0[c], y = e1[c];
    T w = pb + xx;
    T xn = (T(g[fc]) + dt * G * y + c0 * s0 - dt * pb * xx * (T(2) * pb + xx)) / (c2 + dt * w * w);
    T yn = (T(g[sf + fc]) + c1 * s1) / (c3 + U);
    T zn = (T(g[2 * sf + fc]) + c1 * s2 + cp * (pb * yn + xn * nb + xn * yn)) / c3;
    e0[c] = (float)xn;
    e1[c] = (float)yn;
    e2[c] = (float)zn;
  }

  template <int DIM>
  __device__ __forceinline__ static void mx_op(const float* e, long long c, long long sy, long long sz, long long ps,
                                               const float* base, long long fc, long long sf, const float* cf,
                                               const MxParams& mp, float* m) {
    const float* e0 = e;
    const float* e1 = e + ps;
    const float* e2 = e + 2 * ps;
    float dt = mp.p[0], cp = mp.p[1];
    float pb = base[fc], nb = base[sf + fc], G = base[2 * sf + fc], U = base[3 * sf + fc];
    float xx = e0[c], y = e1[c];
    m[0] = xx - cf[0] * ulap<DIM>(e0, c, sy, sz) + dt * xx * (3.0f * pb * (pb + xx) + xx * xx) - dt * G * y;
    m[1] = -cf[1] * ulap<DIM>(e1, c, sy, sz) + U * y;
    m[2] = -cf[1] * ulap<DIM>(e2, c, sy, sz) - cp * (pb * y + xx * nb + xx * y);
  }
};

BSAMG_PLUGIN(Growth)

}  // namespace bsamg
