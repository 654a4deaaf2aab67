// Device plugin of the Cahn-Hilliard problem, PROBLEM/CH/problem.f90: the
// convex-splitting implicit step of the CH equation for (phi, mu) solved by
// the pointwise 2x2 Newton smoother, its operator, source and boundary
// conditions, and its mixed-precision correction form.  The FP64 part keeps
// the reference's expressions and evaluation order (bit-identical to a
// reference build without fused multiply-adds).
#include "plugin_def.cuh"

namespace bsamg {

struct CH {
  static constexpr int kKind = BSAMG_PROBLEM_CH;
  static constexpr const char* kName = "ch";
  static constexpr int kNV = 2;
  static constexpr int kNParams = 2;  // dt, eps
  static constexpr bool kCoeffsOnly = true;
  static constexpr bool kBox = true;
  static constexpr bool kMixed = true;
  static constexpr int kMxBase = 1;    // phib
  static constexpr int kMxUpdate = 1;

  // SetProb (CH/problem.f90:12-34: eps from problemdata, eps2 = eps^2) and
  // the library's dt
  static void set_params(ProbParams& pp, const double* prm, int) {
    pp.dt = prm[0];
    pp.eps2 = prm[1] * prm[1];
  }
  // RelaxGrid2D/3D's constants for spacing h (CH/problem.f90:339-346, :575-582)
  static void coefficients(const ProbParams& pp, int ndims, double h, double* c) {
    double h2 = h * h;
    double k = ndims == 2 ? 4.0 : 6.0;
    c[0] = pp.dt / h2;        // tmp1, CH/problem.f90:341
    c[1] = pp.eps2 / h2;      // tmp2, :342
    c[2] = k * pp.eps2 / h2;  // tmp3, :343 (:579)
    c[3] = k * c[0];          // a(1,2), :346 (:582)
  }
  // UserBC2D reflects both variables (Neumann, CH/problem.f90:770-818);
  // UserBC3D sets 2 - q for both (Dirichlet 1, :842-877)
  static int bc_mask(int ndims) { return ndims == 3 ? 3 : 0; }
  // AfterStep2D: integral of phi and the energy (CH/problem.f90:149-183,
  // Energy2D :512-547); AfterStep3D: the integral (:186-215)
  static int stats(int ndims) { return ndims == 2 ? 3 : 1; }

  // RelaxGrid2D CH/problem.f90:349-367, RelaxGrid3D :589-612
  template <int DIM>
  __device__ __forceinline__ static void relax(const Cell64& x, const double* cf, const ProbParams&) {
    double* q0 = x.q;
    double* q1 = q0 + x.sq;
    const double* f0 = x.f;
    const double* f1 = f0 + x.sf;
    const long long c = x.c, fc = x.fc, sy = x.sy, sz = x.sz;
    double phi = q0[c];
    double a21 = -3.0 * sqr(phi) - cf[2];
    double b1, b2;
    if (DIM == 2) {
      b1 = f0[fc] + cf[0] * (q1[c - 1] + q1[c + 1] + q1[c - sy] + q1[c + sy]);
      b2 = f1[fc] - cf[1] * (q0[c + 1] + q0[c - 1] + q0[c + sy] + q0[c - sy]) - 2.0 * cube(phi);
    } else {
      b1 = f0[fc] + cf[0] * (q1[c - 1] + q1[c + 1] + q1[c - sy] + q1[c + sy] + q1[c - sz] + q1[c + sz]);
      b2 = f1[fc] - cf[1] * (q0[c + 1] + q0[c - 1] + q0[c + sy] + q0[c - sy] + q0[c + sz] + q0[c - sz]) -
           2.0 * cube(phi);
    }
    double det = 1.0 - cf[3] * a21;  // >= 1: a21 <= -tmp3 < 0
    // the reference's two divisions by det, :365-366 (:609-610), each
    // correctly rounded as `/` is, from one reciprocal
    double n0, n1;
    div2_rn(b1 - cf[3] * b2, b2 - a21 * b1, det, n0, n1);
    q0[c] = n0;
    q1[c] = n1;
  }

  // Operator2D/3D, CH/problem.f90:393-422, :638-669
  template <int DIM>
  __device__ __forceinline__ static void op(const double* a, long long c, long long sy, long long sz, long long ps,
                                            const QoldView&, const double* cf, const ProbParams&, double* r) {
    const double* a0 = a;
    const double* a1 = a + ps;
    r[0] = a0[c] - cf[0] * ulap<DIM>(a1, c, sy, sz);
    r[1] = a1[c] - cube(a0[c]) + cf[1] * ulap<DIM>(a0, c, sy, sz);
  }
  // Source2D/3D (CH/problem.f90:425-450, :672-697): f = (phi_old, -phi_old)
  template <int DIM>
  __device__ __forceinline__ static void source(const double*, long long, long long, long long, long long,
                                                const QoldView& qo, const double*, const ProbParams&, double* s) {
    const double o0 = qo.p[0];
    s[0] = o0;
    s[1] = -o0;
  }
  // SourceUpdate2D/3D is zero (CH/problem.f90:453-476, :700-721)
  template <int DIM>
  __device__ __forceinline__ static void source_update(const double*, long long, long long, long long, long long,
                                                       const QoldView&, const double*, const ProbParams&,
                                                       double* su) {
    su[0] = 0.0;
    su[1] = 0.0;
  }

  // ---- correction form (mixed path), FP32 ----
  static MxParams mx_params(const ProbParams&) { return MxParams{{0.f, 0.f, 0.f, 0.f}}; }

  // base plane phib = (float)qbar_phi; g = FP32 image of the FP64 residual
  // (mode 1: the stored rf; mode 2: f - N(qbar) recomputed)
  template <int DIM>
  __device__ __forceinline__ static void mx_prep(const Cell64& x, const double* rf, float* base, float* g, int mode,
                                                 const double* cf, const ProbParams&) {
    const double* q0 = x.q;
    const double* q1 = q0 + x.sq;
    const long long c = x.c, fc = x.fc;
    base[fc] = (float)q0[c];
    if (mode == 0) return;
    double r0, r1;
    if (mode == 1) {
      r0 = rf[fc];
      r1 = rf[x.sf + fc];
    } else {
      double o0 = q0[c] - cf[0] * ulap<DIM>(q1, c, x.sy, x.sz);
      double o1 = q1[c] - q0[c] * q0[c] * q0[c] + cf[1] * ulap<DIM>(q0, c, x.sy, x.sz);
      r0 = x.f[fc] - o0;
      r1 = x.f[x.sf + fc] - o1;
    }
    g[fc] = (float)r0;
    g[x.sf + fc] = (float)r1;
  }

  // red-black pointwise Newton on the correction (RelaxGrid2D/3D in
  // correction form), in arithmetic T (float on every level, double on the
  // coarsest; e, g and the base plane stay FP32, cf is in T):
  //   a21 = -3 (pb + e)^2 - tmp3
  //   b1  = g1 + tmp1 * sum(e_mu neighbours)
  //   b2  = g2 - tmp2 * sum(e_phi neighbours) - e^2 (3 pb + 2 e)
  template <int DIM, typename T>
  __device__ __forceinline__ static void mx_relax(const Cell32& x, const T* cf, const MxParams&) {
    float* e0 = x.e;
    float* e1 = e0 + x.sq;
    const long long c = x.c, fc = x.fc, sy = x.sy, sz = x.sz;
    T tmp1 = cf[0], tmp2 = cf[1], tmp3 = cf[2], a12 = cf[3];
    T pb = x.base[fc];
    T xx = e0[c];
    T w = pb + xx;
    T a21 = T(-3) * w * w - tmp3;
    T s1, s0;
    if (DIM == 2) {
      s1 = T(e1[c - 1]) + T(e1[c + 1]) + T(e1[c - sy]) + T(e1[c + sy]);
      s0 = T(e0[c + 1]) + T(e0[c - 1]) + T(e0[c + sy]) + T(e0[c - sy]);
    } else {
      s1 = T(e1[c - 1]) + T(e1[c + 1]) + T(e1[c - sy]) + T(e1[c + sy]) + T(e1[c - sz]) + T(e1[c + sz]);
      s0 = T(e0[c + 1]) + T(e0[c - 1]) + T(e0[c + sy]) + T(e0[c - sy]) + T(e0[c + sz]) + T(e0[c - sz]);
    }
    T b1 = T(x.g[fc]) + tmp1 * s1;
    T b2 = T(x.g[x.sf + fc]) - tmp2 * s0 - xx * xx * (T(3) * pb + T(2) * xx);
    T rdet = T(1) / (T(1) - a12 * a21);
    e0[c] = (float)((b1 - a12 * b2) * rdet);
    e1[c] = (float)((b2 - a21 * b1) * rdet);
  }

  // M(e) = N(pb + e) - N(pb), written so that no term cancels
  template <int DIM>
  __device__ __forceinline__ static void mx_op(const float* e, long long c, long long sy, long long sz, long long ps,
                                               const float* base, long long fc, long long, const float* cf,
                                               const MxParams&, float* m) {
    const float* e0 = e;
    const float* e1 = e + ps;
    float pb = base[fc];
    float xx = e0[c];
    m[0] = xx - cf[0] * ulap<DIM>(e1, c, sy, sz);
    m[1] = e1[c] - xx * (3.0f * pb * (pb + xx) + xx * xx) + cf[1] * ulap<DIM>(e0, c, sy, sz);
  }
};

BSAMG_PLUGIN(CH)

}  // namespace bsamg
