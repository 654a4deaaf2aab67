// Device plugin of the BioGrowth problem, PROBLEM/BioGrowth/problem.f90: a
// CH-type volume fraction phi with growth G(phi_old) and a quasi-steady
// nutrient n with uptake U(phi_old), relaxed pointwise (phi from its lagged
// equation, then n).  The reference's 3D routines are stubs that return
// zeros (BioGrowth/problem.f90:445-522), restated as such.  No mixed form.
#include "plugin_def.cuh"

namespace bsamg {

struct BioGrowth {
  static constexpr int kKind = BSAMG_PROBLEM_BIOGROWTH;
  static constexpr const char* kName = "biogrowth";
  static constexpr int kNV = 2;
  static constexpr int kNParams = 5;  // dt, eps, gamma, lambda, c0
  static constexpr bool kCoeffsOnly = false;  // dt, gamma, lambda, c0 are kernel arguments
  static constexpr bool kBox = false;
  static constexpr bool kMixed = false;
  static constexpr int kMxBase = 0, kMxUpdate = 0;

  // SetProb (BioGrowth/problem.f90:12-34): eps, gamma, lambda, c0
  static void set_params(ProbParams& pp, const double* prm, int) {
    pp.dt = prm[0];
    pp.eps2 = prm[1] * prm[1];
    pp.gamma = prm[2];
    pp.lambda = prm[3];
    pp.czero = prm[4];
  }
  // RelaxGrid2D's constants for spacing h (BioGrowth/problem.f90:276-288)
  static void coefficients(const ProbParams& pp, int, double h, double* c) {
    double h2 = h * h;
    c[0] = pp.dt * pp.eps2 / h2;  // tmp1, BioGrowth/problem.f90:277
    c[1] = 1.0 / h2;              // tmp3, :278
    c[2] = 4.0 * c[0] + 1.0;      // first two terms of tmp2, :282
    c[3] = 4.0 * c[1];            // first term of tmp4, :288
  }
  // UserBC2D: phi reflected, n = 2 - n (BioGrowth/problem.f90:623-673);
  // UserBC3D: 2 - q for both (:679-736)
  static int bc_mask(int ndims) { return ndims == 3 ? 3 : 2; }
  // AfterStep2D: integral of phi (BioGrowth/problem.f90:107-136); AfterStep3D
  // is empty (:139-152)
  static int stats(int ndims) { return ndims == 3 ? 0 : 1; }

  // RelaxGrid2D BioGrowth/problem.f90:280-294; RelaxGrid3D :467-476 (zeros)
  template <int DIM>
  __device__ __forceinline__ static void relax(const Cell64& x, const double* cf, const ProbParams& pp) {
    double* q0 = x.q;
    double* q1 = q0 + x.sq;
    const long long c = x.c;
    if (DIM == 2) {
      const double* f0 = x.f;
      const double* f1 = f0 + x.sf;
      const long long fc = x.fc, sy = x.sy;
      double dt = pp.dt;
      double phi = q0[c];
      double ol = x.qold[c];
      double tmp2 = cf[2] + dt * sqr(phi);
      q0[c] = (f0[fc] + dt * (pp.gamma * 0.5 * (ol + 1.0)) * (q1[c] - pp.czero) +
               cf[0] * (q0[c - 1] + q0[c + 1] + q0[c - sy] + q0[c + sy])) / tmp2;
      double tmp4 = cf[3] + (pp.lambda * 0.5 * (ol + 1.0));
      q1[c] = (f1[fc] + cf[1] * (q1[c + 1] + q1[c - 1] + q1[c + sy] + q1[c - sy])) / tmp4;
    } else {
      q0[c] = 0.0;
      q1[c] = 0.0;
    }
  }

  // Operator2D BioGrowth/problem.f90:320-353; Operator3D :497-522 (zeros)
  template <int DIM>
  __device__ __forceinline__ static void op(const double* a, long long c, long long sy, long long sz, long long ps,
                                            const QoldView& qo, const double* cf, const ProbParams& pp, double* r) {
    const double o0 = qo.p[0];
    const double* a0 = a;
    const double* a1 = a + ps;
    if (DIM == 2) {
      double dt = pp.dt;
      r[0] = a0[c] - cf[0] * ulap<DIM>(a0, c, sy, sz) + dt * cube(a0[c]) -
             dt * (pp.gamma * 0.5 * (o0 + 1.0)) * (a1[c] - pp.czero);
      r[1] = -cf[1] * ulap<DIM>(a1, c, sy, sz) + (pp.lambda * 0.5 * (o0 + 1.0)) * a1[c];
    } else {
      r[0] = 0.0;
      r[1] = 0.0;
    }
  }
  // Source2D (BioGrowth/problem.f90:356-379): f1 = (1 + dt) phi_old, f2 = 0;
  // Source3D :525-548 (zeros)
  template <int DIM>
  __device__ __forceinline__ static void source(const double*, long long, long long, long long, long long,
                                                const QoldView& qo, const double*, const ProbParams& pp, double* s) {
    const double o0 = qo.p[0];
    s[0] = DIM == 2 ? (1.0 + pp.dt) * o0 : 0.0;
    s[1] = 0.0;
  }
  // SourceUpdate2D/3D is zero (BioGrowth/problem.f90:382-405, :551-574)
  template <int DIM>
  __device__ __forceinline__ static void source_update(const double*, long long, long long, long long, long long,
                                                       const QoldView&, const double*, const ProbParams&,
                                                       double* su) {
    su[0] = 0.0;
    su[1] = 0.0;
  }

  static MxParams mx_params(const ProbParams&) { return MxParams{{0.f, 0.f, 0.f, 0.f}}; }
};

BSAMG_PLUGIN(BioGrowth)

}  // namespace bsamg
